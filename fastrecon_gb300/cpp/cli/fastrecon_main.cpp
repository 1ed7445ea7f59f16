// fastrecon -- the reference's command-line recon program (Program/Main.cpp,
// Program/ProgramOptions.cpp) on the GB300 library, through the C++ drop-in
// classes.
//
//   fastrecon [-g FACTOR] [-w WIDTH] [--pils] [--show] [--gpu] RECON.ini
//
// Same options and the same RECON.ini keys as ProgramOptions.cpp:18-52:
// traj_file, weight_file, data_file (file-name patterns inside the ini's
// directory, matched and sorted by name like QDir(path, filter, QDir::Name)),
// out_file, xres (samples), projections, rcxres, rcyres, rczres,
// overgridding_factor (used when -g is not given).  The pipeline is
// Main.cpp:101-181: load, GridLut plan (LUT length 512) + execute, FFT,
// fftShift, SOS (or PILS), then |image| written as float32 to out_file.
// Computation always runs on the GPU (--gpu is accepted for compatibility);
// --show has no window system to draw into and only reports that.
#include <dirent.h>
#include <fnmatch.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <map>
#include <string>
#include <vector>

#include "fastrecon/GridLut.h"
#include "fastrecon/ImageFilter.h"
#include "fastrecon/ReconData.h"
#include "fastrecon/cuGridLut.h"

namespace {

struct Params {
    std::string path, traj_files, dcf_file, data_files, out_file;
    int samples = 0, projections = 0;
    float overgridding_factor = 0.f;
    float kernel_width = 4.f;
    bool pils = false, show = false, gpu = false;
    unsigned rcxres = 0, rcyres = 0, rczres = 0;
};

void usage(std::ostream &os)
{
    os << "Usage: fastrecon [OPTION...] RECON.ini\n"
          "CPU & GPU MRI recon program (GB300 build: always on the GPU).\n\n"
          " Recon parameters:\n"
          "  -g FACTOR                  Over-gridding factor\n"
          "  -w WIDTH                   Kernel full width\n\n"
          " Recon options:\n"
          "      --pils                 PILS method\n\n"
          " Miscellaneous:\n"
          "      --show                 Display result in a window\n"
          "      --gpu                  Use GPU computation if possible\n\n"
          "Command line options have precedence over RECON.ini.\n";
}

std::string trim(const std::string &s)
{
    size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
    if (a == std::string::npos) return "";
    std::string t = s.substr(a, b - a + 1);
    if (t.size() >= 2 && t.front() == '"' && t.back() == '"') t = t.substr(1, t.size() - 2);
    return t;
}

// QSettings IniFormat subset: "key=value" lines, [sections] and ;/# comments
// ignored.
std::map<std::string, std::string> read_ini(const std::string &name)
{
    std::map<std::string, std::string> kv;
    std::ifstream f(name);
    std::string line;
    while (std::getline(f, line)) {
        line = trim(line);
        if (line.empty() || line[0] == ';' || line[0] == '#' || line[0] == '[') continue;
        const size_t eq = line.find('=');
        if (eq == std::string::npos) continue;
        kv[trim(line.substr(0, eq))] = trim(line.substr(eq + 1));
    }
    return kv;
}

// Files of `dir` matching the name filter, sorted by name, prefixed by `dir`.
std::vector<std::string> list_files(const std::string &dir, const std::string &filter)
{
    std::vector<std::string> names;
    DIR *d = opendir(dir.empty() ? "." : dir.c_str());
    if (!d) return names;
    while (dirent *e = readdir(d)) {
        if (e->d_name[0] == '.' && (!e->d_name[1] || (e->d_name[1] == '.' && !e->d_name[2]))) continue;
        if (fnmatch(filter.c_str(), e->d_name, 0) == 0) names.push_back(e->d_name);
    }
    closedir(d);
    std::sort(names.begin(), names.end());
    for (auto &n : names) n = dir + n;
    return names;
}

bool parse_args(int argc, char **argv, Params &p, std::string &ini)
{
    int positional = 0;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        auto value = [&](const char *opt) -> const char * {
            if (a.size() > 2) return argv[i] + 2;  // -g1.5
            if (i + 1 >= argc) {
                std::cerr << "fastrecon: option requires an argument -- '" << opt << "'" << std::endl;
                std::exit(64);
            }
            return argv[++i];
        };
        if (a == "-h" || a == "--help" || a == "-?") {
            usage(std::cout);
            std::exit(0);
        } else if (a == "--pils") {
            p.pils = true;
        } else if (a == "--show") {
            p.show = true;
        } else if (a == "--gpu") {
            p.gpu = true;
        } else if (a.rfind("-g", 0) == 0) {
            p.overgridding_factor = (float)std::atof(value("g"));
        } else if (a.rfind("-w", 0) == 0) {
            p.kernel_width = (float)std::atof(value("w"));
        } else if (!a.empty() && a[0] == '-') {
            std::cerr << "fastrecon: unrecognized option '" << a << "'" << std::endl;
            usage(std::cerr);
            std::exit(64);
        } else {
            ++positional;
            ini = a;
        }
    }
    if (positional < 1) {
        std::cerr << "fastrecon: Missing RECON.ini arguments" << std::endl;
        return false;
    }
    if (positional > 1) {
        std::cerr << "fastrecon: too many arguments" << std::endl;
        return false;
    }
    return true;
}

}  // namespace

int main(int argc, char **argv)
{
    Params p;
    std::string ini;
    if (!parse_args(argc, argv, p, ini)) return 64;
    std::ifstream probe(ini);
    if (!probe) {
        std::cerr << "File '" << ini << "' does not exist!" << std::endl;
        return 1;
    }
    const auto kv = read_ini(ini);
    auto get = [&](const char *k) {
        auto it = kv.find(k);
        return it == kv.end() ? std::string() : it->second;
    };
    const size_t slash = ini.find_last_of('/');
    p.path = slash == std::string::npos ? "" : ini.substr(0, slash + 1);
    p.traj_files = get("traj_file");
    p.dcf_file = get("weight_file");
    p.data_files = get("data_file");
    p.out_file = get("out_file");
    p.samples = std::atoi(get("xres").c_str());
    p.projections = std::atoi(get("projections").c_str());
    p.rcxres = (unsigned)std::atoi(get("rcxres").c_str());
    p.rcyres = (unsigned)std::atoi(get("rcyres").c_str());
    p.rczres = (unsigned)std::atoi(get("rczres").c_str());
    if (p.overgridding_factor == 0.f) p.overgridding_factor = (float)std::atof(get("overgridding_factor").c_str());

    std::cout << std::left << std::setw(22) << "Samples:" << p.samples << std::endl
              << std::setw(22) << "Projections:" << p.projections << std::endl
              << std::setw(22) << "Overgridding factor:" << p.overgridding_factor << std::endl
              << std::setw(22) << "Kernel width:" << p.kernel_width << std::endl
              << std::setw(22) << "rcxres:" << p.rcxres << std::endl
              << std::setw(22) << "rcyres:" << p.rcyres << std::endl
              << std::setw(22) << "rczres:" << p.rczres << std::endl;

    using clk = std::chrono::steady_clock;
    auto ms = [](clk::time_point a, clk::time_point b) {
        return (long long)std::chrono::duration_cast<std::chrono::milliseconds>(b - a).count();
    };

    // -------------- Load multi-channel data -----------------
    auto reconData = ReconData<float>::Create(p.samples, p.projections, true);
    reconData->loadFromFiles(list_files(p.path, p.data_files), list_files(p.path, p.traj_files),
                             p.path + p.dcf_file);
    const unsigned threads = (unsigned)reconData->channels();

    const auto t0 = clk::now();
    // -------------- Gridding -------------------------------
    auto t = clk::now();
    auto grid = GridLut<float>::Create(*reconData);
    if (auto *cg = dynamic_cast<cuGridLut<float> *>(grid.get())) cg->setNumOfPartitions(25);
    grid->setNumOfThreads(threads);
    grid->plan(p.rcxres, p.overgridding_factor, p.kernel_width, 512);
    auto imgData = grid->execute();
    std::cout << "Gridding total time " << ms(t, clk::now()) << " ms" << std::endl;

    ImageData<float> imgMap;
    if (p.pils) imgMap = *imgData;

    auto filter = ImageFilter<float>::Create(*imgData);
    filter->setNumOfThreads(threads);

    // --------------- FFT ----------------------------------
    filter->fftPlan();
    t = clk::now();
    filter->fftExecute();
    filter->fftShift();
    std::cout << "FFT total time " << ms(t, clk::now()) << " ms" << std::endl;

    // -------------- Recon Methods -----------------------------------
    t = clk::now();
    if (p.pils) {
        auto filterMap = ImageFilter<float>::Create(imgMap);
        std::cout << "\nRecon PILS... " << std::endl;
        filterMap->lowFilter(22);
        filterMap->fftExecute();
        filterMap->fftShift();
        filterMap->normalize();
        std::cout << "\nSum of Square Field Map..." << std::flush;
        filter->SOS(imgMap, {p.rcxres, p.rcyres, p.rczres});
    } else {
        std::cout << "\nRecon SOS... " << std::flush;
        filter->SOS({p.rcxres, p.rcyres, p.rczres});
    }
    std::cout << " | " << ms(t, clk::now()) << " ms" << std::endl;
    std::cout << "\nProgram total time excluding I/O: " << ms(t0, clk::now()) / 1000.0 << " s" << std::endl;

    // -------------------------- Save Data ---------------------------
    FILE *f = std::fopen((p.path + p.out_file).c_str(), "wb");
    if (!f) {
        std::cerr << "cannot write " << p.path + p.out_file << std::endl;
        return 1;
    }
    for (const auto &v : *imgData->getChannelImage()) {
        const float a = std::abs(v);
        std::fwrite(&a, sizeof a, 1, f);
    }
    std::fclose(f);
    if (p.show) std::cout << "--show: no window system here; the image is in " << p.path + p.out_file << std::endl;
    return 0;
}
