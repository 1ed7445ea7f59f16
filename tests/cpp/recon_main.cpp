// The Program/Main.cpp pipeline (Main.cpp:101-181) written against the C++
// drop-in API, for the tests: raw files in, |image| out.
//
//   recon_main DIR SAMPLES ACQ CHANNELS DIM RCX RCY RCZ OS WIDTH KLENGTH [pils]
//
// DIR holds traj_0.f32 .. traj_{DIM-1}.f32, dcf.f32, data_0.c64 ..
// (ReconData::loadFromFiles layout).  Writes DIR/out.f32 (|SOS| image),
// DIR/traj_norm.f32 (trajectory after GridLut::plan, 4 floats per sample) and
// DIR/grid0.c64 (gridded channel 0).
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <string>
#include <vector>

#include "fastrecon/GridLut.h"
#include "fastrecon/ImageFilter.h"
#include "fastrecon/ReconData.h"
#include "fastrecon/cuGridLut.h"

static void write_file(const std::string &name, const void *p, size_t bytes)
{
    FILE *f = std::fopen(name.c_str(), "wb");
    if (!f || std::fwrite(p, 1, bytes, f) != bytes) {
        std::cerr << "cannot write " << name << std::endl;
        std::exit(2);
    }
    std::fclose(f);
}

int main(int argc, char **argv)
{
    if (argc < 12) {
        std::cerr << "usage: recon_main DIR SAMPLES ACQ CHANNELS DIM RCX RCY RCZ OS WIDTH KLENGTH [pils]" << std::endl;
        return 2;
    }
    std::string dir = argv[1];
    int samples = std::atoi(argv[2]), acq = std::atoi(argv[3]), channels = std::atoi(argv[4]);
    int dim = std::atoi(argv[5]);
    unsigned rcx = std::atoi(argv[6]), rcy = std::atoi(argv[7]), rcz = std::atoi(argv[8]);
    float os = std::atof(argv[9]), width = std::atof(argv[10]);
    unsigned klength = std::atoi(argv[11]);
    bool pils = argc > 12 && std::string(argv[12]) == "pils";

    std::vector<std::string> traj_files, data_files;
    for (int d = 0; d < dim; ++d) traj_files.push_back(dir + "/traj_" + std::to_string(d) + ".f32");
    for (int c = 0; c < channels; ++c) data_files.push_back(dir + "/data_" + std::to_string(c) + ".c64");

    auto reconData = ReconData<float>::Create(samples, acq, true);
    reconData->loadFromFiles(data_files, traj_files, dir + "/dcf.f32");

    auto grid = GridLut<float>::Create(*reconData);
    dynamic_cast<cuGridLut<float> *>(grid.get())->setNumOfPartitions(25);
    grid->setNumOfThreads(channels);
    grid->plan(rcx, os, width, klength);
    auto imgData = grid->execute();

    const auto &tr = reconData->getTraj();
    write_file(dir + "/traj_norm.f32", tr.data(), tr.size() * sizeof(Point<float>));
    write_file(dir + "/grid0.c64", imgData->getChannelImage(0)->data(), imgData->dataSize() * 8);

    ImageData<float> imgMap;
    if (pils) imgMap = *imgData;

    auto filter = ImageFilter<float>::Create(*imgData);
    filter->setNumOfThreads(channels);
    filter->fftPlan();
    filter->fftExecute();
    filter->fftShift();
    if (pils) {
        auto filterMap = ImageFilter<float>::Create(imgMap);
        filterMap->lowFilter(22);
        filterMap->fftExecute();
        filterMap->fftShift();
        filterMap->normalize();
        filter->SOS(imgMap, {rcx, rcy, rcz});
    } else {
        filter->SOS({rcx, rcy, rcz});
    }

    std::vector<float> mag;
    for (const auto &v : *imgData->getChannelImage()) mag.push_back(std::abs(v));
    write_file(dir + "/out.f32", mag.data(), mag.size() * sizeof(float));
    std::cout << "recon_main: " << imgData->imageSize().x << "x" << imgData->imageSize().y << "x"
              << imgData->imageSize().z << " image, " << imgData->channels() << " channel" << std::endl;
    return 0;
}
