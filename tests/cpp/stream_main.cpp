// Streaming acquisitions through the C++ drop-in API, for the tests:
// ReconData::loadTraj (interleaved [x, y, (z), dcf] per sample,
// ReconData.cpp:146-177) + addChannelData, GridLut::plan / execute, then
// ReconData::updateSingleAcquisition of some readouts (ReconData.cpp:179-189,
// cuReconData.cu:52-62) and execute again.
//
//   stream_main DIR SAMPLES ACQ CHANNELS DIM RECON OS WIDTH KLENGTH NUPD
//
// DIR holds traj_il.f32 (samples * acq * (DIM + 1) floats), data_c.c64 per
// channel, upd_acq.i32 (NUPD acquisition indices) and upd_k_c.c64 (the new
// readout k of channel c).  Writes grid0.c64, grid1.c64, grid2.c64 (all
// channels: before the updates, after the first half, after the rest),
// traj_norm.f32 and dcf.f32 (after plan), and prints partitions=P (sample
// partitions of the first execute, 0: one plan), incremental1=0|1 and
// incremental2=0|1 for the two executes after updates.
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <string>
#include <vector>

#include "fastrecon/GridLut.h"
#include "fastrecon/ReconData.h"
#include "fastrecon/cuGridLut.h"

template <typename V>
static V read_file(const std::string &name, std::size_t count)
{
    V v(count);
    FILE *f = std::fopen(name.c_str(), "rb");
    if (!f || std::fread(v.data(), sizeof(v[0]), count, f) != count) {
        std::cerr << "cannot read " << name << std::endl;
        std::exit(2);
    }
    std::fclose(f);
    return v;
}

static void write_file(const std::string &name, const void *p, size_t bytes)
{
    FILE *f = std::fopen(name.c_str(), "wb");
    if (!f || std::fwrite(p, 1, bytes, f) != bytes) {
        std::cerr << "cannot write " << name << std::endl;
        std::exit(2);
    }
    std::fclose(f);
}

static void write_grid(const std::string &name, ImageData<float> &img)
{
    std::vector<std::complex<float>> all;
    for (int c = 0; c < img.channels(); ++c) {
        const auto *ch = img.getChannelImage(c);
        all.insert(all.end(), ch->begin(), ch->end());
    }
    write_file(name, all.data(), all.size() * sizeof(all[0]));
}

int main(int argc, char **argv)
{
    if (argc < 11) {
        std::cerr << "usage: stream_main DIR SAMPLES ACQ CHANNELS DIM RECON OS WIDTH KLENGTH NUPD" << std::endl;
        return 2;
    }
    std::string dir = argv[1];
    int samples = std::atoi(argv[2]), acq = std::atoi(argv[3]), channels = std::atoi(argv[4]);
    int dim = std::atoi(argv[5]);
    unsigned recon = std::atoi(argv[6]);
    float os = std::atof(argv[7]), width = std::atof(argv[8]);
    unsigned klength = std::atoi(argv[9]);
    int nupd = std::atoi(argv[10]);
    const std::size_t n = (std::size_t)samples * acq;

    auto data = ReconData<float>::Create(samples, acq, true);
    data->loadTraj(read_file<std::vector<float>>(dir + "/traj_il.f32", n * (dim + 1)), dim);
    for (int c = 0; c < channels; ++c)
        data->addChannelData(read_file<ComplexVector<float>>(dir + "/data_" + std::to_string(c) + ".c64", n));

    auto grid = GridLut<float>::Create(*data);
    grid->plan(recon, os, width, klength);
    auto img0 = grid->execute();
    write_grid(dir + "/grid0.c64", *img0);
    auto *cugrid = dynamic_cast<cuGridLut<float> *>(grid.get());
    std::cout << "partitions=" << cugrid->lastExecutePartitions() << std::endl;

    // two rounds of updates (the first half of the list, then the rest): the
    // first execute after updates regrids everything and keeps the grid, the
    // second regrids only the updated readouts
    auto acqs = read_file<std::vector<int>>(dir + "/upd_acq.i32", nupd);
    for (int round = 0; round < 2; ++round) {
        const int k0 = round == 0 ? 0 : nupd / 2, k1 = round == 0 ? nupd / 2 : nupd;
        for (int k = k0; k < k1; ++k)
            for (int c = 0; c < channels; ++c) {
                auto v = read_file<ComplexVector<float>>(
                    dir + "/upd_" + std::to_string(k) + "_" + std::to_string(c) + ".c64", samples);
                data->updateSingleAcquisition(v.data(), acqs[k], c);
            }
        auto img = grid->execute();
        write_grid(dir + "/grid" + std::to_string(round + 1) + ".c64", *img);
        std::cout << "incremental" << round + 1 << "=" << (cugrid->lastExecuteIncremental() ? 1 : 0) << std::endl;
    }
    const auto &tr = data->getTraj();
    write_file(dir + "/traj_norm.f32", tr.data(), tr.size() * sizeof(Point<float>));
    write_file(dir + "/dcf.f32", data->getDcf().data(), data->getDcf().size() * sizeof(float));
    return 0;
}
