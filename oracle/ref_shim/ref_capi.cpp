// extern "C" driver over the reference's own CPU classes (ReconData,
// GridLut, ConvKernel, ImageData, ImageFilter), compiled unmodified from the
// reference sources.  Test infrastructure: it produces the golden vectors
// that pin the oracle and, where it is built, the reference CPU baseline.
#include <complex>
#include <cstring>
#include <memory>
#include <vector>
#include <QVector>

#include "ConvKernel.h"
#include "GridLut.h"
#include "ImageData.h"
#include "ImageFilter.h"
#include "ReconData.h"

namespace {

std::shared_ptr<ReconData<float>> load(const float *traj4, const float *dcf, const float *kdata,
                                       int samples, int acquisitions, int dim, int channels)
{
    auto rd = ReconData<float>::Create(samples, acquisitions, false);
    size_t n = (size_t)samples * (size_t)acquisitions;
    // ReconData::loadTraj takes [x, y, (z), dcf] interleaved per sample.
    QVector<float> t(n * (dim + 1));
    for (size_t s = 0; s < n; ++s) {
        for (int d = 0; d < dim; ++d)
            t[s * (dim + 1) + d] = traj4[4 * s + d];
        t[s * (dim + 1) + dim] = dcf[s];
    }
    rd->loadTraj(t, dim);
    for (int c = 0; c < channels; ++c) {
        ComplexVector<float> v(n);
        std::memcpy(v.data(), kdata + 2 * n * (size_t)c, n * sizeof(std::complex<float>));
        rd->addChannelData(std::move(v));
    }
    return rd;
}

}  // namespace

extern "C" int ref_kb_lut(float kWidth, float os, int length, float *out)
{
    ConvKernel k(kWidth, os, length);
    const std::vector<float> *d = k.getKernelData();
    std::memcpy(out, d->data(), d->size() * sizeof(float));
    return 0;
}

// GridLut<float>::plan + execute on the CPU path (Main.cpp:117-128).
extern "C" int ref_grid(const float *traj4, const float *dcf, const float *kdata, int samples,
                        int acquisitions, int dim, int channels, unsigned reconSize, float os,
                        float kWidth, unsigned klength, int threads, float *out_grid,
                        float *out_traj_norm)
{
    auto rd = load(traj4, dcf, kdata, samples, acquisitions, dim, channels);
    auto grid = GridLut<float>::Create(*rd);
    grid->setNumOfThreads(threads);
    grid->plan(reconSize, os, kWidth, klength);
    auto img = grid->execute();
    size_t cells = img->dataSize();
    for (int c = 0; c < img->channels(); ++c)
        std::memcpy(out_grid + 2 * cells * (size_t)c, img->getChannelImage(c)->data(),
                    cells * sizeof(std::complex<float>));
    if (out_traj_norm) {
        const auto &tr = rd->getTraj();
        for (size_t s = 0; s < tr.size(); ++s)
            for (int d = 0; d < 4; ++d)
                out_traj_norm[4 * s + d] = d < dim ? tr[s].x[d] : 0.0f;
    }
    return 0;
}

// ImageFilter<float>::fftShift + SOS(reconSize) on channel images
// (Main.cpp:143,168).  out is the recon-size complex image.
extern "C" int ref_shift_sos(const float *imgs, int channels, int dim, unsigned G,
                             const unsigned *recon, float *out)
{
    ImageSize sz = {G, G, G};
    ImageData<float> img(dim, sz);
    size_t cells = img.dataSize();
    for (int c = 0; c < channels; ++c) {
        ComplexVector<float> v(cells);
        std::memcpy(v.data(), imgs + 2 * cells * (size_t)c, cells * sizeof(std::complex<float>));
        img.addChannelImage(std::move(v));
    }
    auto filter = ImageFilter<float>::Create(img);
    filter->fftShift();
    filter->SOS({recon[0], recon[1], recon[2]});
    size_t nout = (size_t)recon[0] * recon[1] * recon[2];
    std::memcpy(out, img.getChannelImage(0)->data(), nout * sizeof(std::complex<float>));
    return 0;
}

// ImageFilter::lowFilter / normalize / SOS(map) on channel images.
// op: 0 = lowFilter(res), 1 = normalize, 2 = SOS(map, recon) (out = complex recon image)
extern "C" int ref_pils_op(int op, float *imgs, const float *maps, int channels, int dim, unsigned G, int res,
                           const unsigned *recon, float *out)
{
    ImageSize sz = {G, G, G};
    ImageData<float> img(dim, sz), map(dim, sz);
    size_t cells = img.dataSize();
    for (int c = 0; c < channels; ++c) {
        ComplexVector<float> v(cells);
        std::memcpy(v.data(), imgs + 2 * cells * (size_t)c, cells * sizeof(std::complex<float>));
        img.addChannelImage(std::move(v));
        if (maps) {
            ComplexVector<float> m(cells);
            std::memcpy(m.data(), maps + 2 * cells * (size_t)c, cells * sizeof(std::complex<float>));
            map.addChannelImage(std::move(m));
        }
    }
    auto filter = ImageFilter<float>::Create(img);
    if (op == 0 || op == 1) {
        if (op == 0)
            filter->lowFilter(res);
        else
            filter->normalize();
        for (int c = 0; c < channels; ++c)
            std::memcpy(imgs + 2 * cells * (size_t)c, img.getChannelImage(c)->data(),
                        cells * sizeof(std::complex<float>));
        return 0;
    }
    filter->SOS(map, {recon[0], recon[1], recon[2]});
    size_t nout = (size_t)recon[0] * recon[1] * recon[2];
    std::memcpy(out, img.getChannelImage(0)->data(), nout * sizeof(std::complex<float>));
    return 0;
}

// The PILS branch of Main.cpp:131-164 without I/O: |SOS(map)| float image.
extern "C" int ref_recon_pils(const float *traj4, const float *dcf, const float *kdata, int samples,
                              int acquisitions, int dim, int channels, unsigned reconSize, float os, float kWidth,
                              unsigned klength, int threads, const unsigned *recon, float *out_mag)
{
    auto rd = load(traj4, dcf, kdata, samples, acquisitions, dim, channels);
    auto grid = GridLut<float>::Create(*rd);
    grid->setNumOfThreads(threads);
    grid->plan(reconSize, os, kWidth, klength);
    auto imgData = grid->execute();
    ImageData<float> imgMap;
    imgMap = *imgData;
    auto filter = ImageFilter<float>::Create(*imgData);
    filter->setNumOfThreads(threads);
    filter->fftPlan();
    filter->fftExecute();
    filter->fftShift();
    auto filterMap = ImageFilter<float>::Create(imgMap);
    filterMap->lowFilter(22);
    filterMap->fftExecute();
    filterMap->fftShift();
    filterMap->normalize();
    filter->SOS(imgMap, {recon[0], recon[1], recon[2]});
    size_t nout = (size_t)recon[0] * recon[1] * recon[2];
    const auto *d = imgData->getChannelImage(0);
    for (size_t i = 0; i < nout; ++i) out_mag[i] = std::abs((*d)[i]);
    return 0;
}

// The whole CPU pipeline of Main.cpp:101-181 without I/O: |SOS| float image.
extern "C" int ref_recon(const float *traj4, const float *dcf, const float *kdata, int samples,
                         int acquisitions, int dim, int channels, unsigned reconSize, float os,
                         float kWidth, unsigned klength, int threads, const unsigned *recon,
                         float *out_mag)
{
    auto rd = load(traj4, dcf, kdata, samples, acquisitions, dim, channels);
    auto grid = GridLut<float>::Create(*rd);
    grid->setNumOfThreads(threads);
    grid->plan(reconSize, os, kWidth, klength);
    auto imgData = grid->execute();
    auto filter = ImageFilter<float>::Create(*imgData);
    filter->setNumOfThreads(threads);
    filter->fftPlan();
    filter->fftExecute();
    filter->fftShift();
    filter->SOS({recon[0], recon[1], recon[2]});
    size_t nout = (size_t)recon[0] * recon[1] * recon[2];
    const auto *d = imgData->getChannelImage(0);
    for (size_t i = 0; i < nout; ++i)
        out_mag[i] = std::abs((*d)[i]);
    return 0;
}
