// GridLut.cpp / cuGridLut.cpp / ConvKernel.cpp -- gridding classes of the C++
// drop-in API.  Interface: ReconData/GridLut.h:9-42, cuGridLut.h:31-57,
// ConvKernel.h:7-22.  All gridding runs through the C ABI (fr_plan_*, fr_grid).
#include <algorithm>
#include <cstdlib>
#include <iostream>
#include <vector>

#include "fastrecon/ConvKernel.h"
#include "fastrecon/cuGridLut.h"
#include "fastrecon_gb300.h"

namespace {
void fr_ok(int st, const char *what)
{
    if (st != FR_OK)
        throw std::runtime_error(std::string(what) + ": " + fr_status_string(st) + ": " + fr_last_error());
}
}  // namespace

// ConvKernel.cpp:7-30 (fr_kb_lut computes the same float/double sequence).
ConvKernel::ConvKernel(float kWidth, float overGridFactor, int length)
    : m_kWidth(kWidth), m_ogFactor(overGridFactor), m_length(length)
{
    auto data = std::make_shared<std::vector<float>>(length > 0 ? length : 0);
    if (length >= 2) fr_ok(fr_kb_lut(kWidth, overGridFactor, length, data->data()), "fr_kb_lut");
    m_kernelData = data;
}

ConvKernel::~ConvKernel() {}

const std::vector<float> *ConvKernel::getKernelData() const { return m_kernelData.get(); }

float ConvKernel::getKernelWidth() const { return m_kWidth; }

template <typename T>
GridLut<T>::GridLut(ReconData<T> &reconData) : m_associatedData(reconData)
{
}

template <typename T>
GridLut<T>::~GridLut()
{
    delete m_kernel;
}

template <typename T>
std::shared_ptr<GridLut<T>> GridLut<T>::Create(ReconData<T> &reconData)
{
    auto cu = dynamic_cast<cuReconData<T> *>(&reconData);
    if (cu == nullptr) {
        std::cerr << "Error: GridLut needs the ReconData returned by ReconData::Create." << std::endl;
        exit(1);
    }
    return std::shared_ptr<GridLut<T>>(new cuGridLut<T>(*cu));
}

// GridLut.cpp:41-51
template <typename T>
void GridLut<T>::plan(unsigned reconSize, float overGridFactor, float kWidth, unsigned klength)
{
    m_dim = m_associatedData.rcDim();
    m_gridSize = unsigned(reconSize * overGridFactor);
    delete m_kernel;
    m_kernel = new ConvKernel(kWidth, overGridFactor, klength);
    m_associatedData.normalizeTraj(m_gridSize);
}

template class GridLut<float>;

// ---------------------------------------------------------------------------
// cuGridLut
// ---------------------------------------------------------------------------

template <typename T>
cuGridLut<T>::cuGridLut(cuReconData<T> &reconData) : GridLut<T>(reconData), m_cuData(reconData)
{
}

template <typename T>
cuGridLut<T>::~cuGridLut()
{
    if (m_plan) fr_plan_destroy(m_plan);
}

template <typename T>
void cuGridLut<T>::setTiling(int tx, int ty, int tz, int coilGroup)
{
    m_tile[0] = tx;
    m_tile[1] = ty;
    m_tile[2] = tz;
    m_coil_group = coilGroup;
}

template <typename T>
void cuGridLut<T>::plan(unsigned reconSize, float overGridFactor, float kWidth, unsigned klength)
{
    GridLut<T>::plan(reconSize, overGridFactor, kWidth, klength);  // normalises the trajectory in place
    if (m_plan) {
        fr_plan_destroy(m_plan);
        m_plan = nullptr;
    }
    const std::vector<float> *lut = this->m_kernel->getKernelData();
    fr_plan_desc d = {};
    d.dim = (int)this->m_dim;
    d.grid_size = this->m_gridSize;
    d.kernel_width = kWidth;
    d.lut_length = (int)lut->size();
    d.lut = lut->data();
    for (int i = 0; i < 3; ++i) d.tile[i] = m_tile[i];
    int cg = m_coil_group;
    if (cg <= 0) {
        cg = 4;
        while (cg < m_cuData.channels() && cg < 16) cg <<= 1;
    }
    d.coil_group = cg;
    d.flags = FR_PLAN_PRENORMALIZED;
    fr_ok(fr_plan_create(&d, &m_plan), "fr_plan_create");
    m_grid_cache.reset();
    m_kwidth = kWidth;
    m_partitioned = false;
    const auto &traj = m_cuData.cuGetTraj();
    const int st = fr_plan_set_trajectory(m_plan, reinterpret_cast<const float *>(traj.data()), traj.size(), nullptr);
    if (st == FR_ERR_OUT_OF_MEMORY) {
        // cuGridLut.cu:182-220 partitions its pair map instead; the plan's
        // partial buffers are released for the partitions' plans
        fr_plan_destroy(m_plan);
        m_plan = nullptr;
        m_partitioned = true;
    } else {
        fr_ok(st, "fr_plan_set_trajectory");
    }
}

// All channels of the device k-space into d_grid: one plan, or sample
// partitions when the single plan did not fit.
template <typename T>
void cuGridLut<T>::gridAll(float *d_grid)
{
    const float *kd = reinterpret_cast<const float *>(m_cuData.cuGetAllChannels());
    const float *dcf = reinterpret_cast<const float *>(m_cuData.cuGetDcf().data());
    const int C = m_cuData.channels();
    m_last_partitions = 0;
    if (!m_partitioned) {
        fr_ok(fr_grid(m_plan, kd, dcf, C, d_grid, nullptr), "fr_grid");
        return;
    }
    const std::vector<float> *lut = this->m_kernel->getKernelData();
    fr_plan_desc d = {};
    d.dim = (int)this->m_dim;
    d.grid_size = this->m_gridSize;
    d.kernel_width = m_kwidth;
    d.lut_length = (int)lut->size();
    d.lut = lut->data();
    for (int i = 0; i < 3; ++i) d.tile[i] = m_tile[i];
    d.coil_group = m_coil_group;
    d.flags = FR_PLAN_PRENORMALIZED;
    const auto &traj = m_cuData.cuGetTraj();
    const std::size_t n = traj.size();
    std::size_t parts = (std::size_t)std::max(m_gpu_partitions, 2);
    for (;;) {
        const std::size_t part = (n + parts - 1) / parts;
        const int st = fr_grid_partitioned(&d, reinterpret_cast<const float *>(traj.data()), n, kd, dcf, C, d_grid,
                                           part, nullptr);
        if (st == FR_ERR_OUT_OF_MEMORY && part > 1) {
            parts *= 2;
            continue;
        }
        fr_ok(st, "fr_grid_partitioned");
        m_last_partitions = (int)((n + part - 1) / std::max<std::size_t>(part, 1));
        return;
    }
}

template <typename T>
void cuGridLut<T>::executeInto(cuImageData<T> &img)
{
    gridAll(reinterpret_cast<float *>(img.cuData()));
    img.cuMarkModified();
}

// cuGridLut.cu:28-48: all channels in one launch instead of one per channel.
//
// Streaming acquisitions (cuReconData.cu:52-62 patches the device k-space
// and the next execute regrids everything): once the data has seen
// single-acquisition updates, the grid of each execute() is kept, and the
// next one grids only dcf * (new - old) of the updated readouts into it
// (fr_grid_update, which also brings the device k-space up to date), then
// returns a copy.  Any change of trajectory, DCF, channels or plan makes it
// a full regrid again.
template <typename T>
std::shared_ptr<ImageData<T>> cuGridLut<T>::execute()
{
    if (m_plan == nullptr && !m_partitioned) {
        std::cerr << "Error: run cuGridLut<T> first.";
        exit(1);
    }
    const unsigned G = this->m_gridSize;
    ImageSize size = {G, G, this->m_dim == 3 ? G : 1u};
    auto img = std::make_shared<cuImageData<T>>((int)this->m_dim, size);
    const int C = m_cuData.channels();
    const std::size_t cells = img->dataSize();
    cuComplexVector<T> buf(cells * (std::size_t)C);
    img->cuReset((int)this->m_dim, size, C, std::move(buf));
    m_last_incremental = false;
    if (!m_grid_cache && !m_cuData.cuHasPending()) {
        executeInto(*img);
        return img;
    }
    // fr_grid_update needs the single plan: partitioned grids regrid in full
    const bool valid = m_grid_cache && !m_partitioned && m_cache_generation == m_cuData.cuGeneration() &&
                       m_cache_channels == C && m_cuData.cuDeviceChannelsRaw() != nullptr;
    if (valid) {
        // group the pending readouts by acquisition: one fr_grid_update per
        // updated acquisition, with every channel's row (unchanged rows give
        // a zero change)
        auto pending = m_cuData.cuTakePending();
        std::vector<int> acqs;
        for (const auto &pc : pending) acqs.push_back(pc.first);
        std::sort(acqs.begin(), acqs.end());
        acqs.erase(std::unique(acqs.begin(), acqs.end()), acqs.end());
        const std::size_t ns = (std::size_t)m_cuData.samplesPerAcquisition();
        cuComplex *kd = m_cuData.cuDeviceChannelsRaw();
        cuComplexVector<T> fresh(ns * (std::size_t)C);
        for (int a : acqs) {
            for (int c = 0; c < C; ++c) {
                const ComplexVector<T> *host = m_cuData.getChannelData(c);
                fastrecon::cuda_check(cudaMemcpy(fresh.data() + ns * c, host->data() + ns * a, ns * sizeof(cuComplex),
                                                 cudaMemcpyHostToDevice),
                                      "updated acquisition upload");
            }
            fr_ok(fr_grid_update(m_plan, reinterpret_cast<float *>(kd), reinterpret_cast<const float *>(fresh.data()),
                                 ns * (std::size_t)a, ns, reinterpret_cast<const float *>(m_cuData.cuGetDcf().data()),
                                 C, reinterpret_cast<float *>(m_grid_cache->data()), nullptr),
                  "fr_grid_update");
        }
        m_last_incremental = true;
    } else {
        m_grid_cache.reset(new cuComplexVector<T>(cells * (std::size_t)C));
        gridAll(reinterpret_cast<float *>(m_grid_cache->data()));
        m_cache_generation = m_cuData.cuGeneration();
        m_cache_channels = C;
    }
    fastrecon::cuda_check(cudaMemcpy(img->cuData(), m_grid_cache->data(), cells * (std::size_t)C * sizeof(cuComplex),
                                     cudaMemcpyDeviceToDevice),
                          "grid copy");
    img->cuMarkModified();
    return img;
}

template class cuGridLut<float>;
