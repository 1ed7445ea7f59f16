// ReconData.cpp / cuReconData.cpp -- k-space containers of the C++ drop-in API.
// Interface: ReconData/ReconData.h:18-65, ReconData/cuReconData.h:7-47.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <limits>

#include "fastrecon/cuReconData.h"
#include "fastrecon_gb300.h"

namespace {
void fr_ok(int st, const char *what)
{
    if (st != FR_OK)
        throw std::runtime_error(std::string(what) + ": " + fr_status_string(st) + ": " + fr_last_error());
}
}  // namespace

template <typename T>
ReconData<T>::ReconData(int samples, int acquisitions) : m_samples(samples), m_acquisitions(acquisitions)
{
    m_size = (std::size_t)samples * acquisitions;
}

template <typename T>
std::shared_ptr<ReconData<T>> ReconData<T>::Create(int samples, int acquisitions, bool)
{
    return std::shared_ptr<ReconData<T>>(new cuReconData<T>(samples, acquisitions));
}

template <typename T>
void ReconData<T>::addChannelData(ComplexVector<T> &&data)
{
    if (m_size != data.size()) {  // ReconData.cpp:33-43
        std::cerr << "Error: trajectory and data have different size!" << std::endl;
        exit(1);
    }
    m_kDataMultiChannel.push_back(std::move(data));
    hostChanged();
}

template <typename T>
void ReconData<T>::setDcf(std::vector<T> &dcf)
{
    if (m_size != dcf.size()) {  // ReconData.cpp:45-54
        std::cerr << "Error: data size does not match!" << std::endl;
        exit(1);
    }
    m_dcf = std::move(dcf);
    hostChanged();
}

template <typename T>
void ReconData<T>::storeTrajComponent(const std::vector<T> &traj_c)
{
    if (m_size != traj_c.size()) {  // ReconData.cpp:56-81
        std::cerr << "Error: data size does not match!" << std::endl;
        exit(1);
    }
    if (m_dim == 4) {
        std::cout << "4-D trajectories have been loaded, ignoring additional data." << std::endl;
        return;
    }
    m_traj.resize(m_size);
    auto bound = std::minmax_element(traj_c.begin(), traj_c.end());
    m_bounds.push_back(std::make_pair(*bound.first, *bound.second));
    auto in = traj_c.begin();
    for (auto &p : m_traj) p.x[m_dim] = *(in++);
    ++m_dim;
}

template <typename T>
void ReconData<T>::loadFromFiles(const std::vector<std::string> &dataFileList,
                                 const std::vector<std::string> &trajFileList, const std::string &dcfFileName)
{
    // ReconData.cpp:83-144: one raw float file per trajectory component, one
    // raw float DCF file, one raw complex64 file per channel.
    auto read_exact = [](const std::string &name, void *dst, std::size_t bytes) {
        std::FILE *f = std::fopen(name.c_str(), "rb");
        std::size_t got = f ? std::fread(dst, 1, bytes, f) : 0;
        if (f) std::fclose(f);
        if (got != bytes) {
            std::cout << "Error: wrong data size in " << name << std::endl;
            std::exit(1);
        }
    };
    m_dim = 0;
    m_bounds.clear();
    for (const auto &name : trajFileList) {
        std::vector<T> traj_c(m_size);
        read_exact(name, traj_c.data(), m_size * sizeof(T));
        storeTrajComponent(traj_c);
    }
    m_dcf.resize(m_size);
    read_exact(dcfFileName, m_dcf.data(), m_size * sizeof(T));
    for (const auto &name : dataFileList) {
        ComplexVector<T> kdata(m_size);
        read_exact(name, kdata.data(), m_size * sizeof(std::complex<T>));
        addChannelData(std::move(kdata));
    }
    hostChanged();
}

template <typename T>
void ReconData<T>::loadTraj(const std::vector<T> &traj, int dim)
{
    if (traj.size() != m_size * (dim + 1)) {  // ReconData.cpp:146-177
        std::cerr << "Error: data size does not match!" << std::endl << std::flush;
        return;
    }
    m_dim = dim;
    m_traj.resize(m_size);
    m_dcf.resize(m_size);
    m_bounds.resize(dim);
    for (auto &bound : m_bounds) {
        bound.first = std::numeric_limits<T>::max();
        bound.second = std::numeric_limits<T>::lowest();
    }
    auto in = traj.begin();
    auto it_dcf = m_dcf.begin();
    for (auto &p : m_traj) {
        for (int i = 0; i < dim; i++) {
            p.x[i] = *(in++);
            if (m_bounds[i].first > p.x[i]) m_bounds[i].first = p.x[i];
            if (m_bounds[i].second < p.x[i]) m_bounds[i].second = p.x[i];
        }
        *(it_dcf++) = *(in++);
    }
    hostChanged();
}

template <typename T>
void ReconData<T>::updateSingleAcquisition(const std::complex<T> *data, int acquisition, int channel)
{
    if (channel > (int)m_kDataMultiChannel.size() - 1) {  // ReconData.cpp:179-189
        std::cerr << "Error: channel " << channel << " is empty!" << std::endl << std::flush;
        return;
    }
    auto &channel_data = m_kDataMultiChannel[channel];
    std::copy_n(data, m_samples, channel_data.begin() + (std::size_t)m_samples * acquisition);
}

template <typename T>
const ComplexVector<T> *ReconData<T>::getChannelData(int channel) const
{
    if (channel < 0 || channel > (int)m_kDataMultiChannel.size() - 1) return nullptr;
    return &m_kDataMultiChannel[channel];
}

// ReconData.cpp:211-225: translation and scale from component 0's bounds,
// applied to every component (on the device, transformLocalTraj).
template <typename T>
void ReconData<T>::normalizeTraj(unsigned size)
{
    auto bounds = getCompBounds(0);
    auto tr = -bounds.first;
    auto scale = (size - 1) / (bounds.second - bounds.first);
    for (int comp = 0; comp < m_dim; ++comp) {
        m_bounds[comp].first = (m_bounds[comp].first + tr) * scale;
        m_bounds[comp].second = (m_bounds[comp].second + tr) * scale;
    }
    transformLocalTraj(tr, scale);
}

template <typename T>
void ReconData<T>::clear()
{
    m_size = 0;
    m_traj.clear();
    m_dcf.clear();
    m_kDataMultiChannel.clear();
    m_bounds.clear();
    hostChanged();
}

template class ReconData<float>;

// ---------------------------------------------------------------------------
// cuReconData
// ---------------------------------------------------------------------------

template <typename T>
cuReconData<T>::cuReconData(int samples, int acquisitions) : ReconData<T>(samples, acquisitions)
{
}

template <typename T>
void cuReconData<T>::hostChanged()
{
    ++m_generation;
    m_pending.clear();
    m_cu_traj.reset();
    m_cu_kData.reset();
    m_cu_channels = 0;
    m_cu_dcf.reset();
    m_views.clear();
}

template <typename T>
typename cuReconData<T>::cuTrajVector &cuReconData<T>::getTrajDevice() const
{
    if (!m_cu_traj) m_cu_traj.reset(new cuTrajVector(this->m_traj));
    return *m_cu_traj;
}

template <typename T>
const typename cuReconData<T>::cuTrajVector &cuReconData<T>::cuGetTraj() const
{
    return getTrajDevice();
}

template <typename T>
const cuVector<T> &cuReconData<T>::cuGetDcf() const
{
    if (!m_cu_dcf) m_cu_dcf.reset(new cuVector<T>(this->m_dcf));
    return *m_cu_dcf;
}

template <typename T>
void cuReconData<T>::applyPending() const
{
    for (const auto &pc : m_pending) {
        const std::size_t off = (std::size_t)this->m_samples * pc.first;
        fastrecon::cuda_check(cudaMemcpy(m_cu_kData->data() + this->m_size * pc.second + off,
                                         this->m_kDataMultiChannel[pc.second].data() + off,
                                         (std::size_t)this->m_samples * sizeof(cuComplex), cudaMemcpyHostToDevice),
                              "acquisition update");
    }
    m_pending.clear();
}

template <typename T>
std::vector<std::pair<int, int>> cuReconData<T>::cuTakePending()
{
    std::vector<std::pair<int, int>> p;
    p.swap(m_pending);
    return p;
}

template <typename T>
cuComplex *cuReconData<T>::cuDeviceChannelsRaw() const
{
    return m_cu_kData && m_cu_channels == this->channels() ? m_cu_kData->data() : nullptr;
}

template <typename T>
const cuComplex *cuReconData<T>::cuGetAllChannels() const
{
    const int C = this->channels();
    if (m_cu_kData && m_cu_channels == C && !m_pending.empty()) applyPending();
    if (!m_cu_kData || m_cu_channels != C) {
        m_pending.clear();
        m_views.clear();
        m_cu_kData.reset(new cuComplexVector<T>(this->m_size * (std::size_t)C));
        for (int c = 0; c < C; ++c)
            fastrecon::cuda_check(cudaMemcpy(m_cu_kData->data() + this->m_size * c, this->m_kDataMultiChannel[c].data(),
                                             this->m_size * sizeof(cuComplex), cudaMemcpyHostToDevice),
                                  "k-space upload");
        m_cu_channels = C;
    }
    return m_cu_kData->data();
}

template <typename T>
const cuComplexVector<T> *cuReconData<T>::cuGetChannelData(int channel) const
{
    if (channel < 0 || channel >= this->channels()) return nullptr;
    const cuComplex *base = cuGetAllChannels();
    m_views.emplace_back(new cuComplexVector<T>(
        cuComplexVector<T>::view(const_cast<cuComplex *>(base) + this->m_size * channel, this->m_size)));
    return m_views.back().get();
}

template <typename T>
void cuReconData<T>::updateSingleAcquisition(const std::complex<T> *data, int acquisition, int channel)
{
    ReconData<T>::updateSingleAcquisition(data, acquisition, channel);
    // cuReconData.cu:52-62 patches the cached device copy at once; here the
    // readout is recorded and reaches the device copy on the next device
    // access (cuGetAllChannels) or through an incremental regrid (cuGridLut)
    if (m_cu_kData && channel >= 0 && channel < m_cu_channels && acquisition >= 0 &&
        acquisition < this->m_acquisitions)
        m_pending.emplace_back(acquisition, channel);
}

template <typename T>
void cuReconData<T>::clear()
{
    ReconData<T>::clear();
}

// cuReconData.cu:88-99: transform on the device, then copy back to the host.
template <typename T>
void cuReconData<T>::transformLocalTraj(T translation, T scale)
{
    ++m_generation;
    cuTrajVector &traj = getTrajDevice();
    fr_ok(fr_transform_trajectory(reinterpret_cast<float *>(traj.data()), traj.size(), this->rcDim(), translation,
                                  scale, nullptr),
          "fr_transform_trajectory");
    traj.copy_to_host(this->m_traj.data());
}

template class cuReconData<float>;
