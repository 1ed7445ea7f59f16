// cuReconData.h -- device caches of ReconData (ReconData/cuReconData.h:7-47).
//
// The trajectory, DCF and k-space are uploaded lazily on first device access.
// Unlike the reference, which keeps one channel on the device
// (cuReconData.cu:12-31), all channels are kept in one contiguous buffer
// (channels x samples complex), the layout the multi-coil scatter reads.
#ifndef FASTRECON_CURECONDATA_H
#define FASTRECON_CURECONDATA_H

#include "ReconData.h"

template <typename T>
class cuReconData : public ReconData<T> {
public:
    typedef cuVector<Point<T>> cuTrajVector;

    cuReconData(int samples, int acquisitions);
    virtual ~cuReconData() {}

    const cuComplexVector<T> *cuGetChannelData(int channel) const;
    const cuTrajVector &cuGetTraj() const;
    const cuVector<T> &cuGetDcf() const;
    // All channels, contiguous on the device.
    const cuComplex *cuGetAllChannels() const;

    // cuReconData.cu:52-62.  With a device copy of the k-space, the readout is
    // recorded as pending instead of copied at once: a cuGridLut holding the
    // previous grid then regrids only the change (fr_grid_update), and every
    // other device access applies the pending readouts first.
    virtual void updateSingleAcquisition(const std::complex<T> *data, int acquisition, int channel = 0) override;
    virtual void clear() override;

    // For incremental regridding (cuGridLut): a counter that changes whenever
    // the trajectory, DCF or channel set changes (not on single-acquisition
    // updates); the pending (acquisition, channel) readouts, handed over once
    // (the caller must then bring the device copy up to date, e.g. through
    // fr_grid_update); the device k-space without applying them.
    unsigned long long cuGeneration() const { return m_generation; }
    bool cuHasPending() const { return !m_pending.empty(); }
    std::vector<std::pair<int, int>> cuTakePending();
    cuComplex *cuDeviceChannelsRaw() const;
    int samplesPerAcquisition() const { return this->m_samples; }

protected:
    void hostChanged() override;

private:
    cuTrajVector &getTrajDevice() const;
    virtual void transformLocalTraj(T translation, T scale) override;

    mutable std::unique_ptr<cuTrajVector> m_cu_traj;
    mutable std::unique_ptr<cuComplexVector<T>> m_cu_kData;  // all channels
    mutable int m_cu_channels = 0;
    mutable std::unique_ptr<cuVector<T>> m_cu_dcf;
    mutable std::vector<std::unique_ptr<cuComplexVector<T>>> m_views;
    unsigned long long m_generation = 0;
    mutable std::vector<std::pair<int, int>> m_pending;  // (acquisition, channel) not yet on the device
    void applyPending() const;
};

#endif  // FASTRECON_CURECONDATA_H
