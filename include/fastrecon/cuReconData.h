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

    virtual void updateSingleAcquisition(const std::complex<T> *data, int acquisition, int channel = 0) override;
    virtual void clear() override;

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
};

#endif  // FASTRECON_CURECONDATA_H
