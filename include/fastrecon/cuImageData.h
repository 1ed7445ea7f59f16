// cuImageData.h -- device-resident multi-channel image (ImageData/cuImageData.h:8-36).
//
// Unlike the reference, which keeps one channel on the device and copies every
// channel to the host as it is added (cuImageData.cu:44-63), all channels live
// in one contiguous device buffer (channel-major, the layout the batched FFT
// and the SoS kernel read).  The host copy is filled on first host access and
// the device copy is refreshed after host modification (invalidateDevice).
#ifndef FASTRECON_CUIMAGEDATA_H
#define FASTRECON_CUIMAGEDATA_H

#include "ImageData.h"
#include "common.h"

template <typename T>
class cuImageData : public ImageData<T> {
public:
    cuImageData();
    cuImageData(const int dim, const ImageSize &imageSize);

    cuImageData(const cuImageData<T> &imageData);
    cuImageData(cuImageData<T> &&imageData);
    virtual ~cuImageData() {}

    cuImageData<T> &operator=(const cuImageData<T> &imageData);
    cuImageData<T> &operator=(cuImageData<T> &&imageData);

    void addChannelImage(ComplexVector<T> &&image);
    void addChannelImage(std::unique_ptr<cuComplexVector<T>> image);
    // Device view of one channel (valid until channels are added or the
    // image is reshaped).  Host copy is considered stale afterwards.
    cuComplexVector<T> *cuGetChannelImage(int channel);

    void syncDeviceToHost();
    void invalidateDevice();

    const ComplexVector<T> *getChannelImage(int channel = 0) const override;
    ComplexVector<T> *getChannelImage(int channel = 0) override;

    // --- device-side interface used by GridLut / ImageFilter ---
    // All channels, contiguous (channels x dataSize complex), uploaded from
    // the host copy if that is newer.
    cuComplex *cuData();
    // Replace the contents by `channels` device images of `size` (the
    // buffer is adopted); the host copy becomes stale.
    void cuReset(int dim, const ImageSize &size, int channels, cuComplexVector<T> &&data);
    // Mark the device copy as modified (host copy stale).
    void cuMarkModified();

private:
    using ImageData<T>::m_size;

    void copy(const ImageData<T> &imageData) override;
    void move(ImageData<T> &imageData) override;
    void fillHost() const;

    cuComplexVector<T> m_dev;
    mutable bool m_host_valid = true;
    bool m_dev_valid = true;
    std::vector<std::unique_ptr<cuComplexVector<T>>> m_views;
};

#endif  // FASTRECON_CUIMAGEDATA_H
