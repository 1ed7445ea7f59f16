// ImageFilter.h -- image-domain operations (ImageFilter/ImageFilter.h:13-38).
//
// Same interface as the reference.  Every operation runs on the GPU through
// the C ABI of libfastrecon_gb300.so: on a cuImageData in place on its device
// buffer, on a host ImageData through a device copy.  fftPlan's sign takes the
// FFTW convention (FFTW_BACKWARD = +1 is the reference default).
#ifndef FASTRECON_IMAGEFILTER_H
#define FASTRECON_IMAGEFILTER_H

#include "ImageData.h"

#ifndef FFTW_FORWARD
#define FFTW_FORWARD (-1)
#endif
#ifndef FFTW_BACKWARD
#define FFTW_BACKWARD (+1)
#endif

struct fr_fft_s;

template <typename T>
class ImageFilter {
public:
    static std::shared_ptr<ImageFilter<T>> Create(ImageData<T> &imageData);
    virtual ~ImageFilter();

    void setNumOfThreads(unsigned threads) { m_num_threads = threads; }
    void fftShift();
    virtual void lowFilter(int res);
    virtual void normalize();
    virtual void crop(const ImageSize &imageSize);
    virtual void SOS(ImageSize reconSize);
    virtual void SOS(const ImageData<T> &map, ImageSize reconSize);
    virtual void fftPlan(int sign = FFTW_BACKWARD);
    void fftExecute();

protected:
    ImageFilter(ImageData<T> &imageData);

    fr_fft_s *m_fft = nullptr;
    int m_fft_sign = FFTW_BACKWARD;
    int m_fft_batch = 0;

private:
    ImageData<T> &m_associatedData;
    unsigned m_num_threads = 1;  // accepted for compatibility; the GPU path ignores it
};

#endif  // FASTRECON_IMAGEFILTER_H
