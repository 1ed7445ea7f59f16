// ImageFilter.cpp -- image-domain operations of the C++ drop-in API
// (ImageFilter/ImageFilter.h:13-38, cuImageFilter.h, FFT.h, cuFFT.h).
// Every operation runs on the GPU through the C ABI; a host ImageData is
// staged through a device copy.
#include <iostream>

#include "fastrecon/ImageFilter.h"
#include "fastrecon/cuImageData.h"
#include "fastrecon_gb300.h"

namespace {

void fr_ok(int st, const char *what)
{
    if (st != FR_OK)
        throw std::runtime_error(std::string(what) + ": " + fr_status_string(st) + ": " + fr_last_error());
}

// Device view of an image's channels (channel-major, contiguous).
template <typename T>
struct DeviceImage {
    ImageData<T> &img;
    cuImageData<T> *cu;
    cuComplexVector<T> staged;
    cuComplex *ptr = nullptr;

    explicit DeviceImage(ImageData<T> &im) : img(im), cu(dynamic_cast<cuImageData<T> *>(&im))
    {
        if (cu) {
            ptr = cu->cuData();
            return;
        }
        const std::size_t cells = img.dataSize();
        staged.resize(cells * img.channels());
        for (int c = 0; c < img.channels(); ++c)
            fastrecon::cuda_check(cudaMemcpy(staged.data() + cells * c, img.getChannelImage(c)->data(),
                                             cells * sizeof(cuComplex), cudaMemcpyHostToDevice),
                                  "image upload");
        ptr = staged.data();
    }
    // the device buffer was modified in place
    void commit()
    {
        if (cu) {
            cu->cuMarkModified();
            return;
        }
        const std::size_t cells = img.dataSize();
        for (int c = 0; c < img.channels(); ++c)
            fastrecon::cuda_check(cudaMemcpy(img.getChannelImage(c)->data(), staged.data() + cells * c,
                                             cells * sizeof(cuComplex), cudaMemcpyDeviceToHost),
                                  "image download");
    }
    // replace the image by `channels` images of `size` held in `data`
    void replace(int dim, const ImageSize &size, int channels, cuComplexVector<T> &&data)
    {
        if (cu) {
            cu->cuReset(dim, size, channels, std::move(data));
            return;
        }
        ImageData<T> out(dim, size);
        const std::size_t cells = out.dataSize();
        for (int c = 0; c < channels; ++c) {
            ComplexVector<T> h(cells);
            fastrecon::cuda_check(cudaMemcpy(h.data(), data.data() + cells * c, cells * sizeof(cuComplex),
                                             cudaMemcpyDeviceToHost),
                                  "image download");
            out.addChannelImage(std::move(h));
        }
        img = std::move(out);
    }
};

void size3(const ImageSize &s, unsigned *out)
{
    out[0] = s.x;
    out[1] = s.y;
    out[2] = s.z;
}

}  // namespace

template <typename T>
std::shared_ptr<ImageFilter<T>> ImageFilter<T>::Create(ImageData<T> &imageData)
{
    return std::shared_ptr<ImageFilter<T>>(new ImageFilter<T>(imageData));
}

template <typename T>
ImageFilter<T>::ImageFilter(ImageData<T> &imageData) : m_associatedData(imageData)
{
}

template <typename T>
ImageFilter<T>::~ImageFilter()
{
    if (m_fft) fr_fft_destroy(m_fft);
}

// ImageFilter.cpp:40-53 (swap semantics, also odd sizes)
template <typename T>
void ImageFilter<T>::fftShift()
{
    if (m_associatedData.channels() == 0) return;
    DeviceImage<T> d(m_associatedData);
    unsigned sz[3];
    size3(m_associatedData.imageSize(), sz);
    fr_ok(fr_fft_shift(reinterpret_cast<float *>(d.ptr), m_associatedData.channels(), m_associatedData.dim(), sz,
                       nullptr),
          "fr_fft_shift");
    d.commit();
}

// ImageFilter.cpp:55-93
template <typename T>
void ImageFilter<T>::lowFilter(int res)
{
    if (m_associatedData.channels() == 0) return;
    DeviceImage<T> d(m_associatedData);
    unsigned sz[3];
    size3(m_associatedData.imageSize(), sz);
    fr_ok(fr_low_filter(reinterpret_cast<float *>(d.ptr), m_associatedData.channels(), m_associatedData.dim(), sz,
                        res, nullptr),
          "fr_low_filter");
    d.commit();
}

// ImageFilter.cpp:95-118
template <typename T>
void ImageFilter<T>::normalize()
{
    if (m_associatedData.channels() == 0) return;
    DeviceImage<T> d(m_associatedData);
    unsigned sz[3];
    size3(m_associatedData.imageSize(), sz);
    fr_ok(fr_normalize_channels(reinterpret_cast<float *>(d.ptr), m_associatedData.channels(),
                                m_associatedData.dim(), sz, nullptr),
          "fr_normalize_channels");
    d.commit();
}

// ImageFilter.cpp:120-157
template <typename T>
void ImageFilter<T>::crop(const ImageSize &imageSize)
{
    ImageSize size = m_associatedData.imageSize();
    if (imageSize.x > size.x || imageSize.y > size.y || imageSize.z > size.z) {
        std::cerr << "Crop size larger than image" << std::endl;
        return;
    }
    const int dim = m_associatedData.dim();
    const int C = m_associatedData.channels();
    ImageSize out = imageSize;
    if (dim == 2) out.z = 1;
    cuComplexVector<T> buf((std::size_t)out.x * out.y * out.z * C);
    if (C > 0) {
        DeviceImage<T> d(m_associatedData);
        unsigned sz[3], cs[3];
        size3(size, sz);
        size3(out, cs);
        fr_ok(fr_crop(reinterpret_cast<const float *>(d.ptr), C, dim, sz, cs, reinterpret_cast<float *>(buf.data()),
                      nullptr),
              "fr_crop");
        d.replace(dim, out, C, std::move(buf));
    } else {
        DeviceImage<T>(m_associatedData).replace(dim, out, 0, std::move(buf));
    }
}

// ImageFilter.cpp:159-168: SOS with the image itself as map, then sqrt;
// channel 0 holds (sqrt(sum |x|^2), 0).
template <typename T>
void ImageFilter<T>::SOS(ImageSize reconSize)
{
    const int dim = m_associatedData.dim();
    const int C = m_associatedData.channels();
    ImageSize out = reconSize;
    if (dim == 2) out.z = 1;
    const std::size_t n = (std::size_t)out.x * out.y * out.z;
    cuVector<float> mag(n);
    cuComplexVector<T> buf(n);
    DeviceImage<T> d(m_associatedData);
    unsigned sz[3], rs[3];
    size3(m_associatedData.imageSize(), sz);
    size3(out, rs);
    if (C > 0) {
        fr_ok(fr_sos(reinterpret_cast<const float *>(d.ptr), C, dim, sz, rs, nullptr, mag.data(), nullptr), "fr_sos");
        fr_ok(fr_real_to_complex(mag.data(), n, reinterpret_cast<float *>(buf.data()), nullptr),
              "fr_real_to_complex");
    } else {
        fastrecon::cuda_check(cudaMemset(buf.data(), 0, n * sizeof(cuComplex)), "memset");
    }
    d.replace(dim, out, 1, std::move(buf));
}

// ImageFilter.cpp:170-209: sum over channels of x * conj(map), no sqrt.
template <typename T>
void ImageFilter<T>::SOS(const ImageData<T> &map, ImageSize reconSize)
{
    const int dim = m_associatedData.dim();
    const int C = m_associatedData.channels();
    ImageSize out = reconSize;
    if (dim == 2) out.z = 1;
    const std::size_t n = (std::size_t)out.x * out.y * out.z;
    cuComplexVector<T> buf(n);
    DeviceImage<T> d(m_associatedData);
    DeviceImage<T> m(const_cast<ImageData<T> &>(map));
    unsigned sz[3], rs[3];
    size3(m_associatedData.imageSize(), sz);
    size3(out, rs);
    if (C > 0)
        fr_ok(fr_sos_map(reinterpret_cast<const float *>(d.ptr), reinterpret_cast<const float *>(m.ptr), C, dim, sz,
                         rs, reinterpret_cast<float *>(buf.data()), nullptr),
              "fr_sos_map");
    else
        fastrecon::cuda_check(cudaMemset(buf.data(), 0, n * sizeof(cuComplex)), "memset");
    d.replace(dim, out, 1, std::move(buf));
}

// ImageFilter.cpp:211-221, cuImageFilter.cpp:23-38: one batched cuFFT plan
// over all channels.
template <typename T>
void ImageFilter<T>::fftPlan(int sign)
{
    if (m_fft) {
        fr_fft_destroy(m_fft);
        m_fft = nullptr;
    }
    m_fft_sign = sign;
    m_fft_batch = m_associatedData.channels();
    if (m_fft_batch < 1) return;
    unsigned sz[3];
    size3(m_associatedData.imageSize(), sz);
    fr_ok(fr_fft_create(m_associatedData.dim(), sz, m_fft_batch, sign, &m_fft), "fr_fft_create");
}

// ImageFilter.cpp:223-229
template <typename T>
void ImageFilter<T>::fftExecute()
{
    if (m_fft == nullptr || m_fft_batch != m_associatedData.channels()) fftPlan(m_fft_sign);
    if (m_fft == nullptr) return;
    DeviceImage<T> d(m_associatedData);
    fr_ok(fr_fft_execute(m_fft, reinterpret_cast<float *>(d.ptr), nullptr), "fr_fft_execute");
    d.commit();
}

template class ImageFilter<float>;
