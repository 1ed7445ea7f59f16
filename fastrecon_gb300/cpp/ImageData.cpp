// ImageData.cpp / cuImageData.cpp -- containers of the C++ drop-in API.
// Interface: ImageData/ImageData.h:8-50 and ImageData/cuImageData.h:8-36.
#include <cstring>
#include <iostream>

#include "fastrecon/ImageData.h"
#include "fastrecon/cuImageData.h"

template <typename T>
ImageData<T>::ImageData(const int dim, const ImageSize &size) : m_dim(dim), m_size(size)
{
    if (dim == 2) m_size.z = 1;  // ImageData.cpp:6-13
}

template <typename T>
ImageData<T>::ImageData(const ImageData<T> &imageData)
{
    copy(imageData);
}

template <typename T>
ImageData<T>::ImageData(ImageData<T> &&imageData)
{
    move(imageData);
}

template <typename T>
ImageData<T> &ImageData<T>::operator=(const ImageData<T> &imageData)
{
    copy(imageData);
    return *this;
}

template <typename T>
ImageData<T> &ImageData<T>::operator=(ImageData<T> &&imageData)
{
    move(imageData);
    return *this;
}

template <typename T>
std::size_t ImageData<T>::dataSize() const
{
    if (m_dim == 3) return (std::size_t)m_size.x * m_size.y * m_size.z;
    return (std::size_t)m_size.x * m_size.y;
}

template <typename T>
void ImageData<T>::addChannelImage(ComplexVector<T> &&image)
{
    if (image.size() != dataSize()) {  // ImageData.cpp:53-63
        std::cerr << "Error: ImageData wrong size!" << std::endl;
        exit(1);
    }
    m_data_multichannel.push_back(std::move(image));
    m_channels = m_data_multichannel.size();
}

template <typename T>
const ComplexVector<T> *ImageData<T>::getChannelImage(int channel) const
{
    if (channel >= 0 && channel < channels()) return &m_data_multichannel[channel];
    return nullptr;
}

template <typename T>
ComplexVector<T> *ImageData<T>::getChannelImage(int channel)
{
    if (channel >= 0 && channel < channels()) return &m_data_multichannel[channel];
    return nullptr;
}

template <typename T>
void ImageData<T>::copy(const ImageData<T> &imageData)
{
    m_dim = imageData.dim();
    m_size = imageData.imageSize();
    m_data_multichannel.clear();
    m_channels = 0;
    for (int c = 0; c < imageData.channels(); ++c) addChannelImage(ComplexVector<T>(*imageData.getChannelImage(c)));
}

template <typename T>
void ImageData<T>::move(ImageData<T> &imageData)
{
    // a device-resident source fills its host copy first (virtual access)
    if (imageData.m_channels > 0) imageData.getChannelImage(0);
    moveFields(imageData);
}

template <typename T>
void ImageData<T>::moveFields(ImageData<T> &imageData)
{
    m_dim = imageData.m_dim;
    m_size = imageData.m_size;
    m_channels = imageData.m_channels;
    m_data_multichannel = std::move(imageData.m_data_multichannel);
    imageData.m_data_multichannel.clear();
    imageData.m_dim = 0;
    imageData.m_size = {0, 0, 0};
    imageData.m_channels = 0;
}

template class ImageData<float>;

// ---------------------------------------------------------------------------
// cuImageData
// ---------------------------------------------------------------------------

template <typename T>
cuImageData<T>::cuImageData()
{
}

template <typename T>
cuImageData<T>::cuImageData(const int dim, const ImageSize &imageSize) : ImageData<T>(dim, imageSize)
{
}

template <typename T>
cuImageData<T>::cuImageData(const cuImageData<T> &imageData) : ImageData<T>()
{
    copy(imageData);
}

template <typename T>
cuImageData<T>::cuImageData(cuImageData<T> &&imageData) : ImageData<T>()
{
    move(imageData);
}

template <typename T>
cuImageData<T> &cuImageData<T>::operator=(const cuImageData<T> &imageData)
{
    copy(imageData);
    return *this;
}

template <typename T>
cuImageData<T> &cuImageData<T>::operator=(cuImageData<T> &&imageData)
{
    move(imageData);
    return *this;
}

template <typename T>
void cuImageData<T>::fillHost() const
{
    if (m_host_valid) return;
    auto self = const_cast<cuImageData<T> *>(this);
    const std::size_t cells = this->dataSize();
    self->m_data_multichannel.resize(this->m_channels);
    for (int c = 0; c < this->m_channels; ++c) {
        auto &h = self->m_data_multichannel[c];
        h.resize(cells);
        if (cells)
            fastrecon::cuda_check(cudaMemcpy(h.data(), m_dev.data() + (std::size_t)c * cells, cells * sizeof(cuComplex),
                                             cudaMemcpyDeviceToHost),
                                  "cuImageData download");
    }
    m_host_valid = true;
}

template <typename T>
cuComplex *cuImageData<T>::cuData()
{
    if (!m_dev_valid) {
        const std::size_t cells = this->dataSize();
        m_views.clear();
        m_dev.resize(cells * this->m_channels);
        for (int c = 0; c < this->m_channels; ++c)
            if (cells)
                fastrecon::cuda_check(cudaMemcpy(m_dev.data() + (std::size_t)c * cells,
                                                 this->m_data_multichannel[c].data(), cells * sizeof(cuComplex),
                                                 cudaMemcpyHostToDevice),
                                      "cuImageData upload");
        m_dev_valid = true;
    }
    return m_dev.data();
}

template <typename T>
void cuImageData<T>::cuMarkModified()
{
    m_host_valid = false;
    m_dev_valid = true;
}

template <typename T>
void cuImageData<T>::cuReset(int dim, const ImageSize &size, int channels, cuComplexVector<T> &&data)
{
    this->m_dim = dim;
    this->m_size = size;
    if (dim == 2) this->m_size.z = 1;
    this->m_channels = channels;
    m_views.clear();
    m_dev = std::move(data);
    this->m_data_multichannel.assign(channels, ComplexVector<T>());
    m_host_valid = false;
    m_dev_valid = true;
}

template <typename T>
void cuImageData<T>::addChannelImage(std::unique_ptr<cuComplexVector<T>> image)
{
    if (image == nullptr) return;
    const std::size_t cells = this->dataSize();
    if (image->size() != cells) {
        std::cerr << "Error: ImageData wrong size!" << std::endl;
        exit(1);
    }
    cuData();
    fillHost();
    cuComplexVector<T> grown(cells * (this->m_channels + 1));
    if (this->m_channels)
        fastrecon::cuda_check(cudaMemcpy(grown.data(), m_dev.data(), cells * this->m_channels * sizeof(cuComplex),
                                         cudaMemcpyDeviceToDevice),
                              "cuImageData grow");
    fastrecon::cuda_check(cudaMemcpy(grown.data() + cells * this->m_channels, image->data(),
                                     cells * sizeof(cuComplex), cudaMemcpyDeviceToDevice),
                          "cuImageData add");
    m_views.clear();
    m_dev = std::move(grown);
    this->m_data_multichannel.emplace_back(cells);
    fastrecon::cuda_check(cudaMemcpy(this->m_data_multichannel.back().data(), image->data(),
                                     cells * sizeof(cuComplex), cudaMemcpyDeviceToHost),
                          "cuImageData add");
    this->m_channels = this->m_data_multichannel.size();
}

template <typename T>
cuComplexVector<T> *cuImageData<T>::cuGetChannelImage(int channel)
{
    if (channel < 0 || channel >= this->channels()) return nullptr;
    const std::size_t cells = this->dataSize();
    cuComplex *base = cuData();
    m_views.emplace_back(new cuComplexVector<T>(cuComplexVector<T>::view(base + (std::size_t)channel * cells, cells)));
    cuMarkModified();
    return m_views.back().get();
}

template <typename T>
void cuImageData<T>::syncDeviceToHost()
{
    fillHost();
}

template <typename T>
void cuImageData<T>::invalidateDevice()
{
    fillHost();
    m_dev_valid = false;
}

template <typename T>
const ComplexVector<T> *cuImageData<T>::getChannelImage(int channel) const
{
    fillHost();
    return ImageData<T>::getChannelImage(channel);
}

template <typename T>
ComplexVector<T> *cuImageData<T>::getChannelImage(int channel)
{
    fillHost();
    m_dev_valid = false;  // the caller may modify the host copy
    return ImageData<T>::getChannelImage(channel);
}

template <typename T>
void cuImageData<T>::addChannelImage(ComplexVector<T> &&image)
{
    fillHost();
    ImageData<T>::addChannelImage(std::move(image));
    m_dev_valid = false;
}

template <typename T>
void cuImageData<T>::copy(const ImageData<T> &imageData)
{
    auto cu = dynamic_cast<const cuImageData<T> *>(&imageData);
    m_views.clear();
    if (cu && !cu->m_host_valid) {
        this->m_dim = cu->m_dim;
        this->m_size = cu->m_size;
        this->m_channels = cu->m_channels;
        this->m_data_multichannel.assign(cu->m_channels, ComplexVector<T>());
        m_dev = cu->m_dev;
        m_host_valid = false;
        m_dev_valid = true;
        return;
    }
    ImageData<T>::copy(imageData);
    m_host_valid = true;
    m_dev_valid = false;
}

template <typename T>
void cuImageData<T>::move(ImageData<T> &imageData)
{
    auto cu = dynamic_cast<cuImageData<T> *>(&imageData);
    m_views.clear();
    if (cu)
        this->moveFields(imageData);
    else
        ImageData<T>::move(imageData);
    if (cu) {
        m_dev.swap(cu->m_dev);
        m_host_valid = cu->m_host_valid;
        m_dev_valid = cu->m_dev_valid;
        cu->m_views.clear();
        cu->m_host_valid = true;
        cu->m_dev_valid = true;
    } else {
        m_host_valid = true;
        m_dev_valid = false;
    }
}

template class cuImageData<float>;
