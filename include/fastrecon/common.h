// common.h -- common types of the fastrecon C++ API (ImageData/common.h).
//
// ImageSize, hostVector and ComplexVector are the reference's
// (ImageData/common.h:7-18).  The device containers stand in for the
// reference's thrust::device_vector aliases (common.h:20-46): cuVector<T> is a
// plain owning (or viewing) CUDA allocation, so user code compiles with any
// C++ compiler and the CUDA runtime headers.
#ifndef FASTRECON_COMMON_H
#define FASTRECON_COMMON_H

#include <cuComplex.h>
#include <cuda_runtime.h>

#include <complex>
#include <cstddef>
#include <stdexcept>
#include <string>
#include <vector>

typedef struct {
    unsigned x;
    unsigned y;
    unsigned z;
} ImageSize;

template <typename T>
using hostVector = std::vector<T>;

template <typename T>
using ComplexVector = hostVector<std::complex<T>>;

namespace fastrecon {
inline void cuda_check(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}
}  // namespace fastrecon

// Device array of T.  Owning by default; view() wraps memory owned elsewhere.
template <typename T>
class cuVector {
public:
    typedef T value_type;
    cuVector() {}
    explicit cuVector(std::size_t n) { resize(n); }
    explicit cuVector(const std::vector<T> &host) { assign(host.data(), host.size()); }
    cuVector(const cuVector &o) { assign_device(o.data(), o.size()); }
    cuVector(cuVector &&o) noexcept { swap(o); }
    cuVector &operator=(const cuVector &o)
    {
        if (this != &o) assign_device(o.data(), o.size());
        return *this;
    }
    cuVector &operator=(cuVector &&o) noexcept
    {
        swap(o);
        return *this;
    }
    cuVector &operator=(const std::vector<T> &host)
    {
        assign(host.data(), host.size());
        return *this;
    }
    ~cuVector() { release(); }

    static cuVector view(T *ptr, std::size_t n)
    {
        cuVector v;
        v.m_ptr = ptr;
        v.m_n = n;
        v.m_own = false;
        return v;
    }

    std::size_t size() const { return m_n; }
    bool empty() const { return m_n == 0; }
    T *data() { return m_ptr; }
    const T *data() const { return m_ptr; }

    // Contents are not preserved.
    void resize(std::size_t n)
    {
        if (n == m_n && (m_own || !m_ptr)) return;
        release();
        if (n) fastrecon::cuda_check(cudaMalloc(reinterpret_cast<void **>(&m_ptr), n * sizeof(T)), "cudaMalloc");
        m_n = n;
        m_own = true;
    }
    void assign(const T *host, std::size_t n)
    {
        resize(n);
        if (n) fastrecon::cuda_check(cudaMemcpy(m_ptr, host, n * sizeof(T), cudaMemcpyHostToDevice), "upload");
    }
    void assign_device(const T *dev, std::size_t n)
    {
        resize(n);
        if (n) fastrecon::cuda_check(cudaMemcpy(m_ptr, dev, n * sizeof(T), cudaMemcpyDeviceToDevice), "copy");
    }
    void copy_to_host(T *host) const
    {
        if (m_n) fastrecon::cuda_check(cudaMemcpy(host, m_ptr, m_n * sizeof(T), cudaMemcpyDeviceToHost), "download");
    }
    std::vector<T> to_host() const
    {
        std::vector<T> h(m_n);
        copy_to_host(h.data());
        return h;
    }
    void swap(cuVector &o) noexcept
    {
        std::swap(m_ptr, o.m_ptr);
        std::swap(m_n, o.m_n);
        std::swap(m_own, o.m_own);
    }

private:
    void release()
    {
        if (m_own && m_ptr) cudaFree(m_ptr);
        m_ptr = nullptr;
        m_n = 0;
        m_own = true;
    }
    T *m_ptr = nullptr;
    std::size_t m_n = 0;
    bool m_own = true;
};

template <typename T>
struct cuComplexVectorType {
};

template <>
struct cuComplexVectorType<float> {
    typedef cuVector<cuComplex> type;
};

template <typename T>
using cuComplexVector = typename cuComplexVectorType<T>::type;

#endif  // FASTRECON_COMMON_H
