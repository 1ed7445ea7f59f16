// ConvKernel.h -- radial Kaiser-Bessel kernel LUT (ReconData/ConvKernel.h:7-22).
#ifndef FASTRECON_CONVKERNEL_H
#define FASTRECON_CONVKERNEL_H

#include <memory>
#include <vector>

#include "common.h"

class ConvKernel {
public:
    ConvKernel(float kWidth, float overGridFactor, int length = 32);
    ~ConvKernel();

    const std::vector<float> *getKernelData() const;
    float getKernelWidth() const;

private:
    float m_kWidth;
    float m_ogFactor;
    int m_length;

    std::shared_ptr<std::vector<float>> m_kernelData;
};

#endif  // FASTRECON_CONVKERNEL_H
