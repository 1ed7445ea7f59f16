// GridLut.h -- gridding (ReconData/GridLut.h:9-42).
//
// Create() returns a cuGridLut for the cuReconData every ReconData::Create
// returns; plan() normalises the trajectory in place (as the reference does,
// GridLut.cpp:41-51) and bins it; execute() grids every channel on the GPU and
// returns a cuImageData.
#ifndef FASTRECON_GRIDLUT_H
#define FASTRECON_GRIDLUT_H

#include "ImageData.h"
#include "ReconData.h"

class ConvKernel;

template <typename T>
class GridLut {
protected:
    GridLut(ReconData<T> &reconData);

public:
    virtual ~GridLut();
    static std::shared_ptr<GridLut<T>> Create(ReconData<T> &reconData);

    virtual void plan(unsigned reconSize, float overGridFactor, float kWidth, unsigned klength = 32);
    virtual std::shared_ptr<ImageData<T>> execute() = 0;
    void setNumOfThreads(unsigned threads) { m_num_threads = threads; }
    void setIndex(int index) { m_index = index; }

protected:
    ReconData<T> &m_associatedData;
    unsigned m_dim = 0;
    unsigned m_gridSize = 0;
    ConvKernel *m_kernel = nullptr;

    unsigned m_num_threads = 1;  // accepted for compatibility; the GPU path ignores it
    int m_index = 0;
};

#endif  // FASTRECON_GRIDLUT_H
