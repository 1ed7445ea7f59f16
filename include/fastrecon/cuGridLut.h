// cuGridLut.h -- GPU gridding (ReconData/cuGridLut.h:31-57), backed by the
// C ABI of libfastrecon_gb300.so (fr_plan_*, fr_grid).
//
// Differences from the reference: the plan belongs to this object and is
// built for this object's trajectory (the reference caches one plan per
// process, keyed on nothing, cuGridLut.cu:14-18,158-159).  Partitions
// (setNumOfPartitions) are used only when the single plan does not fit in
// device memory: execute() then grids sample ranges with
// fr_grid_partitioned (at least 2 partitions, doubled while a partition's
// plan still does not fit) instead of chunking a host-side pair map.
#ifndef FASTRECON_CUGRIDLUT_H
#define FASTRECON_CUGRIDLUT_H

#include "GridLut.h"
#include "cuImageData.h"
#include "cuReconData.h"

struct fr_plan_s;

template <typename T>
class cuGridLut : public GridLut<T> {
public:
    cuGridLut(cuReconData<T> &reconData);
    virtual ~cuGridLut();

    virtual void plan(unsigned reconSize, float overGridFactor, float kWidth, unsigned klength = 32) override;
    virtual std::shared_ptr<ImageData<T>> execute() override;
    void setNumOfPartitions(int partitions) { m_gpu_partitions = partitions; }

    // Tile shape and coils per scatter pass used by the next plan() (0 = default).
    void setTiling(int tx, int ty, int tz, int coilGroup);
    // Grid into an existing image whose device buffer holds channels x G^d (no allocation).
    void executeInto(cuImageData<T> &img);
    // Whether the last execute() regridded only the acquisitions updated
    // since the one before (ReconData::updateSingleAcquisition) instead of
    // the whole k-space.
    bool lastExecuteIncremental() const { return m_last_incremental; }
    // Sample partitions of the last execute() (0: one plan).
    int lastExecutePartitions() const { return m_last_partitions; }

private:
    cuReconData<T> &m_cuData;
    fr_plan_s *m_plan = nullptr;
    int m_gpu_partitions = 1;
    // the single plan did not fit: grid in sample partitions
    bool m_partitioned = false;
    int m_last_partitions = 0;
    float m_kwidth = 0.f;
    void gridAll(float *d_grid);
    int m_tile[3] = {0, 0, 0};
    int m_coil_group = 0;
    // streaming acquisitions: the grid of the last execute(), kept once the
    // data has seen single-acquisition updates
    std::unique_ptr<cuComplexVector<T>> m_grid_cache;
    unsigned long long m_cache_generation = 0;
    int m_cache_channels = 0;
    bool m_last_incremental = false;
};

#endif  // FASTRECON_CUGRIDLUT_H
