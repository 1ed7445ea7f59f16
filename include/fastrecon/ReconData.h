// ReconData.h -- k-space samples, trajectory and DCF (ReconData/ReconData.h:18-65).
//
// Same interface as the reference with the Qt types replaced by standard ones:
// loadFromFiles takes std::vector<std::string> / std::string (QStringList /
// QString), loadTraj takes std::vector<T> (QVector<T>).  Error behaviour is the
// reference's: size mismatches print and exit(1), a bad channel prints and
// returns.
#ifndef FASTRECON_RECONDATA_H
#define FASTRECON_RECONDATA_H

#include <complex>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "common.h"

template <typename T>
struct Point {
    T x[4];
};

template <typename T>
class ReconData {
protected:
    ReconData(int samples, int acquisitions);

public:
    typedef std::vector<Point<T>> TrajVector;
    // The GB300 build has no CPU gridding path: the returned object is always
    // a cuReconData (the gpu flag is accepted for source compatibility).
    static std::shared_ptr<ReconData<T>> Create(int samples, int acquisitions, bool gpu = false);
    virtual ~ReconData() {}

    void loadFromFiles(const std::vector<std::string> &dataFileList, const std::vector<std::string> &trajFileList,
                       const std::string &dcfFileName);
    void addChannelData(ComplexVector<T> &&data);
    void setDcf(std::vector<T> &dcf);
    void loadTraj(const std::vector<T> &traj, int dim);
    virtual void updateSingleAcquisition(const std::complex<T> *data, int acquisition, int channel = 0);
    void normalizeTraj(unsigned size);
    std::pair<T, T> getCompBounds(int comp) const { return m_bounds[comp]; }
    int dataSize() const { return m_size; }
    int rcDim() const { return m_dim; }
    const TrajVector &getTraj() const { return m_traj; }
    const std::vector<T> &getDcf() const { return m_dcf; }
    const ComplexVector<T> *getChannelData(int channel) const;
    int channels() const { return m_kDataMultiChannel.size(); }
    virtual void clear();

protected:
    int m_samples;
    int m_acquisitions;
    std::size_t m_size;
    int m_dim = 0;
    std::vector<std::pair<T, T>> m_bounds;

    TrajVector m_traj;
    std::vector<ComplexVector<T>> m_kDataMultiChannel;
    std::vector<T> m_dcf;

    // Host data changed: device caches must be rebuilt.
    virtual void hostChanged() {}

private:
    virtual void transformLocalTraj(T translation, T scale) = 0;
    void storeTrajComponent(const std::vector<T> &traj_c);
};

#endif  // FASTRECON_RECONDATA_H
