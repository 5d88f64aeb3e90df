// Device-resident stores of factor measurements and pose values.
//
// The host keeps only what the reference's bookkeeping needs (factor kinds
// and keys, the key -> row maps); measured poses, covariances,
// square-root informations and the current values live in HBM and are
// gathered by row on the device by the kernels that use them.
#pragma once
#include <cstdint>
#include <map>
#include <vector>

#include "common.cuh"

namespace rpgo {

struct FactorRec {
  int32_t kind = 0;  // 0 between, 1 prior
  uint64_t k1 = 0, k2 = 0;
  int64_t row = 0;   // row in the FactorStore
};

// dst[k * width + c] = src[idx[k] * width + c]
void gather_rows(int64_t n, const int64_t* idx, const double* src, int width, double* dst, cudaStream_t st);
// dst[idx[k] * width + c] = src[k * width + c]
void scatter_rows(int64_t n, const int64_t* idx, const double* src, int width, double* dst, cudaStream_t st);

class FactorStore {
 public:
  FactorStore(int stride, int d) : stride_(stride), dd_(d * d) {}
  // appends n rows; pointers are host (on_device = false) or device arrays
  int64_t append(int64_t n, const double* meas, const double* cov, const double* sqrt_info, bool on_device,
                 cudaStream_t st);
  const double* meas() const { return meas_.get(); }
  const double* cov() const { return cov_.get(); }
  const double* sqrt_info() const { return sqrt_.get(); }
  int64_t rows() const { return rows_; }
  // host copy of one row's measured pose (for getters / saveData)
  void download_meas(const std::vector<int64_t>& rows, std::vector<double>* out, cudaStream_t st) const;
  void download_sqrt(const std::vector<int64_t>& rows, std::vector<double>* out, cudaStream_t st) const;

 private:
  int stride_, dd_;
  int64_t rows_ = 0;
  DeviceBuffer<double> meas_, cov_, sqrt_;
};

class ValueStore {
 public:
  explicit ValueStore(int stride) : stride_(stride) {}
  bool has(uint64_t k) const { return row_.count(k) != 0; }
  int64_t row(uint64_t k) const { return row_.at(k); }
  size_t size() const { return row_.size(); }
  const std::map<uint64_t, int64_t>& rows() const { return row_; }
  // appends poses for new keys (caller checked uniqueness)
  void append(int64_t n, const uint64_t* keys, const double* poses, bool on_device, cudaStream_t st);
  double* pose() { return pose_.get(); }
  const double* pose() const { return pose_.get(); }
  int stride() const { return stride_; }
  // values in key order (host)
  void download_sorted(std::vector<uint64_t>* keys, std::vector<double>* poses, cudaStream_t st) const;

 private:
  int stride_;
  std::map<uint64_t, int64_t> row_;
  int64_t rows_ = 0;
  DeviceBuffer<double> pose_;
};

}  // namespace rpgo
