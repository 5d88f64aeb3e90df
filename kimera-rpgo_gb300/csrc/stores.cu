// Device stores and the row gather / scatter kernels; see stores.hpp.
#include "stores.hpp"

namespace rpgo {
namespace {

__global__ void k_gather_rows(int64_t n, const int64_t* __restrict__ idx, const double* __restrict__ src, int width,
                              double* __restrict__ dst) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n * width) return;
  const int64_t k = t / width, c = t % width;
  dst[t] = src[idx[k] * width + c];
}
__global__ void k_scatter_rows(int64_t n, const int64_t* __restrict__ idx, const double* __restrict__ src, int width,
                               double* __restrict__ dst) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n * width) return;
  const int64_t k = t / width, c = t % width;
  dst[idx[k] * width + c] = src[t];
}

}  // namespace

void gather_rows(int64_t n, const int64_t* idx, const double* src, int width, double* dst, cudaStream_t st) {
  if (n <= 0) return;
  k_gather_rows<<<div_up(n * width, 256), 256, 0, st>>>(n, idx, src, width, dst);
  RPGO_LAUNCHED();
}
void scatter_rows(int64_t n, const int64_t* idx, const double* src, int width, double* dst, cudaStream_t st) {
  if (n <= 0) return;
  k_scatter_rows<<<div_up(n * width, 256), 256, 0, st>>>(n, idx, src, width, dst);
  RPGO_LAUNCHED();
}

int64_t FactorStore::append(int64_t n, const double* meas, const double* cov, const double* sqrt_info,
                            bool on_device, cudaStream_t st) {
  const int64_t first = rows_;
  if (n <= 0) return first;
  meas_.grow((size_t)(rows_ + n) * stride_, st);
  cov_.grow((size_t)(rows_ + n) * dd_, st);
  sqrt_.grow((size_t)(rows_ + n) * dd_, st);
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  RPGO_CUDA(cudaMemcpyAsync(meas_.get() + (size_t)rows_ * stride_, meas, (size_t)n * stride_ * sizeof(double), kind,
                            st));
  RPGO_CUDA(cudaMemcpyAsync(cov_.get() + (size_t)rows_ * dd_, cov, (size_t)n * dd_ * sizeof(double), kind, st));
  RPGO_CUDA(cudaMemcpyAsync(sqrt_.get() + (size_t)rows_ * dd_, sqrt_info, (size_t)n * dd_ * sizeof(double), kind,
                            st));
  rows_ += n;
  return first;
}

void FactorStore::download_meas(const std::vector<int64_t>& rows, std::vector<double>* out, cudaStream_t st) const {
  out->assign(rows.size() * stride_, 0.0);
  if (rows.empty()) return;
  DeviceBuffer<int64_t> idx;
  idx.upload(rows, st);
  DeviceBuffer<double> tmp(rows.size() * stride_);
  gather_rows((int64_t)rows.size(), idx.get(), meas_.get(), stride_, tmp.get(), st);
  tmp.download(out->data(), out->size(), st);
  RPGO_CUDA(cudaStreamSynchronize(st));
}
void FactorStore::download_sqrt(const std::vector<int64_t>& rows, std::vector<double>* out, cudaStream_t st) const {
  out->assign(rows.size() * dd_, 0.0);
  if (rows.empty()) return;
  DeviceBuffer<int64_t> idx;
  idx.upload(rows, st);
  DeviceBuffer<double> tmp(rows.size() * dd_);
  gather_rows((int64_t)rows.size(), idx.get(), sqrt_.get(), dd_, tmp.get(), st);
  tmp.download(out->data(), out->size(), st);
  RPGO_CUDA(cudaStreamSynchronize(st));
}

void ValueStore::append(int64_t n, const uint64_t* keys, const double* poses, bool on_device, cudaStream_t st) {
  if (n <= 0) return;
  pose_.grow((size_t)(rows_ + n) * stride_, st);
  RPGO_CUDA(cudaMemcpyAsync(pose_.get() + (size_t)rows_ * stride_, poses, (size_t)n * stride_ * sizeof(double),
                            on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
  for (int64_t k = 0; k < n; ++k) row_[keys[k]] = rows_ + k;
  rows_ += n;
}

void ValueStore::download_sorted(std::vector<uint64_t>* keys, std::vector<double>* poses, cudaStream_t st) const {
  keys->clear();
  std::vector<int64_t> rows;
  for (const auto& kv : row_) {
    keys->push_back(kv.first);
    rows.push_back(kv.second);
  }
  poses->assign(rows.size() * stride_, 0.0);
  if (rows.empty()) return;
  DeviceBuffer<int64_t> idx;
  idx.upload(rows, st);
  DeviceBuffer<double> tmp(rows.size() * stride_);
  gather_rows((int64_t)rows.size(), idx.get(), pose_.get(), stride_, tmp.get(), st);
  tmp.download(poses->data(), poses->size(), st);
  RPGO_CUDA(cudaStreamSynchronize(st));
}

}  // namespace rpgo
