// Shared CUDA plumbing for the rpgo_gb300 library: error handling, device
// buffers, launch accounting.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

namespace rpgo {

struct CudaError : std::runtime_error {
  explicit CudaError(const std::string& s) : std::runtime_error(s) {}
};

inline void cuda_check(cudaError_t e, const char* what, const char* file, int line) {
  if (e != cudaSuccess) {
    char buf[512];
    std::snprintf(buf, sizeof(buf), "%s failed at %s:%d: %s", what, file, line, cudaGetErrorString(e));
    throw CudaError(buf);
  }
}
#define RPGO_CUDA(x) ::rpgo::cuda_check((x), #x, __FILE__, __LINE__)
#define RPGO_LAUNCHED() ::rpgo::note_launch(cudaGetLastError(), __FILE__, __LINE__)

// Count of kernels this library has launched (process-wide), and by the
// calling host thread (per-update figures of concurrent solvers stay apart).
std::atomic<int64_t>& launch_counter();
int64_t& thread_launch_counter();
// device and pinned host allocations made by this library's buffers (process-wide)
std::atomic<int64_t>& alloc_counter();

// Device memory is stream-ordered (cudaMallocAsync / cudaFreeAsync from the
// device's default pool): a free never synchronises the device, so solvers on
// different streams and host threads run concurrently. Every buffer is
// allocated and freed on the calling thread's allocation stream, which each C
// ABI entry point sets to the stream its work runs on (AllocStreamScope).
cudaStream_t& alloc_stream();
class AllocStreamScope {
 public:
  explicit AllocStreamScope(cudaStream_t st) : prev_(alloc_stream()) { alloc_stream() = st; }
  ~AllocStreamScope() { alloc_stream() = prev_; }
  AllocStreamScope(const AllocStreamScope&) = delete;
  AllocStreamScope& operator=(const AllocStreamScope&) = delete;

 private:
  cudaStream_t prev_;
};

// Device time of the dominant kernels, measured with CUDA events on the
// launching stream (running sums of the calling host thread).
struct KernelTimes {
  double pcg_ms = 0.0, pcg_bytes = 0.0;
  int64_t pcg_launches = 0;
  double pair_ms = 0.0;
  int64_t pair_launches = 0;
  double chol_ms = 0.0, chol_flops = 0.0, chol_bytes = 0.0;
  int64_t chol_levels = 0, chol_tail = 0;  // of the last plan used
  int64_t chol_launches = 0;
};
KernelTimes& kernel_times();

// RAII pair of events around one launch; elapsed() synchronises the end event.
class EventTimer {
 public:
  explicit EventTimer(cudaStream_t st) : st_(st) {
    cudaEventCreate(&a_);
    cudaEventCreate(&b_);
    cudaEventRecord(a_, st_);
  }
  ~EventTimer() {
    cudaEventDestroy(a_);
    cudaEventDestroy(b_);
  }
  double elapsed_ms() {
    cudaEventRecord(b_, st_);
    cudaEventSynchronize(b_);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a_, b_);
    return ms;
  }

 private:
  cudaStream_t st_;
  cudaEvent_t a_, b_;
};
inline void note_launch(cudaError_t e, const char* file, int line) {
  cuda_check(e, "kernel launch", file, line);
  launch_counter().fetch_add(1, std::memory_order_relaxed);
  ++thread_launch_counter();
}

template <class T>
class DeviceBuffer {
 public:
  DeviceBuffer() = default;
  explicit DeviceBuffer(size_t n) { resize(n); }
  DeviceBuffer(const DeviceBuffer&) = delete;
  DeviceBuffer& operator=(const DeviceBuffer&) = delete;
  DeviceBuffer(DeviceBuffer&& o) noexcept : p_(o.p_), n_(o.n_), cap_(o.cap_), st_(o.st_) {
    o.p_ = nullptr; o.n_ = o.cap_ = 0;
  }
  DeviceBuffer& operator=(DeviceBuffer&& o) noexcept {
    if (this != &o) {
      release();
      p_ = o.p_; n_ = o.n_; cap_ = o.cap_; st_ = o.st_;
      o.p_ = nullptr; o.n_ = o.cap_ = 0;
    }
    return *this;
  }
  ~DeviceBuffer() { release(); }
  // resize without preserving contents
  void resize(size_t n) {
    if (n > cap_) {
      release();
      size_t c = n < 16 ? 16 : n;
      alloc_counter().fetch_add(1, std::memory_order_relaxed);
      RPGO_CUDA(cudaMallocAsync((void**)&p_, c * sizeof(T), alloc_stream()));
      st_ = alloc_stream();
      cap_ = c;
    }
    n_ = n;
  }
  // grow keeping the first n_ elements (capacity doubles); st must be the
  // allocation stream or ordered after it
  void grow(size_t n, cudaStream_t st) {
    if (n > cap_) {
      size_t c = cap_ ? cap_ : 16;
      while (c < n) c *= 2;
      T* q = nullptr;
      alloc_counter().fetch_add(1, std::memory_order_relaxed);
      RPGO_CUDA(cudaMallocAsync((void**)&q, c * sizeof(T), alloc_stream()));
      if (p_ && n_) RPGO_CUDA(cudaMemcpyAsync(q, p_, n_ * sizeof(T), cudaMemcpyDeviceToDevice, st));
      release();
      p_ = q;
      st_ = alloc_stream();
      cap_ = c;
    }
    n_ = n;
  }
  void upload(const T* h, size_t n, cudaStream_t st) {
    resize(n);
    if (n) RPGO_CUDA(cudaMemcpyAsync(p_, h, n * sizeof(T), cudaMemcpyHostToDevice, st));
  }
  void upload(const std::vector<T>& h, cudaStream_t st) { upload(h.data(), h.size(), st); }
  void download(T* h, size_t n, cudaStream_t st) const {
    if (n) RPGO_CUDA(cudaMemcpyAsync(h, p_, n * sizeof(T), cudaMemcpyDeviceToHost, st));
  }
  void zero(cudaStream_t st) {
    if (n_) RPGO_CUDA(cudaMemsetAsync(p_, 0, n_ * sizeof(T), st));
  }
  T* get() const { return p_; }
  size_t size() const { return n_; }

 private:
  // freed on the stream the buffer was allocated on: every use of a buffer
  // is on that stream (or synchronised before the free)
  void release() {
    if (p_) cudaFreeAsync(p_, st_);
    p_ = nullptr;
    n_ = cap_ = 0;
  }
  T* p_ = nullptr;
  size_t n_ = 0, cap_ = 0;
  cudaStream_t st_ = nullptr;
};

// A few page-locked host words for device-to-host copies that must not block
// the host until a later synchronisation (pageable copies synchronise).
template <class T>
class PinnedBuffer {
 public:
  PinnedBuffer() = default;
  PinnedBuffer(const PinnedBuffer&) = delete;
  PinnedBuffer& operator=(const PinnedBuffer&) = delete;
  ~PinnedBuffer() {
    if (p_) cudaFreeHost(p_);
  }
  T* get(size_t n) {
    if (n > n_) {
      if (p_) cudaFreeHost(p_);
      p_ = nullptr;
      alloc_counter().fetch_add(1, std::memory_order_relaxed);
      RPGO_CUDA(cudaMallocHost((void**)&p_, n * sizeof(T)));
      n_ = n;
    }
    return p_;
  }

 private:
  T* p_ = nullptr;
  size_t n_ = 0;
};

inline int div_up(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

// SM count of the current device (looked up once per process).
inline int device_sm_count() {
  static const int sms = [] {
    int dev = 0, n = 0;
    RPGO_CUDA(cudaGetDevice(&dev));
    RPGO_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
    return n;
  }();
  return sms;
}

}  // namespace rpgo
