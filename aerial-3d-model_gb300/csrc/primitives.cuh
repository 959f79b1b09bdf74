// Device primitives used to build the per-call problem structure: a
// stream-ordered buffer, an exclusive scan and a stable LSD radix sort.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <stdexcept>
#include <string>
#include <utility>

namespace ba {

struct CudaError : std::runtime_error {
  cudaError_t code;
  CudaError(cudaError_t c, const std::string& what)
      : std::runtime_error(what + ": " + cudaGetErrorString(c)), code(c) {}
};

inline void check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw CudaError(e, what);
}

// Counts kernels launched through the library (reported in ba_stats).
extern thread_local int64_t g_launches;
#define BA_LAUNCH(...)                                    \
  do {                                                    \
    __VA_ARGS__;                                          \
    ::ba::g_launches++;                                   \
    ::ba::check(cudaGetLastError(), "kernel launch");     \
  } while (0)

// Device bytes held by DevBuf buffers of the calling thread, and the peak.
inline size_t& dev_bytes_live() {
  static thread_local size_t v = 0;
  return v;
}
inline size_t& dev_bytes_peak() {
  static thread_local size_t v = 0;
  return v;
}

// Device-memory budget of the current call on this thread: DevBuf
// allocations that would take the bytes held since the call began above
// `limit` fail with cudaErrorMemoryAllocation (BA_OOM) before cudaMallocAsync
// is called.  limit 0: no budget.
struct DevBudget {
  int64_t limit = 0, base = 0;
};
inline DevBudget& dev_budget() {
  static thread_local DevBudget b;
  return b;
}
// Sets the budget for its scope; an enclosing budget (ba_solve around its
// upload and solve) stays in force.
struct DevBudgetScope {
  bool set = false;
  explicit DevBudgetScope(int64_t limit) {
    if (limit > 0 && dev_budget().limit == 0) {
      dev_budget() = DevBudget{limit, (int64_t)dev_bytes_live()};
      set = true;
    }
  }
  ~DevBudgetScope() {
    if (set) dev_budget() = DevBudget{};
  }
  DevBudgetScope(const DevBudgetScope&) = delete;
  DevBudgetScope& operator=(const DevBudgetScope&) = delete;
};

// Stream-ordered device buffer (cudaMallocAsync from the device's default
// pool, whose release threshold the context raises so freed blocks are
// reused by the next solve instead of being returned to the driver).
template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaStream_t s = nullptr;
  DevBuf() = default;
  DevBuf(size_t count, cudaStream_t st) { alloc(count, st); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept { *this = std::move(o); }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p, n = o.n, s = o.s;
      o.p = nullptr, o.n = 0;
    }
    return *this;
  }
  ~DevBuf() { release(); }
  void alloc(size_t count, cudaStream_t st) {
    release();
    s = st;
    n = count;
    if (count) {
      const DevBudget& bud = dev_budget();
      if (bud.limit > 0 &&
          (int64_t)dev_bytes_live() - bud.base + (int64_t)(count * sizeof(T)) > bud.limit) {
        n = 0;
        throw CudaError(cudaErrorMemoryAllocation,
                        "device allocation of " + std::to_string(count * sizeof(T)) +
                            " bytes beyond the call's workspace limit of " +
                            std::to_string(bud.limit) + " bytes");
      }
      cudaError_t e = cudaMallocAsync((void**)&p, count * sizeof(T), st);
      if (e != cudaSuccess) {
        p = nullptr;
        n = 0;
        throw CudaError(e, "device allocation of " +
                               std::to_string(count * sizeof(T)) + " bytes");
      }
      dev_bytes_live() += count * sizeof(T);
      if (dev_bytes_live() > dev_bytes_peak()) dev_bytes_peak() = dev_bytes_live();
    }
  }
  void release() {
    if (p) {
      cudaFreeAsync(p, s);
      dev_bytes_live() -= n * sizeof(T);
    }
    p = nullptr;
    n = 0;
  }
  void zero() {
    if (n) check(cudaMemsetAsync(p, 0, n * sizeof(T), s), "memset");
  }
  size_t bytes() const { return n * sizeof(T); }
  operator T*() const { return p; }
};

// out[i] = sum_{j<i} in[i]; returns the total (synchronises the stream).
// `in` and `out` may alias.
uint64_t exclusive_scan_u32(const uint32_t* in, uint32_t* out, size_t n,
                            cudaStream_t s);

// Stable LSD radix sort of (key, value) pairs on the low `bits` bits of the
// keys.  The result is left in keys/vals; the *_tmp arrays are scratch of the
// same length.
void radix_sort_u64_u32(uint64_t* keys, uint32_t* vals, uint64_t* keys_tmp,
                        uint32_t* vals_tmp, size_t n, int bits,
                        cudaStream_t s);
void radix_sort_u64_u64(uint64_t* keys, uint64_t* vals, uint64_t* keys_tmp,
                        uint64_t* vals_tmp, size_t n, int bits,
                        cudaStream_t s);

// p[i] = lower_bound(sorted[0..n), i) for i in [0, m].
void lower_bounds_u32(const uint32_t* sorted, size_t n, uint32_t* p, size_t m,
                      cudaStream_t s);
void lower_bounds_u64(const uint64_t* sorted, size_t n, uint32_t* p, size_t m,
                      uint64_t key_mul, cudaStream_t s);

inline unsigned grid_for(size_t n, unsigned block) {
  size_t g = (n + block - 1) / block;
  if (g == 0) g = 1;
  if (g > 0x7fffffffu) g = 0x7fffffffu;
  return (unsigned)g;
}

}  // namespace ba
