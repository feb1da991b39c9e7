// Shared helpers for the dmgb CUDA sources: error reporting, launch shapes,
// block-level scans and float atomics on an order-preserving integer map.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <string>

#include "../../include/dmgb.h"

namespace dm {

// Last error message of this host thread (returned by dm_last_error).
void set_error(const char *fmt, ...);
const char *last_error();

#define DM_CUDA_TRY(call)                                                   \
  do {                                                                      \
    cudaError_t e_ = (call);                                                \
    if (e_ != cudaSuccess) {                                                \
      ::dm::set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                      __FILE__, __LINE__);                                  \
      return DM_ERR_CUDA;                                                   \
    }                                                                       \
  } while (0)

#define DM_LAUNCH_CHECK()                                                   \
  do {                                                                      \
    cudaError_t e_ = cudaGetLastError();                                    \
    if (e_ != cudaSuccess) {                                                \
      ::dm::set_error("kernel launch failed: %s (%s:%d)",                   \
                      cudaGetErrorString(e_), __FILE__, __LINE__);          \
      return DM_ERR_CUDA;                                                   \
    }                                                                       \
  } while (0)

#define DM_ARG_CHECK(cond, msg)                                             \
  do {                                                                      \
    if (!(cond)) {                                                          \
      ::dm::set_error("invalid argument: %s", msg);                         \
      return DM_ERR_ARG;                                                    \
    }                                                                       \
  } while (0)

constexpr int kSMs = 152;  // GB300: 2 dies x 76 SMs

inline int grid_for(int64_t n, int threads, int max_blocks = 152 * 16) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > max_blocks) b = max_blocks;
  return (int)b;
}

inline size_t align_up(size_t x, size_t a = 256) { return (x + a - 1) / a * a; }

// Bump allocator over a caller-provided workspace.
struct Carve {
  char *base;
  size_t used, cap;
  Carve(void *b, size_t c) : base((char *)b), used(0), cap(c) {}
  template <typename T>
  T *take(size_t count) {
    size_t off = align_up(used);
    used = off + count * sizeof(T);
    return base ? (T *)(base + off) : nullptr;
  }
  bool ok() const { return used <= cap; }
};

// order-preserving map float <-> int for atomicMin/atomicMax on floats
__device__ __forceinline__ int f2o(float f) {
  int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float o2f(int i) {
  return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff);
}

__device__ __forceinline__ void flag_or(int64_t *counters, int64_t bits) {
  atomicOr((unsigned long long *)&counters[DM_CNT_FLAGS],
           (unsigned long long)bits);
}

// warp-aggregated increment of a 64-bit counter; returns this lane's slot
__device__ __forceinline__ int64_t warp_append(int64_t *ctr, bool want) {
  unsigned m = __ballot_sync(0xffffffffu, want);
  if (!m) return -1;
  int lane = threadIdx.x & 31;
  int leader = __ffs(m) - 1;
  int64_t base = 0;
  if (lane == leader)
    base = (int64_t)atomicAdd((unsigned long long *)ctr,
                              (unsigned long long)__popc(m));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (!want) return -1;
  return base + __popc(m & ((1u << lane) - 1));
}

// Exclusive scan of int32 counts (n < 2^32) into out[0..n]; out[n] = total.
// tmp must hold >= scan_tmp_elems(n) ints (block sums, and above 4M
// elements their scan and a second level of sums).
inline int64_t scan_tmp_elems(int64_t n) {
  const int64_t nb = (n + 1023) / 1024 + 1;
  return 2 * (nb + 1) + (nb + 1023) / 1024 + 16;
}
int exclusive_scan_i32(const int32_t *in, int32_t *out, int64_t n,
                       int32_t *tmp, cudaStream_t s);

}  // namespace dm
