// Error reporting and the exclusive scan used by the counting sorts.
#include <stdarg.h>

#include "dm_common.cuh"

namespace dm {

static thread_local std::string g_last_error;

void set_error(const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

const char *last_error() { return g_last_error.c_str(); }

// ---- three-phase exclusive scan (1024 elements per block of 256 threads)
__device__ __forceinline__ int warp_incl_scan(int v) {
  int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// block-wide exclusive scan of one value per thread; returns the block total
template <int THREADS>
__device__ __forceinline__ int block_excl_scan(int v, int &excl) {
  __shared__ int wsum[THREADS / 32];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int incl = warp_incl_scan(v);
  if (lane == 31) wsum[w] = incl;
  __syncthreads();
  if (w == 0) {
    int s = lane < THREADS / 32 ? wsum[lane] : 0;
    int si = warp_incl_scan(s);
    if (lane < THREADS / 32) wsum[lane] = si - s;
  }
  __syncthreads();
  excl = incl - v + wsum[w];
  int total = 0;
  // total = last thread's inclusive value
  __shared__ int tot;
  if (threadIdx.x == THREADS - 1) tot = excl + v;
  __syncthreads();
  total = tot;
  __syncthreads();
  return total;
}

__global__ void k_scan_reduce(const int32_t *in, int64_t n, int32_t *bsum) {
  int64_t base = (int64_t)blockIdx.x * 1024;
  int s = 0;
  for (int k = 0; k < 4; ++k) {
    int64_t i = base + threadIdx.x + k * 256;
    if (i < n) s += in[i];
  }
  int ex;
  int tot = block_excl_scan<256>(s, ex);
  if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

__global__ void k_scan_bsums(int32_t *bsum, int nb) {
  // one block of 1024 threads, 4 sums each (nb <= 4096)
  int v[4], s = 0;
  for (int k = 0; k < 4; ++k) {
    int i = threadIdx.x * 4 + k;
    v[k] = i < nb ? bsum[i] : 0;
    s += v[k];
  }
  int ex;
  int tot = block_excl_scan<1024>(s, ex);
  for (int k = 0; k < 4; ++k) {
    int i = threadIdx.x * 4 + k;
    if (i < nb) bsum[i] = ex;
    ex += v[k];
  }
  if (threadIdx.x == 0) bsum[nb] = tot;
}

__global__ void k_scan_apply(const int32_t *in, int32_t *out, int64_t n,
                             const int32_t *bsum, int nb) {
  int64_t base = (int64_t)blockIdx.x * 1024 + threadIdx.x * 4;
  int v[4], s = 0;
  for (int k = 0; k < 4; ++k) {
    int64_t i = base + k;
    v[k] = i < n ? in[i] : 0;
    s += v[k];
  }
  int ex;
  block_excl_scan<256>(s, ex);
  ex += bsum[blockIdx.x];
  for (int k = 0; k < 4; ++k) {
    int64_t i = base + k;
    if (i < n) out[i] = ex;
    ex += v[k];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = bsum[nb];
}

int exclusive_scan_i32(const int32_t *in, int32_t *out, int64_t n,
                       int32_t *tmp, cudaStream_t s) {
  int64_t nb = (n + 1023) / 1024;
  if (nb < 1) nb = 1;
  if (nb <= 4096) {
    k_scan_reduce<<<(int)nb, 256, 0, s>>>(in, n, tmp);
    k_scan_bsums<<<1, 1024, 0, s>>>(tmp, (int)nb);
    k_scan_apply<<<(int)nb, 256, 0, s>>>(in, out, n, tmp, (int)nb);
    DM_LAUNCH_CHECK();
    return DM_OK;
  }
  // two levels: the block sums are scanned like the input
  const int64_t nb2 = (nb + 1023) / 1024;
  if (nb2 > 4096) {
    set_error("exclusive_scan_i32: n=%lld exceeds 2^32", (long long)n);
    return DM_ERR_CAPACITY;
  }
  int32_t *b1 = tmp, *b1x = tmp + nb + 1, *b2 = b1x + nb + 1;
  k_scan_reduce<<<(int)nb, 256, 0, s>>>(in, n, b1);
  k_scan_reduce<<<(int)nb2, 256, 0, s>>>(b1, nb, b2);
  k_scan_bsums<<<1, 1024, 0, s>>>(b2, (int)nb2);
  k_scan_apply<<<(int)nb2, 256, 0, s>>>(b1, b1x, nb, b2, (int)nb2);
  k_scan_apply<<<(int)nb, 256, 0, s>>>(in, out, n, b1x, (int)nb);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

}  // namespace dm
