// Fourier-feature MLP signed distance: training (FP32, SIMT) and inference
// on the 5th-generation tensor cores (BF16 operands, FP32 accumulation in
// tensor memory).
//
//   x_n  = (x - center) * inv_scale
//   f    = [sin(2 pi F x_n), cos(2 pi F x_n)]             64 features
//   h_l  = relu(W_l h_{l-1} + b_l), l = 1..4              width 128
//   d    = out_scale * (w5 . h_4 + b5)
//
// Parameter layout (FP32, DM_MLP_NPARAMS floats):
//   W1[128][64] b1[128] W2[128][128] b2 W3 b3 W4 b4 w5[128] b5
// and BF16 copies of W1..W4 back to back for the inference kernel.
#include <cuda.h>
#include <cuda_bf16.h>

#include <cstring>
#include <mutex>

#include "dm_common.cuh"

namespace dm {

void note_launches(int k);

constexpr int kW = 128, kF = 64, kNF = 32;
// offsets of layer l (0..3) in the FP32 parameters and the BF16 copies
__host__ __device__ constexpr int kK(int l) { return l == 0 ? 64 : 128; }
__host__ __device__ constexpr int64_t kOffW(int l) { return l == 0 ? 0 : 8320 + (l - 1) * 16512; }
__host__ __device__ constexpr int64_t kOffB(int l) { return kOffW(l) + 128 * kK(l); }
__host__ __device__ constexpr int64_t kOffWb(int l) { return l == 0 ? 0 : 8192 + (l - 1) * 16384; }
constexpr int64_t kOffW5 = 57856, kOffB5 = 57984;
static_assert(kOffB(3) + 128 == kOffW5, "parameter layout");
static_assert(kOffB5 + 1 == DM_MLP_NPARAMS, "parameter layout");
static_assert(kOffWb(3) + 16384 == DM_MLP_NBF16, "bf16 layout");

struct MlpDev {
  float freq[kNF * 3];
  float center[3];
  float inv_scale;
  float out_scale;
  const float *params;
};

static MlpDev to_dev(const dm_mlp *m) {
  MlpDev d;
  std::memset(&d, 0, sizeof(d));
  std::memcpy(d.freq, m->freq, sizeof(d.freq));
  for (int i = 0; i < 3; ++i) d.center[i] = m->center[i];
  d.inv_scale = m->inv_scale;
  d.out_scale = m->out_scale;
  d.params = m->params;
  return d;
}

// feature k (< 32) of the point: sin and cos of 2 pi (F_k . x_n), with the
// argument reduced to one period first.  Shared by training and inference.
__device__ __forceinline__ void fourier(const MlpDev &m, const float *x, int k, float *s,
                                        float *c) {
  const float x0 = (x[0] - m.center[0]) * m.inv_scale;
  const float x1 = (x[1] - m.center[1]) * m.inv_scale;
  const float x2 = (x[2] - m.center[2]) * m.inv_scale;
  float t = __fmul_rn(m.freq[3 * k], x0);
  t = __fadd_rn(t, __fmul_rn(m.freq[3 * k + 1], x1));
  t = __fadd_rn(t, __fmul_rn(m.freq[3 * k + 2], x2));
  t = t - rintf(t);
  sincospif(2.f * t, s, c);
}

// ---------------------------------------------------------------------------
// training: FP32 kernels

__global__ void k_features(MlpDev m, const float *x, int stride, int64_t n, float *feat) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n * kNF;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / kNF;
    const int k = (int)(i % kNF);
    float s, c;
    fourier(m, x + r * stride, k, &s, &c);
    feat[r * kF + k] = s;
    feat[r * kF + kNF + k] = c;
  }
}

enum { EPI_PLAIN = 0, EPI_BIAS_RELU = 1, EPI_RELU_GRAD = 2 };

// C[m][n] = sum_k A(m, k) B(k, n) over k in this split's chunk, with
// A(m, k) = A[m*lam + k*lak], B(k, n) = B[k*lbk + n*lbn]; 64x64 tiles,
// 16-deep k steps, 4x4 outputs per thread.  Split z writes C + z*M*ldc.
template <int EPI>
__global__ void __launch_bounds__(256)
    k_gemm(int M, int N, int K, int kchunk, const float *__restrict__ A, int64_t lam,
           int64_t lak, const float *__restrict__ B, int64_t lbk, int64_t lbn, float *C,
           int64_t ldc, const float *bias, float *H, const float *Zprev) {
  __shared__ __align__(16) float As[16][68];
  __shared__ __align__(16) float Bs[16][68];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
  const int kb = blockIdx.z * kchunk, ke = min(K, kb + kchunk);
  const bool a_kfast = lak == 1, b_nfast = lbn == 1;
  float acc[4][4] = {};
  for (int k0 = kb; k0 < ke; k0 += 16) {
    for (int e = threadIdx.x; e < 1024; e += 256) {
      int mm = a_kfast ? e >> 4 : e & 63, kk = a_kfast ? e & 15 : e >> 6;
      int gm = m0 + mm, gk = k0 + kk;
      As[kk][mm] = (gm < M && gk < ke) ? A[gm * lam + gk * lak] : 0.f;
      int nn = b_nfast ? e & 63 : e >> 4, kq = b_nfast ? e >> 6 : e & 15;
      int gn = n0 + nn, gq = k0 + kq;
      Bs[kq][nn] = (gn < N && gq < ke) ? B[gq * lbk + gn * lbn] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      float4 a = *reinterpret_cast<const float4 *>(&As[kk][ty * 4]);
      float4 b = *reinterpret_cast<const float4 *>(&Bs[kk][tx * 4]);
      float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
    }
    __syncthreads();
  }
  float *Cz = C + (int64_t)blockIdx.z * M * ldc;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + ty * 4 + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gn = n0 + tx * 4 + j;
      if (gn >= N) continue;
      float v = acc[i][j];
      if (EPI == EPI_BIAS_RELU) {
        v += bias[gn];
        H[gm * ldc + gn] = fmaxf(v, 0.f);
      } else if (EPI == EPI_RELU_GRAD) {
        v = Zprev[gm * ldc + gn] > 0.f ? v : 0.f;
      }
      Cz[gm * ldc + gn] = v;
    }
  }
}

// out[i] = sum over s of part[s][i] (fixed order: deterministic)
__global__ void k_sum_parts(const float *part, int nsplit, int64_t len, float *out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int z = 0; z < nsplit; ++z) s += part[z * len + i];
    out[i] = s;
  }
}

// part[s][c] = sum over rows of split s of X[r][c] (times w[r] if given)
__global__ void k_colsum(const float *X, const float *w, int64_t rows, int cols, int64_t chunk,
                         float *part) {
  const int c = threadIdx.x;
  if (c >= cols) return;
  const int64_t r0 = blockIdx.x * chunk, r1 = min(rows, r0 + chunk);
  float s = 0.f;
  for (int64_t r = r0; r < r1; ++r) s += w ? w[r] * X[r * cols + c] : X[r * cols + c];
  part[blockIdx.x * cols + c] = s;
}

// output layer and loss: y = w5 . h + b5; dy = 2 w (y - t) / B;
// per-block partial losses
__global__ void k_out_loss(const float *h, const float *params, const float *target,
                           const float *weight, int64_t B, float *y, float *dy, float *lpart) {
  __shared__ float red[8];
  float l = 0.f;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < B;
       r += (int64_t)gridDim.x * blockDim.x) {
    float s = params[kOffB5];
    for (int k = 0; k < kW; ++k) s = fmaf(params[kOffW5 + k], h[r * kW + k], s);
    y[r] = s;
    if (target) {
      const float w = weight ? weight[r] : 1.f, e = s - target[r];
      dy[r] = 2.f * w * e / (float)B;
      l += w * e * e / (float)B;
    }
  }
  for (int o = 16; o; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = l;
  __syncthreads();
  if (threadIdx.x == 0 && lpart) {
    float t = 0.f;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += red[i];
    lpart[blockIdx.x] = t;
  }
}

// dz4[r][k] = dy[r] w5[k] (z4[r][k] > 0)
__global__ void k_out_back(const float *dy, const float *params, const float *z, int64_t B,
                           float *dz) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < B * kW;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / kW;
    const int k = (int)(i % kW);
    dz[i] = z[i] > 0.f ? dy[r] * params[kOffW5 + k] : 0.f;
  }
}

__global__ void k_scale_out(const float *y, int64_t n, float scale, float *d) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    d[i] = scale * y[i];
}

__global__ void k_adam(float *p, const float *g, float *m1, float *m2, int64_t n, float lr,
                       float b1, float b2, float eps, float c1, float c2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float a = b1 * m1[i] + (1.f - b1) * gi;
    const float v = b2 * m2[i] + (1.f - b2) * gi * gi;
    m1[i] = a;
    m2[i] = v;
    p[i] -= lr * (a / c1) / (sqrtf(v / c2) + eps);
  }
}

__global__ void k_to_bf16(const float *p, uint16_t *w) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < DM_MLP_NBF16;
       i += (int64_t)gridDim.x * blockDim.x) {
    int l = i < 8192 ? 0 : 1 + (int)((i - 8192) / 16384);
    int64_t j = i - kOffWb(l);
    __nv_bfloat16 b = __float2bfloat16_rn(p[kOffW(l) + j]);
    w[i] = *reinterpret_cast<uint16_t *>(&b);
  }
}

struct TrainWs {
  float *feat, *z[4], *h[4], *y, *dy, *dza, *dzb, *part, *lpart;
};
constexpr int kSplit = 64;
constexpr int kLossBlocks = 256;

static size_t carve_train(Carve &c, int64_t B, TrainWs *w) {
  w->feat = c.take<float>(B * kF);
  for (int l = 0; l < 4; ++l) w->z[l] = c.take<float>(B * kW);
  for (int l = 0; l < 4; ++l) w->h[l] = c.take<float>(B * kW);
  w->y = c.take<float>(B);
  w->dy = c.take<float>(B);
  w->dza = c.take<float>(B * kW);
  w->dzb = c.take<float>(B * kW);
  w->part = c.take<float>((int64_t)kSplit * kW * kW);
  w->lpart = c.take<float>(kLossBlocks);
  return c.used;
}

size_t mlp_train_workspace(int64_t batch) {
  Carve c(nullptr, 0);
  TrainWs w;
  return carve_train(c, batch, &w) + 256;
}

template <int EPI>
static void gemm(cudaStream_t s, int M, int N, int K, int nsplit, const float *A, int64_t lam,
                 int64_t lak, const float *B, int64_t lbk, int64_t lbn, float *C, int64_t ldc,
                 const float *bias = nullptr, float *H = nullptr, const float *Z = nullptr) {
  int kchunk = (K + nsplit - 1) / nsplit;
  kchunk = (kchunk + 15) / 16 * 16;
  dim3 grid((N + 63) / 64, (M + 63) / 64, nsplit);
  k_gemm<EPI><<<grid, 256, 0, s>>>(M, N, K, kchunk, A, lam, lak, B, lbk, lbn, C, ldc, bias, H, Z);
}

// forward of B points into ws (features, z, h, y)
static void forward(const MlpDev &m, const float *x, int stride, int64_t B, TrainWs &w,
                    cudaStream_t s) {
  k_features<<<grid_for(B * kNF, 256), 256, 0, s>>>(m, x, stride, B, w.feat);
  const float *a = w.feat;
  for (int l = 0; l < 4; ++l) {
    gemm<EPI_BIAS_RELU>(s, (int)B, kW, kK(l), 1, a, kK(l), 1, m.params + kOffW(l), 1, kK(l),
                        w.z[l], kW, m.params + kOffB(l), w.h[l]);
    a = w.h[l];
  }
}

int mlp_forward_backward(const dm_mlp *mp, const float *x, const float *target,
                         const float *weight, int64_t B, float *grads, float *loss, void *ws,
                         size_t ws_bytes, cudaStream_t s) {
  DM_ARG_CHECK(mp && mp->params && x && target && grads && B > 0, "mlp training");
  Carve c(ws, ws_bytes);
  TrainWs w;
  carve_train(c, B, &w);
  if (!c.ok() || !ws) {
    set_error("mlp_forward_backward: workspace %zu < required %zu", ws_bytes, c.used);
    return DM_ERR_WORKSPACE;
  }
  const MlpDev m = to_dev(mp);
  forward(m, x, 4, B, w, s);
  k_out_loss<<<kLossBlocks, 256, 0, s>>>(w.h[3], m.params, target, weight, B, w.y, w.dy, w.lpart);
  if (loss) k_sum_parts<<<1, 32, 0, s>>>(w.lpart, kLossBlocks, 1, loss);
  // output layer: w5, b5 and dz of layer 4
  const int64_t chunk = (B + kSplit - 1) / kSplit;
  k_colsum<<<kSplit, kW, 0, s>>>(w.h[3], w.dy, B, kW, chunk, w.part);
  k_sum_parts<<<1, kW, 0, s>>>(w.part, kSplit, kW, grads + kOffW5);
  k_colsum<<<kSplit, 1, 0, s>>>(w.dy, nullptr, B, 1, chunk, w.part);
  k_sum_parts<<<1, 32, 0, s>>>(w.part, kSplit, 1, grads + kOffB5);
  k_out_back<<<grid_for(B * kW, 256), 256, 0, s>>>(w.dy, m.params, w.z[3], B, w.dza);
  float *dz = w.dza, *dzn = w.dzb;
  for (int l = 3; l >= 0; --l) {
    const float *a = l ? w.h[l - 1] : w.feat;
    const int K = kK(l);
    // dW_l[n][k] = sum_r dz[r][n] a[r][k]: split over the batch
    gemm<EPI_PLAIN>(s, kW, K, (int)B, kSplit, dz, 1, kW, a, K, 1, w.part, K);
    k_sum_parts<<<grid_for(kW * K, 256), 256, 0, s>>>(w.part, kSplit, (int64_t)kW * K,
                                                        grads + kOffW(l));
    k_colsum<<<kSplit, kW, 0, s>>>(dz, nullptr, B, kW, chunk, w.part);
    k_sum_parts<<<1, kW, 0, s>>>(w.part, kSplit, kW, grads + kOffB(l));
    if (l) {
      // dz_{l-1} = (dz_l W_l) * (z_{l-1} > 0)
      gemm<EPI_RELU_GRAD>(s, (int)B, kW, kW, 1, dz, kW, 1, m.params + kOffW(l), K, 1, dzn, kW,
                          nullptr, nullptr, w.z[l - 1]);
      float *t = dz;
      dz = dzn;
      dzn = t;
    }
  }
  note_launches(30);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

int mlp_adam(float *p, const float *g, float *m1, float *m2, int64_t n, float lr, float b1,
             float b2, float eps, int t, cudaStream_t s) {
  DM_ARG_CHECK(p && g && m1 && m2 && n > 0 && t >= 1, "adam");
  const float c1 = 1.f - powf(b1, (float)t), c2 = 1.f - powf(b2, (float)t);
  k_adam<<<grid_for(n, 256), 256, 0, s>>>(p, g, m1, m2, n, lr, b1, b2, eps, c1, c2);
  note_launches(1);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

int mlp_to_bf16(const float *params, uint16_t *w, cudaStream_t s) {
  DM_ARG_CHECK(params && w, "pointers");
  k_to_bf16<<<grid_for(DM_MLP_NBF16, 256), 256, 0, s>>>(params, w);
  note_launches(1);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

int mlp_eval_fp32(const dm_mlp *mp, const float *pts, int stride, int64_t n, float *d, void *ws,
                  size_t ws_bytes, cudaStream_t s) {
  DM_ARG_CHECK(mp && mp->params && pts && d && n >= 0 && stride >= 3, "mlp eval");
  const int64_t B = 16384;
  Carve c(ws, ws_bytes);
  TrainWs w;
  carve_train(c, B, &w);
  if (!c.ok() || !ws) {
    set_error("mlp_eval_fp32: workspace %zu < required %zu (dm_mlp_train_workspace_size(16384))",
              ws_bytes, c.used);
    return DM_ERR_WORKSPACE;
  }
  const MlpDev m = to_dev(mp);
  for (int64_t r0 = 0; r0 < n; r0 += B) {
    const int64_t b = n - r0 < B ? n - r0 : B;
    forward(m, pts + r0 * stride, stride, b, w, s);
    k_out_loss<<<kLossBlocks, 256, 0, s>>>(w.h[3], m.params, nullptr, nullptr, b, w.y, nullptr,
                                           nullptr);
    k_scale_out<<<grid_for(b, 256), 256, 0, s>>>(w.y, b, m.out_scale, d + r0);
  }
  note_launches(7);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

// ---------------------------------------------------------------------------
// inference: tcgen05 (cta_group::1, kind::f16), M = N = 128, K = 16 per MMA.
//
// One persistent CTA per SM with two warpgroups.  Each warpgroup owns a
// tile of 128 points at a time, its activation tiles and a 128-column FP32
// accumulator in tensor memory, and runs features -> 4 x (MMAs, epilogue)
// on its own; the tensor core executes one group's MMAs while the other
// group is in its epilogue.
//
// Shared memory (1024-aligned), all operand tiles K-major with the 128-byte
// swizzle: a tile is 128 rows x 64 BF16 (128 B per row, 8-row groups of
// 1024 B, 16-byte chunk j of row r stored at chunk j ^ (r & 7)), which is
// what a TMA load with CU_TENSOR_MAP_SWIZZLE_128B writes.
//   W1: 1 tile; W2..W4: 2 tiles each (K = 0..63, 64..127); per group, A: 2
//   tiles (activations of the current layer; layer 1 uses the first).
// Tensor memory: 256 columns; group g's accumulator is columns 128 g..,
// lane r = row r (point r of its tile), column j = output feature j.  Warp w
// of a group reads lanes 32 (w mod 4)...
constexpr int kTile = 128;
constexpr int kTileBytes = 128 * 128;  // 128 rows x 128 B
constexpr uint32_t kIdesc = (1u << 4)            // D: FP32
                            | (1u << 7)          // A: BF16
                            | (1u << 10)         // B: BF16
                            | ((128u >> 3) << 17)  // N
                            | ((128u >> 4) << 24);  // M
constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s per wait

// set when a wait of the tensor-core kernel gave up (read by
// dm_mlp_eval_status)
static __device__ int g_mlp_err;

struct TcSmem {
  uint8_t w1[kTileBytes];
  uint8_t w[3][2][kTileBytes];
  uint8_t a[2][2][kTileBytes];  // [group][K half]
  float bias[4][kW];
  float w5[kW];
  float b5;
  int err;
  uint32_t tmem;
  uint64_t bar_w;
  uint64_t bar_mma[2];
};
constexpr size_t kTcSmemBytes = sizeof(TcSmem) + 1024;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4)      // start address
         | ((uint64_t)1 << 16)                   // leading byte offset (unused: swizzled K-major)
         | ((uint64_t)(1024 >> 4) << 32)         // stride byte offset: 8 rows x 128 B
         | ((uint64_t)1 << 46)                   // descriptor version
         | ((uint64_t)2 << 61);                  // 128-byte swizzle
}

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// bounded wait on an mbarrier phase: false after kWaitNs
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  const unsigned long long t0 = now_ns();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if (now_ns() - t0 > kWaitNs) return false;
  }
}

// barrier of one warpgroup (named barrier 1 + g, 128 threads) that also
// returns whether v holds for all of its threads
__device__ __forceinline__ bool group_and(bool v, int g) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.and.pred q, %2, 128, p;\n"
      " selp.u32 %0, 1, 0, q;\n}\n"
      : "=r"(r)
      : "r"((uint32_t)v), "r"(1 + g)
      : "memory");
  return r != 0;
}
__device__ __forceinline__ void group_sync(int g) {
  asm volatile("bar.sync %0, 128;\n" ::"r"(1 + g) : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);  // .x = a (low half)
  return *reinterpret_cast<uint32_t *>(&h);
}

// 8 BF16 values (16 bytes) into chunk j (0..15 over K = 0..127) of row r of
// group g's activation tiles
__device__ __forceinline__ void st_chunk(TcSmem &S, int g, int r, int j, const float *v8) {
  const int tile = j >> 3, cj = j & 7;
  uint8_t *p = S.a[g][tile] + r * 128 + ((cj ^ (r & 7)) << 4);
  uint4 q = make_uint4(pack_bf16(v8[0], v8[1]), pack_bf16(v8[2], v8[3]),
                       pack_bf16(v8[4], v8[5]), pack_bf16(v8[6], v8[7]));
  *reinterpret_cast<uint4 *>(p) = q;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int c0, int c1,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, "
      "{%2, %3}], [%4];\n" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
      : "memory");
}

__global__ void __launch_bounds__(256, 1)
    k_mlp_infer_tc(const __grid_constant__ CUtensorMap tw1, const __grid_constant__ CUtensorMap tw2,
                   const __grid_constant__ CUtensorMap tw3, const __grid_constant__ CUtensorMap tw4,
                   MlpDev m, const float *__restrict__ pts, int stride, int64_t n,
                   float *__restrict__ dout) {
  extern __shared__ uint8_t smem_raw[];
  TcSmem &S = *reinterpret_cast<TcSmem *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int tid = threadIdx.x, warp = tid >> 5;
  const int g = warp >> 2, r = tid & 127;  // warpgroup, row of its tile
  const int64_t ntiles = (n + kTile - 1) / kTile;

  if (tid == 0) {
    S.err = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&S.bar_w)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&S.bar_mma[0])));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&S.bar_mma[1])));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {  // tensor memory: 2 x 128 columns
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;\n" ::"r"(
        smem_u32(&S.tmem)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  for (int i = tid; i < 4 * kW; i += blockDim.x)
    S.bias[i / kW][i % kW] = m.params[kOffB(i / kW) + i % kW];
  for (int i = tid; i < kW; i += blockDim.x) S.w5[i] = m.params[kOffW5 + i];
  if (tid == 0) S.b5 = m.params[kOffB5];
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = S.tmem + (uint32_t)(g * 128);  // this group's accumulator

  if (tid == 0) {  // the weights, once per CTA (7 TMA tiles of 16 KB)
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(
                     smem_u32(&S.bar_w)),
                 "r"(7 * kTileBytes)
                 : "memory");
    tma_load_2d(S.w1, &tw1, 0, 0, &S.bar_w);
    const CUtensorMap *maps[3] = {&tw2, &tw3, &tw4};
    for (int l = 0; l < 3; ++l) {
      tma_load_2d(S.w[l][0], maps[l], 0, 0, &S.bar_w);
      tma_load_2d(S.w[l][1], maps[l], 64, 0, &S.bar_w);
    }
  }
  bool ok = __syncthreads_and(mbar_wait(&S.bar_w, 0));
  uint32_t phase = 0;
  bool mma_pending = false;

  // every decision that ends a loop is taken by the whole warpgroup
  for (int64_t tile = 2 * (int64_t)blockIdx.x + g; ok && tile < ntiles;
       tile += 2 * (int64_t)gridDim.x) {
    // layer-1 input: Fourier features of point r of the tile
    const int64_t row = tile * kTile + r;
    float xp[3] = {0.f, 0.f, 0.f};
    if (row < n) {
      const float *x = pts + row * stride;
      xp[0] = x[0];
      xp[1] = x[1];
      xp[2] = x[2];
    }
    for (int j = 0; j < 4; ++j) {  // chunks 0..3: sin, 4..7: cos
      float sv[8], cv[8];
      for (int q = 0; q < 8; ++q) fourier(m, xp, 8 * j + q, &sv[q], &cv[q]);
      st_chunk(S, g, r, j, sv);
      st_chunk(S, g, r, 4 + j, cv);
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    group_sync(g);

    for (int l = 0; l < 4 && ok; ++l) {
      if (r == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const int nk = kK(l) / 16;
        for (int k = 0; k < nk; ++k) {
          const int t = k >> 2, off = (k & 3) * 32;
          const uint8_t *btile = l == 0 ? S.w1 : S.w[l - 1][t];
          mma_bf16(tmem, sw128_desc(smem_u32(S.a[g][t]) + off),
                   sw128_desc(smem_u32(btile) + off), k > 0);
        }
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                smem_u32(&S.bar_mma[g]))
            : "memory");
      }
      mma_pending = true;
      ok = group_and(mbar_wait(&S.bar_mma[g], phase), g);
      if (!ok) break;
      mma_pending = false;
      phase ^= 1;
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const uint32_t taddr = tmem + ((uint32_t)((warp & 3) * 32) << 16);
      if (l < 3) {
        for (int c0 = 0; c0 < kW; c0 += 32) {
          float v[32];
          tmem_ld32(taddr + c0, v);
          for (int i = 0; i < 32; ++i) v[i] = fmaxf(v[i] + S.bias[l][c0 + i], 0.f);
          for (int j = 0; j < 4; ++j) st_chunk(S, g, r, (c0 >> 3) + j, v + 8 * j);
        }
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        group_sync(g);
      } else {
        float acc = S.b5;
        for (int c0 = 0; c0 < kW; c0 += 32) {
          float v[32];
          tmem_ld32(taddr + c0, v);
          for (int i = 0; i < 32; ++i)
            acc = fmaf(S.w5[c0 + i], fmaxf(v[i] + S.bias[3][c0 + i], 0.f), acc);
        }
        if (row < n) dout[row] = m.out_scale * acc;
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        group_sync(g);
      }
    }
  }
  if (!ok) {
    if (r == 0) atomicExch(&g_mlp_err, 1);
    if (mma_pending) mbar_wait(&S.bar_mma[g], phase);  // bounded: let an issued MMA drain
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;\n" ::"r"(S.tmem));
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
  static std::once_flag once;
  static EncodeTiledFn fn = nullptr;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

// [128 rows][K] BF16 row-major weights, boxes of 64 (K) x 128 rows
static int weight_map(CUtensorMap *map, const uint16_t *w, int K) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) {
    set_error("mlp_eval: cuTensorMapEncodeTiled is not available from the driver");
    return DM_ERR_CUDA;
  }
  cuuint64_t dims[2] = {(cuuint64_t)K, 128};
  cuuint64_t strides[1] = {(cuuint64_t)K * 2};
  cuuint32_t box[2] = {64, 128};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<uint16_t *>(w), dims,
                  strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("mlp_eval: cuTensorMapEncodeTiled failed (%d)", (int)r);
    return DM_ERR_CUDA;
  }
  return DM_OK;
}

static std::mutex g_tc_mu;
static bool g_tc_attr[64];

int mlp_eval_tc(const dm_mlp *mp, const float *pts, int stride, int64_t n, float *d,
                cudaStream_t s) {
  DM_ARG_CHECK(mp && mp->params && mp->wbf16 && pts && d && n >= 0 && stride >= 3,
               "mlp eval");
  DM_ARG_CHECK((reinterpret_cast<uintptr_t>(mp->wbf16) & 15) == 0, "wbf16 16-byte aligned");
  if (n == 0) return DM_OK;
  CUtensorMap maps[4];
  for (int l = 0; l < 4; ++l) {
    int rc = weight_map(&maps[l], mp->wbf16 + kOffWb(l), kK(l));
    if (rc) return rc;
  }
  int dev = 0;
  DM_CUDA_TRY(cudaGetDevice(&dev));
  DM_ARG_CHECK(dev >= 0 && dev < 64, "device ordinal");
  {
    std::lock_guard<std::mutex> lock(g_tc_mu);
    if (!g_tc_attr[dev]) {
      DM_CUDA_TRY(cudaFuncSetAttribute(k_mlp_infer_tc,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kTcSmemBytes));
      g_tc_attr[dev] = true;
    }
  }
  const MlpDev m = to_dev(mp);
  int sms = 0;
  DM_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int64_t npairs = (n + 2 * kTile - 1) / (2 * kTile);
  const int grid = (int)(npairs < sms ? npairs : sms);
  k_mlp_infer_tc<<<grid, 256, kTcSmemBytes, s>>>(maps[0], maps[1], maps[2], maps[3], m, pts,
                                                 stride, n, d);
  note_launches(1);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

// whether a wait of the tensor-core kernel gave up since the last call
// (synchronises the stream; clears the flag)
int mlp_tc_status(cudaStream_t s, int *status) {
  DM_ARG_CHECK(status, "status");
  DM_CUDA_TRY(cudaMemcpyFromSymbolAsync(status, g_mlp_err, sizeof(int), 0,
                                        cudaMemcpyDeviceToHost, s));
  DM_CUDA_TRY(cudaStreamSynchronize(s));
  const int zero = 0;
  DM_CUDA_TRY(cudaMemcpyToSymbolAsync(g_mlp_err, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, s));
  DM_CUDA_TRY(cudaStreamSynchronize(s));
  return DM_OK;
}

}  // namespace dm
