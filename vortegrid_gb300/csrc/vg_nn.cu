// Learned warm start for the vector-potential solve (no counterpart in the
// reference; the solve it warms is VortonSim::SolveVelocityFromVorticityUsingPoisson,
// VortonFluid/vortonSim.cpp:2480-2560).
//
// A 3D U-Net on the grid's (n+1)^3 points minus the last plane per axis
// (n^3 voxels, n a multiple of 8):
//
//   level  edge  channels  encoder                      decoder
//   0      n     16        enc0a, enc0b                 dec0a(up dec1b ++ enc0b), dec0b, out
//   1      n/2   32        pool, enc1a, enc1b           dec1a(up dec2b ++ enc1b), dec1b
//   2      n/4   64        pool, enc2a, enc2b           dec2a(up enc3b ++ enc2b), dec2b
//   3      n/8   128       pool, enc3a, enc3b
//
// Every convolution is 3x3x3 with zero padding, bias and a leaky ReLU (slope
// 0.1 below zero; none on the output); pooling is a 2x2x2 average and upsampling is nearest-neighbour.
// Input channels: the right-hand side (minus the vorticity) / s and the
// Dirichlet boundary values / (s h^2 K) (at the low faces, and at the voxels
// next to the high faces, the value of their outer neighbour), where s is the
// RMS of the right-hand side and K the network's output scale.  Output
// channels 0..2, times s h^2 K, replace the interior of the initial vector
// potential; multigrid then finishes the solve to its tolerance.
//
// Weights and activations are BF16, accumulation FP32; the master parameters,
// gradients and Adam moments are FP32.  Training runs forward, backward and the
// optimiser step entirely in this library's kernels.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <vector>

#include "vg_nn.cuh"

namespace vg {
namespace nn {

namespace {

constexpr int kLayers = 15;
constexpr int kRedBlocks = 304;  // partial sums of the norm reductions (a fixed width)
constexpr float kSlope = 0.1f;  // leaky ReLU: v > 0 ? v : kSlope v

struct LayerDesc {
  int level, ci, co, cup, relu;
};
// cup = channels of the first input read through 2x upsampling (decoder layers)
constexpr LayerDesc kNet[kLayers] = {
    {0, 16, 16, 0, 1},     {0, 16, 16, 0, 1},   {1, 16, 32, 0, 1},   {1, 32, 32, 0, 1},   {2, 32, 64, 0, 1},
    {2, 64, 64, 0, 1},     {3, 64, 128, 0, 1},  {3, 128, 128, 0, 1}, {2, 192, 64, 128, 1}, {2, 64, 64, 0, 1},
    {1, 96, 32, 64, 1},    {1, 32, 32, 0, 1},   {0, 48, 16, 32, 1},  {0, 16, 16, 0, 1},   {0, 16, 16, 0, 0},
};

// Activations (outputs of the layers, the pooled tensors and the network input).
enum Act {
  A_X, A_E0A, A_E0B, A_P1, A_E1A, A_E1B, A_P2, A_E2A, A_E2B, A_P3, A_E3A, A_E3B,
  A_D2A, A_D2B, A_D1A, A_D1B, A_D0A, A_D0B, A_NUM
};
constexpr int kActLevel[A_NUM] = {0, 0, 0, 1, 1, 1, 2, 2, 2, 3, 3, 3, 2, 2, 1, 1, 0, 0};
constexpr int kActC[A_NUM] = {16, 16, 16, 16, 32, 32, 32, 64, 64, 64, 128, 128, 64, 64, 32, 32, 16, 16};
constexpr int kIn1[kLayers] = {A_X,   A_E0A, A_P1,  A_E1A, A_P2,  A_E2A, A_P3, A_E3A,
                               A_E3B, A_D2A, A_D2B, A_D1A, A_D1B, A_D0A, A_D0B};
constexpr int kIn2[kLayers] = {-1, -1, -1, -1, -1, -1, -1, -1, A_E2B, -1, A_E1B, -1, A_E0B, -1, -1};
constexpr int kOut[kLayers] = {A_E0A, A_E0B, A_E1A, A_E1B, A_E2A, A_E2B, A_E3A, A_E3B,
                               A_D2A, A_D2B, A_D1A, A_D1B, A_D0A, A_D0B, -1};

}  // namespace

struct Net {
  Ctx ctx;  // stream and error state of calls made on the network itself
  int n = 0;
  float out_scale = 1.f;
  size_t nparam = 0, nw = 0;
  size_t wofs[kLayers], bofs[kLayers], wbofs[kLayers];
  float* master = nullptr;  // FP32 parameters: per layer W[27][Co][Ci] then b[Co]
  float* grad = nullptr;
  float* m1 = nullptr;
  float* m2 = nullptr;
  __nv_bfloat16* w = nullptr;   // BF16 W per layer
  __nv_bfloat16* wt = nullptr;  // BF16 W'[26 - tap][Ci][Co] (input gradients)
  long step = 0;
  bool have_params = false;
  __nv_bfloat16* act[A_NUM] = {};
  float* out = nullptr;          // [n^3][16] FP32
  __nv_bfloat16* g[kLayers] = {};    // gradients w.r.t. each layer's pre-activation output
  __nv_bfloat16* gin[kLayers] = {};  // gradients w.r.t. the inputs of layers 2, 4, 6, 8, 10, 12
  float* scales = nullptr;       // [0] 1/s, [1] 1/(s h^2 K), [2] s h^2 K
  double* partials = nullptr;    // kRedBlocks
  float* loss = nullptr;         // [0] loss, [1] target energy, [2] loss-gradient scale
  int dims(int level) const { return n >> level; }
  size_t vox(int level) const {
    const size_t e = (size_t)dims(level);
    return e * e * e;
  }
};

namespace {

__device__ __forceinline__ float bf(const __nv_bfloat16 v) { return __bfloat162float(v); }

__device__ __forceinline__ void block_sum_to(double v, double* dst) {
  __shared__ double sh[32];
  for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) *dst = v;
  }
}

__device__ __forceinline__ float ld(const float* p, size_t i) { return p[i]; }
__device__ __forceinline__ float ld(const __nv_bfloat16* p, size_t i) { return __bfloat162float(p[i]); }

// Sum of squares of count values, one fixed partial per block (deterministic).
template <typename T>
__global__ void k_sumsq(const T* __restrict__ a, size_t count, double* __restrict__ partials) {
  double s = 0.0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
    const float v = ld(a, i);
    s += (double)v * v;
  }
  block_sum_to(s, partials + blockIdx.x);
}

__global__ void k_scales(const double* __restrict__ partials, int nb, double count, float h2k, float* scales) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int i = 0; i < nb; ++i) s += partials[i];
  double rms = sqrt(s / count);
  if (!(rms > 0.0) || !isfinite(rms)) rms = 1.0;
  scales[0] = (float)(1.0 / rms);
  scales[1] = (float)(1.0 / (rms * h2k));
  scales[2] = (float)(rms * h2k);
}

// Network input for voxel (i, j, k) of n^3 from the (n+1)^3 point grids.
template <typename T>
__global__ void k_pack_input(const T* __restrict__ rhs, const T* __restrict__ vp, int n, const float* __restrict__ scales,
                             __nv_bfloat16* __restrict__ x) {
  const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t nv = (size_t)n * n * n;
  if (v >= nv) return;
  const int i = (int)(v % n), j = (int)((v / n) % n), k = (int)(v / ((size_t)n * n));
  const int np = n + 1;
  const size_t p = ((size_t)k * np + j) * np + i;
  const float s_in = scales[0], s_bc = scales[1];
  float c[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) c[q] = 0.f;
  c[0] = ld(rhs, 3 * p) * s_in;
  c[1] = ld(rhs, 3 * p + 1) * s_in;
  c[2] = ld(rhs, 3 * p + 2) * s_in;
  size_t pb = (size_t)-1;
  if (i == 0 || j == 0 || k == 0) {
    pb = p;
  } else if (i == n - 1 || j == n - 1 || k == n - 1) {
    const int bi = i == n - 1 ? n : i, bj = j == n - 1 ? n : j, bk = k == n - 1 ? n : k;
    pb = ((size_t)bk * np + bj) * np + bi;
  }
  if (pb != (size_t)-1) {
    c[3] = ld(vp, 3 * pb) * s_bc;
    c[4] = ld(vp, 3 * pb + 1) * s_bc;
    c[5] = ld(vp, 3 * pb + 2) * s_bc;
  }
  __align__(16) __nv_bfloat162 h[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) h[q] = __floats2bfloat162_rn(c[2 * q], c[2 * q + 1]);
  uint4* dst = reinterpret_cast<uint4*>(x + v * 16);
  dst[0] = *reinterpret_cast<const uint4*>(&h[0]);
  dst[1] = *reinterpret_cast<const uint4*>(&h[4]);
}

// Interior points (all indices in 1..n-1) of the vector potential from the network output.
__global__ void k_unpack_output(const float* __restrict__ out, int n, const float* __restrict__ scales,
                                float* __restrict__ vp) {
  const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= (size_t)n * n * n) return;
  const int i = (int)(v % n), j = (int)((v / n) % n), k = (int)(v / ((size_t)n * n));
  if (i == 0 || j == 0 || k == 0) return;
  const int np = n + 1;
  const size_t p = ((size_t)k * np + j) * np + i;
  const float s = scales[2];
  const float4 o = *reinterpret_cast<const float4*>(out + v * 16);
  vp[3 * p] = o.x * s;
  vp[3 * p + 1] = o.y * s;
  vp[3 * p + 2] = o.z * s;
}

// Target energy: sum over interior voxels (all indices >= 1) and channels 0..2
// of (target / (s h^2 K))^2, one fixed partial per block.
template <typename T>
__global__ void k_target_energy(const T* __restrict__ vp, int n, const float* __restrict__ scales,
                                double* __restrict__ partials) {
  double s = 0.0;
  const size_t nv = (size_t)n * n * n;
  const int np = n + 1;
  const float s_t = scales[1];
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(v % n), j = (int)((v / n) % n), k = (int)(v / ((size_t)n * n));
    if (i && j && k) {
      const size_t p = ((size_t)k * np + j) * np + i;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float t = ld(vp, 3 * p + c) * s_t;
        s += (double)t * t;
      }
    }
  }
  block_sum_to(s, partials + blockIdx.x);
}

// e[1] = target energy (1 if zero), e[2] = 2 / e[1] (the loss gradient's scale)
__global__ void k_finish_energy(const double* __restrict__ partials, int nb, float* e) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int i = 0; i < nb; ++i) s += partials[i];
  if (!(s > 0.0) || !isfinite(s)) s = 1.0;
  e[1] = (float)s;
  e[2] = (float)(2.0 / s);
}

// Loss = sum over interior voxels and channels 0..2 of (out - target / (s h^2 K))^2,
// divided by the target energy e[1] (a relative squared error per field); writes
// its gradient (BF16, 16 channels, zero outside channels 0..2 and at boundary voxels).
template <typename T>
__global__ void k_loss_grad(const float* __restrict__ out, const T* __restrict__ vp, int n,
                            const float* __restrict__ scales, const float* __restrict__ e,
                            __nv_bfloat16* __restrict__ g, double* __restrict__ partials) {
  double s = 0.0;
  const size_t nv = (size_t)n * n * n;
  const int np = n + 1;
  const float s_t = scales[1], gscale = e[2];
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(v % n), j = (int)((v / n) % n), k = (int)(v / ((size_t)n * n));
    float d[3] = {0.f, 0.f, 0.f};
    if (i && j && k) {
      const size_t p = ((size_t)k * np + j) * np + i;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        d[c] = out[v * 16 + c] - ld(vp, 3 * p + c) * s_t;
        s += (double)d[c] * d[c];
      }
    }
    __align__(16) __nv_bfloat162 h[8];
    h[0] = __floats2bfloat162_rn(d[0] * gscale, d[1] * gscale);
    h[1] = __floats2bfloat162_rn(d[2] * gscale, 0.f);
#pragma unroll
    for (int q = 2; q < 8; ++q) h[q] = __floats2bfloat162_rn(0.f, 0.f);
    uint4* dst = reinterpret_cast<uint4*>(g + v * 16);
    dst[0] = *reinterpret_cast<const uint4*>(&h[0]);
    dst[1] = *reinterpret_cast<const uint4*>(&h[4]);
  }
  block_sum_to(s, partials + blockIdx.x);
}

// e[0] = loss = sum of squared differences / target energy
__global__ void k_finish_loss(const double* __restrict__ partials, int nb, float* e) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int i = 0; i < nb; ++i) s += partials[i];
  e[0] = (float)(s / (double)e[1]);
}

// 8 BF16 channels as floats.
__device__ __forceinline__ void load8(const __nv_bfloat16* p, float* f) {
  const uint4 u = *reinterpret_cast<const uint4*>(p);
  const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const float2 t = __bfloat1622float2(h[q]);
    f[2 * q] = t.x;
    f[2 * q + 1] = t.y;
  }
}
__device__ __forceinline__ void store8(__nv_bfloat16* p, const float* f) {
  __align__(16) __nv_bfloat162 h[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) h[q] = __floats2bfloat162_rn(f[2 * q], f[2 * q + 1]);
  *reinterpret_cast<uint4*>(p) = *reinterpret_cast<const uint4*>(h);
}

// 2x2x2 average pool: fine e^3 -> coarse (e/2)^3, C channels.
__global__ void k_pool(const __nv_bfloat16* __restrict__ in, int ec, int C, __nv_bfloat16* __restrict__ out) {
  const int c8 = C / 8;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t nvc = (size_t)ec * ec * ec;
  if (t >= nvc * c8) return;
  const int cc = (int)(t % c8) * 8;
  const size_t v = t / c8;
  const int i = (int)(v % ec), j = (int)((v / ec) % ec), k = (int)(v / ((size_t)ec * ec));
  const int ef = 2 * ec;
  float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int d = 0; d < 8; ++d) {
    const size_t f = (((size_t)(2 * k + (d >> 2)) * ef + 2 * j + ((d >> 1) & 1)) * ef + 2 * i + (d & 1)) * C + cc;
    float a[8];
    load8(in + f, a);
#pragma unroll
    for (int q = 0; q < 8; ++q) s[q] += a[q];
  }
#pragma unroll
  for (int q = 0; q < 8; ++q) s[q] *= 0.125f;
  store8(out + v * C + cc, s);
}

// Gradient of a decoder layer's upsampled input, back at the coarse level:
// g[v][c] = (y[v][c] > 0 ? 1 : kSlope) * sum over the 8 children of gin[child][c] (c < C1).
__global__ void k_up_grad(const __nv_bfloat16* __restrict__ gin, int ccat, const __nv_bfloat16* __restrict__ y, int ec,
                          int C1, __nv_bfloat16* __restrict__ g) {
  const int c8 = C1 / 8;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t nvc = (size_t)ec * ec * ec;
  if (t >= nvc * c8) return;
  const int cc = (int)(t % c8) * 8;
  const size_t v = t / c8;
  const int i = (int)(v % ec), j = (int)((v / ec) % ec), k = (int)(v / ((size_t)ec * ec));
  const int ef = 2 * ec;
  float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int d = 0; d < 8; ++d) {
    const size_t f = ((size_t)(2 * k + (d >> 2)) * ef + 2 * j + ((d >> 1) & 1)) * ef + 2 * i + (d & 1);
    float a[8];
    load8(gin + f * ccat + cc, a);
#pragma unroll
    for (int q = 0; q < 8; ++q) s[q] += a[q];
  }
  float m[8];
  load8(y + v * C1 + cc, m);
#pragma unroll
  for (int q = 0; q < 8; ++q)
    if (!(m[q] > 0.f)) s[q] *= kSlope;
  store8(g + v * C1 + cc, s);
}

// Gradient of an encoder output that feeds both a skip connection and a pool:
// g[v][c] = (e[v][c] > 0 ? 1 : kSlope) * (gin_cat[v][C1 + c] + gp[parent(v)][c] / 8).
__global__ void k_skip_grad(const __nv_bfloat16* __restrict__ gcat, int ccat, int C1, const __nv_bfloat16* __restrict__ gp,
                            const __nv_bfloat16* __restrict__ e, int ef, int C, __nv_bfloat16* __restrict__ g) {
  const int c8 = C / 8;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t nv = (size_t)ef * ef * ef;
  if (t >= nv * c8) return;
  const int cc = (int)(t % c8) * 8;
  const size_t v = t / c8;
  const int i = (int)(v % ef), j = (int)((v / ef) % ef), k = (int)(v / ((size_t)ef * ef));
  const int ec = ef / 2;
  const size_t pv = ((size_t)(k >> 1) * ec + (j >> 1)) * ec + (i >> 1);
  float a[8], b[8], m[8];
  load8(gcat + v * ccat + C1 + cc, a);
  load8(gp + pv * C + cc, b);
  load8(e + v * C + cc, m);
#pragma unroll
  for (int q = 0; q < 8; ++q) a[q] = (m[q] > 0.f ? 1.f : kSlope) * (a[q] + 0.125f * b[q]);
  store8(g + v * C + cc, a);
}

// db[c] += sum over voxels of g[v][c].
__global__ void k_colsum(const __nv_bfloat16* __restrict__ g, size_t nv, int C, float* __restrict__ db) {
  __shared__ float sh[256];
  const int lanes = blockDim.x / C;  // voxels handled side by side
  const int c = threadIdx.x % C, l = threadIdx.x / C;
  float s = 0.f;
  if (l < lanes)
    for (size_t v = (size_t)blockIdx.x * lanes + l; v < nv; v += (size_t)gridDim.x * lanes) s += bf(g[v * C + c]);
  sh[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x < C) {
    float t = 0.f;
    for (int q = 0; q < lanes; ++q) t += sh[q * C + threadIdx.x];
    atomicAdd(db + threadIdx.x, t);
  }
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1, float* __restrict__ m2,
                       size_t count, float lr_t, float b1, float b2, float eps) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float gi = g[i];
  const float a = b1 * m1[i] + (1.f - b1) * gi;
  const float b = b2 * m2[i] + (1.f - b2) * gi * gi;
  m1[i] = a;
  m2[i] = b;
  p[i] -= lr_t * a / (sqrtf(b) + eps);
}

// BF16 copies of one layer's weights: w[tap][co][ci] and wt[26 - tap][ci][co].
__global__ void k_to_bf16_layer(const float* __restrict__ master, int co, int ci, __nv_bfloat16* __restrict__ w,
                                __nv_bfloat16* __restrict__ wt) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t cnt = (size_t)27 * co * ci;
  if (t >= cnt) return;
  const int i = (int)(t % ci), o = (int)((t / ci) % co), tap = (int)(t / ((size_t)ci * co));
  const __nv_bfloat16 h = __float2bfloat16_rn(master[t]);
  w[t] = h;
  wt[((size_t)(26 - tap) * ci + i) * co + o] = h;
}

__global__ void k_f32_to_bf16(const float* __restrict__ a, size_t count, __nv_bfloat16* __restrict__ b) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) b[i] = __float2bfloat16_rn(a[i]);
}

template <typename T>
vg_status device_alloc(Ctx* c, T** p, size_t count) {
  VG_CUDA(c, cudaMalloc((void**)p, count * sizeof(T) + 256));
  return VG_OK;
}

ConvIn layer_input(const Net* N, int l) {
  const LayerDesc& L = kNet[l];
  ConvIn in;
  const int e = N->dims(L.level);
  in.D = in.H = in.W = e;
  if (L.cup) {
    in.x1 = N->act[kIn1[l]];
    in.C1 = L.cup;
    in.up1 = 1;
    in.x2 = N->act[kIn2[l]];
    in.C2 = L.ci - L.cup;
  } else {
    in.x1 = N->act[kIn1[l]];
    in.C1 = L.ci;
    in.up1 = 0;
    in.x2 = nullptr;
    in.C2 = 0;
  }
  return in;
}

vg_status pool(Ctx* c, const Net* N, int a_in, int a_out) {
  const int ec = N->dims(kActLevel[a_out]);
  const int C = kActC[a_in];
  const size_t cnt = (size_t)ec * ec * ec * (C / 8);
  k_pool<<<blocks_for(cnt, 256), 256, 0, c->stream>>>(N->act[a_in], ec, C, N->act[a_out]);
  VG_LAUNCHED(c);
  return VG_OK;
}

vg_status forward(Ctx* c, Net* N) {
  vg_status st;
  for (int l = 0; l < kLayers; ++l) {
    if (l == 2 && (st = pool(c, N, A_E0B, A_P1)) != VG_OK) return st;
    if (l == 4 && (st = pool(c, N, A_E1B, A_P2)) != VG_OK) return st;
    if (l == 6 && (st = pool(c, N, A_E2B, A_P3)) != VG_OK) return st;
    const LayerDesc& L = kNet[l];
    ConvOut o;
    o.y = kOut[l] >= 0 ? N->act[kOut[l]] : nullptr;
    o.yf = kOut[l] >= 0 ? nullptr : N->out;
    o.bias = N->master + N->bofs[l];
    o.mask = nullptr;
    o.Co = L.co;
    o.relu = L.relu;
    o.slope = kSlope;
    o.mask_slope = 1.f;
    if ((st = conv3_fwd(c, layer_input(N, l), N->w + N->wbofs[l], o)) != VG_OK) return st;
  }
  return VG_OK;
}

// Backward pass from N->g[14]; accumulates into N->grad.
vg_status backward(Ctx* c, Net* N) {
  vg_status st;
  for (int l = kLayers - 1; l >= 0; --l) {
    const LayerDesc& L = kNet[l];
    const int e = N->dims(L.level);
    const size_t nv = N->vox(L.level);
    if ((st = conv3_wgrad(c, layer_input(N, l), N->g[l], L.co, N->grad + N->wofs[l])) != VG_OK) return st;
    {
      const int lanes = 256 / L.co;
      unsigned nb = (unsigned)std::min<size_t>((nv + lanes - 1) / lanes, 4 * (size_t)sm_count());
      k_colsum<<<nb, 256, 0, c->stream>>>(N->g[l], nv, L.co, N->grad + N->bofs[l]);
      VG_LAUNCHED(c);
    }
    if (l == 0) break;
    ConvIn gi;
    gi.x1 = N->g[l];
    gi.C1 = L.co;
    gi.x2 = nullptr;
    gi.C2 = 0;
    gi.up1 = 0;
    gi.D = gi.H = gi.W = e;
    ConvOut o;
    o.yf = nullptr;
    o.bias = nullptr;
    o.Co = L.ci;
    o.relu = 0;
    o.slope = 1.f;
    o.mask_slope = kSlope;
    const __nv_bfloat16* wt = N->wt + N->wbofs[l];
    if (L.cup) {
      // gradient of the concatenated input, then its upsampled part back at the coarse level
      o.y = N->gin[l];
      o.mask = nullptr;
      if ((st = conv3_fwd(c, gi, wt, o)) != VG_OK) return st;
      const int ec = e / 2;
      const size_t cnt = (size_t)ec * ec * ec * (L.cup / 8);
      k_up_grad<<<blocks_for(cnt, 256), 256, 0, c->stream>>>(N->gin[l], L.ci, N->act[kIn1[l]], ec, L.cup,
                                                               N->g[l - 1]);
      VG_LAUNCHED(c);
    } else if (l == 2 || l == 4 || l == 6) {
      // gradient of the pooled input, combined with the skip connection's share
      o.y = N->gin[l];
      o.mask = nullptr;
      if ((st = conv3_fwd(c, gi, wt, o)) != VG_OK) return st;
      const int user = l == 2 ? 12 : (l == 4 ? 10 : 8);  // decoder layer that reads the same tensor as a skip
      const int skip_act = l == 2 ? A_E0B : (l == 4 ? A_E1B : A_E2B);
      const int ef = N->dims(kActLevel[skip_act]);
      const int C = kActC[skip_act];
      const size_t cnt = (size_t)ef * ef * ef * (C / 8);
      k_skip_grad<<<blocks_for(cnt, 256), 256, 0, c->stream>>>(N->gin[user], kNet[user].ci, kNet[user].cup, N->gin[l],
                                                                 N->act[skip_act], ef, C, N->g[l - 1]);
      VG_LAUNCHED(c);
    } else {
      o.y = N->g[l - 1];
      o.mask = N->act[kIn1[l]];
      if ((st = conv3_fwd(c, gi, wt, o)) != VG_OK) return st;
    }
  }
  return VG_OK;
}

vg_status refresh_bf16(Ctx* c, Net* N) {
  for (int l = 0; l < kLayers; ++l) {
    const size_t cnt = (size_t)27 * kNet[l].co * kNet[l].ci;
    k_to_bf16_layer<<<blocks_for(cnt, 256), 256, 0, c->stream>>>(N->master + N->wofs[l], kNet[l].co, kNet[l].ci,
                                                                  N->w + N->wbofs[l], N->wt + N->wbofs[l]);
    VG_LAUNCHED(c);
  }
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

float grid_h2(const Geom& g) {
  return (g.cell[0] * g.cell[0] + g.cell[1] * g.cell[1] + g.cell[2] * g.cell[2]) / 3.0f;
}

vg_status check_grid(Ctx* c, const Net* N, const Geom& g) {
  const unsigned np = (unsigned)N->n + 1;
  if (g.np[0] != np || g.np[1] != np || g.np[2] != np) return fail(c, VG_INVALID, "grid shape does not match the network");
  return VG_OK;
}

template <typename T>
vg_status prepare_input(Ctx* c, Net* N, const Geom& g, const T* rhs, const T* vp) {
  const size_t pts = g.points();
  k_sumsq<T><<<kRedBlocks, 256, 0, c->stream>>>(rhs, pts * 3, N->partials);
  k_scales<<<1, 32, 0, c->stream>>>(N->partials, kRedBlocks, (double)pts * 3, grid_h2(g) * N->out_scale, N->scales);
  const size_t nv = N->vox(0);
  k_pack_input<T><<<blocks_for(nv, 256), 256, 0, c->stream>>>(rhs, vp, N->n, N->scales, N->act[A_X]);
  c->launches += 3;
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

template <typename T>
vg_status backward_pair(Ctx* c, Net* N, const Geom& g, const T* rhs, const T* vp, bool accumulate) {
  vg_status st;
  if ((st = prepare_input<T>(c, N, g, rhs, vp)) != VG_OK) return st;
  if ((st = forward(c, N)) != VG_OK) return st;
  const int n = N->n;
  k_target_energy<T><<<kRedBlocks, 256, 0, c->stream>>>(vp, n, N->scales, N->partials);
  k_finish_energy<<<1, 32, 0, c->stream>>>(N->partials, kRedBlocks, N->loss);
  k_loss_grad<T><<<kRedBlocks, 256, 0, c->stream>>>(N->out, vp, n, N->scales, N->loss, N->g[kLayers - 1],
                                                    N->partials);
  k_finish_loss<<<1, 32, 0, c->stream>>>(N->partials, kRedBlocks, N->loss);
  c->launches += 4;
  if (!accumulate) VG_CUDA(c, cudaMemsetAsync(N->grad, 0, N->nparam * sizeof(float), c->stream));
  return backward(c, N);
}

vg_status alloc_net(Net* N) {
  Ctx* c = &N->ctx;
  vg_status st;
  size_t off = 0, woff = 0;
  for (int l = 0; l < kLayers; ++l) {
    N->wofs[l] = off;
    off += (size_t)27 * kNet[l].co * kNet[l].ci;
    N->bofs[l] = off;
    off += kNet[l].co;
    N->wbofs[l] = woff;
    woff += (size_t)27 * kNet[l].co * kNet[l].ci;
  }
  N->nparam = off;
  N->nw = woff;
  if ((st = device_alloc(c, &N->master, off)) != VG_OK) return st;
  if ((st = device_alloc(c, &N->w, woff)) != VG_OK) return st;
  if ((st = device_alloc(c, &N->wt, woff)) != VG_OK) return st;
  for (int a = 0; a < A_NUM; ++a)
    if ((st = device_alloc(c, &N->act[a], N->vox(kActLevel[a]) * kActC[a])) != VG_OK) return st;
  if ((st = device_alloc(c, &N->out, N->vox(0) * 16)) != VG_OK) return st;
  if ((st = device_alloc(c, &N->scales, 4)) != VG_OK) return st;
  if ((st = device_alloc(c, &N->partials, kRedBlocks)) != VG_OK) return st;
  if ((st = device_alloc(c, &N->loss, 4)) != VG_OK) return st;
  if ((st = device_alloc(c, &c->dflag, 64)) != VG_OK) return st;
  VG_CUDA(c, cudaMemset(c->dflag, 0, 64 * sizeof(int)));
  VG_CUDA(c, cudaMemset(N->master, 0, off * sizeof(float)));
  return VG_OK;
}

vg_status alloc_training(Net* N) {
  if (N->grad) return VG_OK;
  Ctx* c = &N->ctx;
  vg_status st;
  if ((st = device_alloc(c, &N->grad, N->nparam)) != VG_OK) return st;
  if ((st = device_alloc(c, &N->m1, N->nparam)) != VG_OK) return st;
  if ((st = device_alloc(c, &N->m2, N->nparam)) != VG_OK) return st;
  VG_CUDA(c, cudaMemset(N->m1, 0, N->nparam * sizeof(float)));
  VG_CUDA(c, cudaMemset(N->m2, 0, N->nparam * sizeof(float)));
  for (int l = 0; l < kLayers; ++l) {
    if ((st = device_alloc(c, &N->g[l], N->vox(kNet[l].level) * kNet[l].co)) != VG_OK) return st;
    if (l == 2 || l == 4 || l == 6 || kNet[l].cup)
      if ((st = device_alloc(c, &N->gin[l], N->vox(kNet[l].level) * kNet[l].ci)) != VG_OK) return st;
  }
  N->step = 0;
  return VG_OK;
}

void free_net(Net* N) {
  if (N->ctx.stream) cudaStreamSynchronize(N->ctx.stream);
  void* ps[] = {N->master, N->grad, N->m1, N->m2, N->w, N->wt, N->out, N->scales, N->partials, N->loss, N->ctx.dflag};
  for (void* p : ps)
    if (p) cudaFree(p);
  for (int a = 0; a < A_NUM; ++a)
    if (N->act[a]) cudaFree(N->act[a]);
  for (int l = 0; l < kLayers; ++l) {
    if (N->g[l]) cudaFree(N->g[l]);
    if (N->gin[l]) cudaFree(N->gin[l]);
  }
  if (N->ctx.own_stream) cudaStreamDestroy(N->ctx.stream);
}

// Weight file: "VGUNET01", u32 layers, u32 edge trained on, f32 output scale,
// then per layer the BF16 bits of W[27][Co][Ci] and the FP32 bias[Co] (little endian).
const char kMagic[8] = {'V', 'G', 'U', 'N', 'E', 'T', '0', '1'};

uint16_t f2bf_bits(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return (uint16_t)((u >> 16) | ((u & 0xffffu) ? 0x40u : 0u));
  u += 0x7fffu + ((u >> 16) & 1u);  // round to nearest even
  return (uint16_t)(u >> 16);
}
float bf_bits2f(uint16_t b) {
  const uint32_t u = (uint32_t)b << 16;
  float f;
  memcpy(&f, &u, 4);
  return f;
}

}  // namespace

size_t param_count() {
  size_t off = 0;
  for (int l = 0; l < kLayers; ++l) off += (size_t)27 * kNet[l].co * kNet[l].ci + kNet[l].co;
  return off;
}

bool fits(const Net* N, const Geom& g) {
  const unsigned np = (unsigned)N->n + 1;
  return N->have_params && g.np[0] == np && g.np[1] == np && g.np[2] == np;
}

// Writes the network's guess into the interior of vp (whose boundary already
// holds the Dirichlet values); rhs is the solver's right-hand side.
vg_status guess(Ctx* c, Net* N, const Geom& g, const float* rhs, float* vp) {
  vg_status st;
  if (!N->have_params) return fail(c, VG_INVALID, "network has no parameters");
  if ((st = check_grid(c, N, g)) != VG_OK) return st;
  if ((st = prepare_input<float>(c, N, g, rhs, vp)) != VG_OK) return st;
  if ((st = forward(c, N)) != VG_OK) return st;
  const size_t nv = N->vox(0);
  k_unpack_output<<<blocks_for(nv, 256), 256, 0, c->stream>>>(N->out, N->n, N->scales, vp);
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

}  // namespace nn
}  // namespace vg

using namespace vg;
using namespace vg::nn;

struct vg_net : public vg::nn::Net {};

namespace {

vg_status net_status(vg_net* N, vg_status st) {
  if (st != VG_OK) cudaGetLastError();
  return st;
}

bool edge_ok(unsigned n) {
  if (n < 32 || n % 8 || n > 1024) return false;
  for (int k = 0; k < kLayers; ++k) {
    const int e = (int)(n >> kNet[k].level);
    const int c1 = kNet[k].cup ? kNet[k].cup : kNet[k].ci, c2 = kNet[k].ci - c1;
    if (!conv_shape_ok(e, e, e, c1, c2, kNet[k].co) || !conv_shape_ok(e, e, e, kNet[k].co, 0, kNet[k].ci)) return false;
  }
  return true;
}

}  // namespace

extern "C" {

vg_status vg_net_create(int device, void* stream, unsigned edge, vg_net** out) {
  if (!out) return set_noctx_error(VG_INVALID, "vg_net_create: null output");
  *out = nullptr;
  if (!edge_ok(edge)) return set_noctx_error(VG_INVALID, "vg_net_create: edge must be 32 or a multiple of 64 up to 1024");
  vg_net* N = new (std::nothrow) vg_net();
  if (!N) return set_noctx_error(VG_OOM, "vg_net_create: out of host memory");
  N->n = (int)edge;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess && stream) {
    N->ctx.stream = (cudaStream_t)stream;
  } else if (e == cudaSuccess) {
    e = cudaStreamCreateWithFlags(&N->ctx.stream, cudaStreamNonBlocking);
    N->ctx.own_stream = e == cudaSuccess;
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    delete N;
    return set_noctx_error(VG_CUDA_ERROR, std::string("vg_net_create: ") + cudaGetErrorString(e));
  }
  vg_status st = alloc_net(N);
  if (st != VG_OK) {
    set_noctx_error(st, N->ctx.err);
    cudaGetLastError();
    free_net(N);
    delete N;
    return st;
  }
  *out = N;
  return VG_OK;
}

vg_status vg_net_destroy(vg_net* N) {
  if (!N) return VG_OK;
  free_net(N);
  delete N;
  return VG_OK;
}

const char* vg_net_last_error(const vg_net* N) { return N ? N->ctx.err.c_str() : ""; }

size_t vg_net_param_count(void) { return param_count(); }

vg_status vg_net_set_params(vg_net* N, const float* params, size_t count, float out_scale) {
  if (!N || !params) return VG_INVALID;
  if (count != N->nparam) return fail(&N->ctx, VG_INVALID, "vg_net_set_params: wrong parameter count");
  if (!(out_scale > 0.f) || !std::isfinite(out_scale)) return fail(&N->ctx, VG_INVALID, "vg_net_set_params: bad scale");
  Ctx* c = &N->ctx;
  VG_CUDA(c, cudaMemcpyAsync(N->master, params, count * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  N->out_scale = out_scale;
  vg_status st = refresh_bf16(c, N);
  if (st != VG_OK) return net_status(N, st);
  if (vg_status sst = sync_and_check(c, "network"); sst != VG_OK) return sst;
  if (N->m1) {
    VG_CUDA(c, cudaMemset(N->m1, 0, N->nparam * sizeof(float)));
    VG_CUDA(c, cudaMemset(N->m2, 0, N->nparam * sizeof(float)));
    N->step = 0;
  }
  N->have_params = true;
  return VG_OK;
}

vg_status vg_net_get_params(vg_net* N, float* params, size_t count, float* out_scale) {
  if (!N || !params) return VG_INVALID;
  if (count != N->nparam) return fail(&N->ctx, VG_INVALID, "vg_net_get_params: wrong parameter count");
  Ctx* c = &N->ctx;
  if (vg_status sst = sync_and_check(c, "network"); sst != VG_OK) return sst;
  VG_CUDA(c, cudaMemcpy(params, N->master, count * sizeof(float), cudaMemcpyDeviceToHost));
  if (out_scale) *out_scale = N->out_scale;
  return VG_OK;
}

vg_status vg_net_get_grads(vg_net* N, float* grads, size_t count) {
  if (!N || !grads) return VG_INVALID;
  if (count != N->nparam || !N->grad) return fail(&N->ctx, VG_INVALID, "vg_net_get_grads: no gradients");
  Ctx* c = &N->ctx;
  if (vg_status sst = sync_and_check(c, "network"); sst != VG_OK) return sst;
  VG_CUDA(c, cudaMemcpy(grads, N->grad, count * sizeof(float), cudaMemcpyDeviceToHost));
  return VG_OK;
}

vg_status vg_net_get_output(vg_net* N, float* out, size_t count) {
  if (!N || !out) return VG_INVALID;
  if (count != N->vox(0) * 16) return fail(&N->ctx, VG_INVALID, "vg_net_get_output: count must be edge^3 * 16");
  Ctx* c = &N->ctx;
  if (vg_status sst = sync_and_check(c, "network"); sst != VG_OK) return sst;
  VG_CUDA(c, cudaMemcpy(out, N->out, count * sizeof(float), cudaMemcpyDeviceToHost));
  return VG_OK;
}

vg_status vg_net_get_activation(vg_net* N, int which, float* out, size_t count) {
  if (!N || !out || which < 0 || which >= A_NUM) return VG_INVALID;
  const size_t cnt = N->vox(kActLevel[which]) * kActC[which];
  if (count != cnt) return fail(&N->ctx, VG_INVALID, "vg_net_get_activation: wrong count");
  Ctx* c = &N->ctx;
  if (vg_status sst = sync_and_check(c, "network"); sst != VG_OK) return sst;
  std::vector<uint16_t> b(cnt);
  VG_CUDA(c, cudaMemcpy(b.data(), N->act[which], cnt * 2, cudaMemcpyDeviceToHost));
  for (size_t i = 0; i < cnt; ++i) out[i] = bf_bits2f(b[i]);
  return VG_OK;
}

vg_status vg_net_get_gradient(vg_net* N, int layer, int of_input, float* out, size_t count) {
  if (!N || !out || layer < 0 || layer >= kLayers) return VG_INVALID;
  const __nv_bfloat16* src = of_input ? N->gin[layer] : N->g[layer];
  if (!src) return fail(&N->ctx, VG_INVALID, "vg_net_get_gradient: no such gradient (run a backward pass first)");
  const size_t cnt = N->vox(kNet[layer].level) * (of_input ? kNet[layer].ci : kNet[layer].co);
  if (count != cnt) return fail(&N->ctx, VG_INVALID, "vg_net_get_gradient: wrong count");
  Ctx* c = &N->ctx;
  if (vg_status sst = sync_and_check(c, "network"); sst != VG_OK) return sst;
  std::vector<uint16_t> b(cnt);
  VG_CUDA(c, cudaMemcpy(b.data(), src, cnt * 2, cudaMemcpyDeviceToHost));
  for (size_t i = 0; i < cnt; ++i) out[i] = bf_bits2f(b[i]);
  return VG_OK;
}

vg_status vg_net_save(vg_net* N, const char* path) {
  if (!N || !path) return VG_INVALID;
  std::vector<float> p(N->nparam);
  vg_status st = vg_net_get_params(N, p.data(), p.size(), nullptr);
  if (st != VG_OK) return st;
  FILE* f = fopen(path, "wb");
  if (!f) return fail(&N->ctx, VG_INVALID, std::string("vg_net_save: cannot open ") + path);
  bool ok = fwrite(kMagic, 1, 8, f) == 8;
  const uint32_t hdr[2] = {(uint32_t)kLayers, (uint32_t)N->n};
  ok = ok && fwrite(hdr, 4, 2, f) == 2 && fwrite(&N->out_scale, 4, 1, f) == 1;
  for (int l = 0; l < kLayers && ok; ++l) {
    const size_t cnt = (size_t)27 * kNet[l].co * kNet[l].ci;
    std::vector<uint16_t> b(cnt);
    for (size_t i = 0; i < cnt; ++i) b[i] = f2bf_bits(p[N->wofs[l] + i]);
    ok = fwrite(b.data(), 2, cnt, f) == cnt && fwrite(&p[N->bofs[l]], 4, kNet[l].co, f) == (size_t)kNet[l].co;
  }
  ok = fclose(f) == 0 && ok;
  return ok ? VG_OK : fail(&N->ctx, VG_INVALID, std::string("vg_net_save: write failed for ") + path);
}

vg_status vg_net_load(vg_net* N, const char* path) {
  if (!N || !path) return VG_INVALID;
  FILE* f = fopen(path, "rb");
  if (!f) return fail(&N->ctx, VG_INVALID, std::string("vg_net_load: cannot open ") + path);
  char magic[8];
  uint32_t hdr[2];
  float scale = 0.f;
  bool ok = fread(magic, 1, 8, f) == 8 && memcmp(magic, kMagic, 8) == 0 && fread(hdr, 4, 2, f) == 2 &&
            hdr[0] == (uint32_t)kLayers && fread(&scale, 4, 1, f) == 1;
  std::vector<float> p(N->nparam);
  for (int l = 0; l < kLayers && ok; ++l) {
    const size_t cnt = (size_t)27 * kNet[l].co * kNet[l].ci;
    std::vector<uint16_t> b(cnt);
    ok = fread(b.data(), 2, cnt, f) == cnt && fread(&p[N->bofs[l]], 4, kNet[l].co, f) == (size_t)kNet[l].co;
    for (size_t i = 0; ok && i < cnt; ++i) p[N->wofs[l] + i] = bf_bits2f(b[i]);
  }
  char extra;
  ok = ok && fread(&extra, 1, 1, f) == 0;
  fclose(f);
  if (!ok) return fail(&N->ctx, VG_INVALID, std::string("vg_net_load: not a network weight file: ") + path);
  return vg_net_set_params(N, p.data(), p.size(), scale);
}

vg_status vg_net_guess_device(vg_net* N, const vg_grid_geom* g, const float* rhs3, float* vecpot3) {
  if (!N || !g || !rhs3 || !vecpot3) return VG_INVALID;
  return net_status(N, guess(&N->ctx, N, to_geom(*g), rhs3, vecpot3));
}

vg_status vg_net_backward_device(vg_net* N, const vg_grid_geom* g, int pair_bf16, const void* rhs3,
                                 const void* vecpot3, int accumulate, float* loss) {
  if (!N || !g || !rhs3 || !vecpot3) return VG_INVALID;
  Ctx* c = &N->ctx;
  if (!N->have_params) return fail(c, VG_INVALID, "network has no parameters");
  const Geom G = to_geom(*g);
  vg_status st = check_grid(c, N, G);
  if (st == VG_OK) st = alloc_training(N);
  if (st == VG_OK)
    st = pair_bf16 ? backward_pair<__nv_bfloat16>(c, N, G, (const __nv_bfloat16*)rhs3, (const __nv_bfloat16*)vecpot3,
                                                  accumulate != 0)
                   : backward_pair<float>(c, N, G, (const float*)rhs3, (const float*)vecpot3, accumulate != 0);
  if (st != VG_OK) return net_status(N, st);
  if (loss) {
    if (vg_status sst = sync_and_check(c, "network"); sst != VG_OK) return sst;
    VG_CUDA(c, cudaMemcpy(loss, N->loss, sizeof(float), cudaMemcpyDeviceToHost));
  }
  return VG_OK;
}

vg_status vg_net_adam_step(vg_net* N, float lr, float beta1, float beta2, float eps) {
  if (!N) return VG_INVALID;
  Ctx* c = &N->ctx;
  if (!N->grad) return fail(c, VG_INVALID, "vg_net_adam_step: no gradients (call vg_net_backward_device first)");
  N->step += 1;
  const double bc1 = 1.0 - pow((double)beta1, (double)N->step), bc2 = 1.0 - pow((double)beta2, (double)N->step);
  const float lr_t = (float)(lr * sqrt(bc2) / bc1);
  k_adam<<<blocks_for(N->nparam, 256), 256, 0, c->stream>>>(N->master, N->grad, N->m1, N->m2, N->nparam, lr_t, beta1,
                                                             beta2, eps);
  VG_LAUNCHED(c);
  return net_status(N, refresh_bf16(c, N));
}

vg_status vg_net_to_bf16_device(const float* src, void* dst, size_t count, void* stream) {
  if (!src || !dst) return set_noctx_error(VG_INVALID, "vg_net_to_bf16_device: null pointer");
  k_f32_to_bf16<<<blocks_for(count, 256), 256, 0, (cudaStream_t)stream>>>(src, count, (__nv_bfloat16*)dst);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_noctx_error(VG_CUDA_ERROR, cudaGetErrorString(e));
  return VG_OK;
}

vg_status vg_net_synchronize(vg_net* N) {
  if (!N) return VG_INVALID;
  Ctx* c = &N->ctx;
  if (vg_status sst = sync_and_check(c, "network"); sst != VG_OK) return sst;
  return VG_OK;
}

}  // extern "C"
