// BF16 tensor-core 3x3x3 convolutions for the learned warm start.
//
// Products are BF16 x BF16 with FP32 accumulation (mma.sync.m16n8k16).
//
//  * k_conv3_fwd: implicit GEMM, M = voxels, N = output channels, K = 27 taps x
//    input channels.  A CTA (4 warps, 2 m16 tiles each) owns a tile of 128
//    output voxels (8 x 4 x 4 in x, y, z) x CO_T output channels.  Per
//    16-channel input slice it stages the zero-padded halo of the tile and the
//    slice's 27 x CO_T x 16 weights in shared memory (16-byte chunks XOR-
//    swizzled so that ldmatrix rows fall in distinct banks), then per tap each
//    warp issues one ldmatrix.x4 per m16 tile and CO_T/8 ldmatrix.x2 + MMAs.
//    The input may be the channel concatenation of two tensors, the first read
//    through a nearest 2x upsampling (the decoder), so neither the upsampled
//    nor the concatenated tensor exists in memory.
//    Epilogue: + bias, leaky ReLU, mask, BF16 or FP32 store.  With flipped,
//    transposed weights the same kernel computes input gradients.
//  * k_conv3_wgrad: dW[tap][co][ci] = sum_v dY[v][co] X[v + tap][ci] as per-tap
//    GEMMs (M = 16 output channels, N = 16 input channels, K = voxels) with
//    ldmatrix.trans operands; a CTA owns one 16 x 16 (co, ci) block and strides
//    over voxel tiles, each warp owns a quarter of the taps, and the FP32
//    partials are added to dW atomically once per CTA.
#include <algorithm>

#include "vg_nn.cuh"

namespace vg {
namespace nn {

namespace {

constexpr int kTileVox = 128;
constexpr int kWarps = 4;
constexpr int kMT = 2;          // m16 tiles per warp
constexpr int kMaxHalo = 360;   // (tx+2)(ty+2)(tz+2) for the tiles make_tile builds when W, H >= 4

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void ldsm_x4(const void* p, unsigned& r0, unsigned& r1, unsigned& r2, unsigned& r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x2(const void* p, unsigned& r0, unsigned& r1) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];" : "=r"(r0), "=r"(r1) : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x4_t(const void* p, unsigned& r0, unsigned& r1, unsigned& r2, unsigned& r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(smem_u32(p)));
}
__device__ __forceinline__ void mma_bf16(float* d, unsigned a0, unsigned a1, unsigned a2, unsigned a3, unsigned b0,
                                         unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// A row of 16 BF16 values (two 16-byte chunks) lives at uint4 index 2*s + (c ^ ((s >> 2) & 1)).
__device__ __forceinline__ int chunk_at(int s, int c) { return 2 * s + (c ^ ((s >> 2) & 1)); }

// Output tile: tx x ty x tz voxels (tx = min(W, 8), ty = min(H, 4), tz fills 128).
struct Tile {
  int tx, ty, tz, vox;
  int nx, ny, nz;
};
__host__ __device__ inline Tile make_tile(int D, int H, int W) {
  Tile t;
  t.tx = W < 8 ? W : 8;
  t.ty = H < 4 ? H : 4;
  const int rest = kTileVox / (t.tx * t.ty);
  t.tz = D < rest ? D : rest;
  t.vox = t.tx * t.ty * t.tz;
  t.nx = W / t.tx;
  t.ny = H / t.ty;
  t.nz = D / t.tz;
  return t;
}

// Copies 16 channels (ci0..ci0+15) of voxel (z, y, x) of the input into the
// two swizzled chunks of halo slot s; zeros outside the volume.
__device__ __forceinline__ void load_vox16(uint4* sx, int s, const ConvIn& in, int z, int y, int x, int ci0) {
  uint4 a = make_uint4(0, 0, 0, 0), b = a;
  if (z >= 0 && y >= 0 && x >= 0 && z < in.D && y < in.H && x < in.W) {
    const __nv_bfloat16* p;
    if (ci0 < in.C1) {
      if (in.up1) {
        const int H1 = in.H >> 1, W1 = in.W >> 1;
        p = in.x1 + (((size_t)(z >> 1) * H1 + (y >> 1)) * W1 + (x >> 1)) * in.C1 + ci0;
      } else {
        p = in.x1 + (((size_t)z * in.H + y) * in.W + x) * in.C1 + ci0;
      }
    } else {
      p = in.x2 + (((size_t)z * in.H + y) * in.W + x) * in.C2 + (ci0 - in.C1);
    }
    const uint4* q = reinterpret_cast<const uint4*>(p);
    a = __ldg(q);
    b = __ldg(q + 1);
  }
  sx[chunk_at(s, 0)] = a;
  sx[chunk_at(s, 1)] = b;
}

__device__ __forceinline__ void tile_origin(const Tile& T, int b, int& x0, int& y0, int& z0) {
  x0 = (b % T.nx) * T.tx;
  b /= T.nx;
  y0 = (b % T.ny) * T.ty;
  z0 = (b / T.ny) * T.tz;
}

__device__ __forceinline__ void stage_halo(uint4* sx, const Tile& T, const ConvIn& in, int x0, int y0, int z0, int ci0) {
  const int hx = T.tx + 2, hy = T.ty + 2, nh = hx * hy * (T.tz + 2);
  for (int s = threadIdx.x; s < nh; s += blockDim.x) {
    const int ix = s % hx, iy = (s / hx) % hy, iz = s / (hx * hy);
    load_vox16(sx, s, in, z0 + iz - 1, y0 + iy - 1, x0 + ix - 1, ci0);
  }
}

// Halo slot of tile voxel v (its centre tap).
__device__ __forceinline__ int centre_slot(const Tile& T, int v) {
  const int vx = v % T.tx, vy = (v / T.tx) % T.ty, vz = v / (T.tx * T.ty);
  return ((vz + 1) * (T.ty + 2) + vy + 1) * (T.tx + 2) + vx + 1;
}

// Epilogue of one output tile: C fragment rows (voxels) lane/4 and lane/4 + 8,
// columns 2 (lane % 4) + {0, 1}; + bias, activation, mask, store.
template <int CO_T>
__device__ __forceinline__ void store_tile(const float (&acc)[kMT][CO_T / 8][4], const bool (&active)[kMT],
                                           const ConvIn& in, const ConvOut& out, const Tile& T, int x0, int y0, int z0,
                                           int co0) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, q2 = (lane & 3) * 2, Co = out.Co;
#pragma unroll
  for (int mt = 0; mt < kMT; ++mt) {
    if (!active[mt]) continue;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int v = (warp * kMT + mt) * 16 + g + 8 * h;
      const int vx = x0 + v % T.tx, vy = y0 + (v / T.tx) % T.ty, vz = z0 + v / (T.tx * T.ty);
      const size_t vox = ((size_t)vz * in.H + vy) * in.W + vx;
#pragma unroll
      for (int n = 0; n < CO_T / 8; ++n) {
        const int co = co0 + n * 8 + q2;
        float v0 = acc[mt][n][2 * h], v1 = acc[mt][n][2 * h + 1];
        if (out.bias) {
          v0 += out.bias[co];
          v1 += out.bias[co + 1];
        }
        if (out.relu) {
          v0 = v0 > 0.f ? v0 : out.slope * v0;
          v1 = v1 > 0.f ? v1 : out.slope * v1;
        }
        if (out.mask) {
          const __nv_bfloat162 mk = *reinterpret_cast<const __nv_bfloat162*>(out.mask + vox * Co + co);
          if (!(__bfloat162float(mk.x) > 0.f)) v0 *= out.mask_slope;
          if (!(__bfloat162float(mk.y) > 0.f)) v1 *= out.mask_slope;
        }
        if (out.yf)
          *reinterpret_cast<float2*>(out.yf + vox * Co + co) = make_float2(v0, v1);
        else
          *reinterpret_cast<__nv_bfloat162*>(out.y + vox * Co + co) = __floats2bfloat162_rn(v0, v1);
      }
    }
  }
}

template <int CO_T>
__global__ void __launch_bounds__(kWarps * 32) k_conv3_fwd(const ConvIn in, const __nv_bfloat16* __restrict__ wt,
                                                           const ConvOut out) {
  extern __shared__ __align__(16) uint4 smem4[];
  const Tile T = make_tile(in.D, in.H, in.W);
  const int hx = T.tx + 2, hy = T.ty + 2, nh = hx * hy * (T.tz + 2);
  uint4* sx = smem4;
  uint4* sw = smem4 + 2 * nh;
  int x0, y0, z0;
  tile_origin(T, blockIdx.x, x0, y0, z0);
  const int co0 = blockIdx.y * CO_T;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int Ci = in.C1 + in.C2, Co = out.Co;
  int cslot[kMT];
  bool active[kMT];
#pragma unroll
  for (int mt = 0; mt < kMT; ++mt) {
    const int m0 = (warp * kMT + mt) * 16;
    active[mt] = m0 < T.vox;
    cslot[mt] = active[mt] ? centre_slot(T, m0 + (lane & 15)) : 0;
  }
  float acc[kMT][CO_T / 8][4];
#pragma unroll
  for (int mt = 0; mt < kMT; ++mt)
#pragma unroll
    for (int n = 0; n < CO_T / 8; ++n) acc[mt][n][0] = acc[mt][n][1] = acc[mt][n][2] = acc[mt][n][3] = 0.f;

  for (int ci0 = 0; ci0 < Ci; ci0 += 16) {
    __syncthreads();
    stage_halo(sx, T, in, x0, y0, z0, ci0);
    for (int r = threadIdx.x; r < 27 * CO_T; r += blockDim.x) {
      const int tap = r / CO_T, co = r % CO_T;
      const uint4* q = reinterpret_cast<const uint4*>(wt + ((size_t)tap * Co + co0 + co) * Ci + ci0);
      sw[chunk_at(r, 0)] = __ldg(q);
      sw[chunk_at(r, 1)] = __ldg(q + 1);
    }
    __syncthreads();
#pragma unroll 1
    for (int tap = 0; tap < 27; ++tap) {
      const int off = ((tap / 9 - 1) * hy + ((tap / 3) % 3 - 1)) * hx + (tap % 3 - 1);
      unsigned a[kMT][4];
#pragma unroll
      for (int mt = 0; mt < kMT; ++mt)
        if (active[mt]) ldsm_x4(sx + chunk_at(cslot[mt] + off, lane >> 4), a[mt][0], a[mt][1], a[mt][2], a[mt][3]);
#pragma unroll
      for (int n = 0; n < CO_T / 8; ++n) {
        const int row = tap * CO_T + n * 8 + (lane & 7);
        unsigned b0, b1;
        ldsm_x2(sw + chunk_at(row, (lane >> 3) & 1), b0, b1);
#pragma unroll
        for (int mt = 0; mt < kMT; ++mt)
          if (active[mt]) mma_bf16(acc[mt][n], a[mt][0], a[mt][1], a[mt][2], a[mt][3], b0, b1);
      }
    }
  }
  store_tile<CO_T>(acc, active, in, out, T, x0, y0, z0, co0);
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, int src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smem_u32(smem)), "l"(gmem), "r"(src_bytes));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all_but_newest() { asm volatile("cp.async.wait_group 1;\n" ::); }

// Issues asynchronous copies of one 16-channel slice of a tile's halo into sx;
// voxels outside the volume are zero-filled (a 0-byte source read).
__device__ __forceinline__ void issue_halo(uint4* sx, const Tile& T, const ConvIn& in, int x0, int y0, int z0,
                                           int ci0) {
  const int hx = T.tx + 2, hy = T.ty + 2, nh = hx * hy * (T.tz + 2);
  for (int s = threadIdx.x; s < nh; s += blockDim.x) {
    const int ix = s % hx, iy = (s / hx) % hy, iz = s / (hx * hy);
    const int z = z0 + iz - 1, y = y0 + iy - 1, x = x0 + ix - 1;
    const bool inside = z >= 0 && y >= 0 && x >= 0 && z < in.D && y < in.H && x < in.W;
    const __nv_bfloat16* p = in.x1;  // a valid address when nothing is read
    if (inside) {
      if (ci0 < in.C1) {
        if (in.up1) {
          const int H1 = in.H >> 1, W1 = in.W >> 1;
          p = in.x1 + (((size_t)(z >> 1) * H1 + (y >> 1)) * W1 + (x >> 1)) * in.C1 + ci0;
        } else {
          p = in.x1 + (((size_t)z * in.H + y) * in.W + x) * in.C1 + ci0;
        }
      } else {
        p = in.x2 + (((size_t)z * in.H + y) * in.W + x) * in.C2 + (ci0 - in.C1);
      }
    }
    const int nb = inside ? 16 : 0;
    cp_async16(sx + chunk_at(s, 0), p, nb);
    cp_async16(sx + chunk_at(s, 1), p + 8, nb);
  }
}

// Persistent form of k_conv3_fwd for layers whose weights (one output-channel
// group, every input slice) fit in shared memory: each CTA keeps its group's
// weights resident, walks its tiles (blockIdx / ncog, then every
// gridDim / ncog) slice by slice, and copies the next slice's halo with
// cp.async while the tensor cores work on the current one (two buffers).
template <int CO_T>
__global__ void __launch_bounds__(kWarps * 32) k_conv3_fwd_resident(const ConvIn in,
                                                                    const __nv_bfloat16* __restrict__ wt,
                                                                    const ConvOut out, int ncog) {
  extern __shared__ __align__(16) uint4 smem4[];
  const Tile T = make_tile(in.D, in.H, in.W);
  const int hx = T.tx + 2, hy = T.ty + 2, nh = hx * hy * (T.tz + 2);
  const int Ci = in.C1 + in.C2, nsl = Ci / 16, Co = out.Co;
  const int wrows = 27 * CO_T;
  uint4* sw = smem4;  // row i = slice * wrows + tap * CO_T + co, two chunks each
  uint4* sxb0 = sw + 2 * wrows * nsl;
  uint4* sxb1 = sxb0 + 2 * nh;
  const int co0 = (blockIdx.x % ncog) * CO_T;
  const int t0 = blockIdx.x / ncog, tstride = gridDim.x / ncog;
  const int ntiles = T.nx * T.ny * T.nz;
  if (t0 >= ntiles) return;  // whole CTA: no barrier is skipped by part of it
  const int nst = ((ntiles - t0 + tstride - 1) / tstride) * nsl;
  for (int i = threadIdx.x; i < wrows * nsl; i += blockDim.x) {
    const int sl = i / wrows, r = i % wrows, tap = r / CO_T, co = r % CO_T;
    const __nv_bfloat16* src = wt + ((size_t)tap * Co + co0 + co) * Ci + sl * 16;
    cp_async16(sw + chunk_at(i, 0), src, 16);
    cp_async16(sw + chunk_at(i, 1), src + 8, 16);
  }
  {
    int x0, y0, z0;
    tile_origin(T, t0, x0, y0, z0);
    issue_halo(sxb0, T, in, x0, y0, z0, 0);
  }
  cp_async_commit();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int cslot[kMT];
  bool active[kMT];
#pragma unroll
  for (int mt = 0; mt < kMT; ++mt) {
    const int m0 = (warp * kMT + mt) * 16;
    active[mt] = m0 < T.vox;
    cslot[mt] = active[mt] ? centre_slot(T, m0 + (lane & 15)) : 0;
  }
  float acc[kMT][CO_T / 8][4];
#pragma unroll
  for (int mt = 0; mt < kMT; ++mt)
#pragma unroll
    for (int n = 0; n < CO_T / 8; ++n) acc[mt][n][0] = acc[mt][n][1] = acc[mt][n][2] = acc[mt][n][3] = 0.f;
  for (int st = 0; st < nst; ++st) {
    if (st + 1 < nst) {
      int x0, y0, z0;
      tile_origin(T, t0 + ((st + 1) / nsl) * tstride, x0, y0, z0);
      issue_halo((st + 1) & 1 ? sxb1 : sxb0, T, in, x0, y0, z0, ((st + 1) % nsl) * 16);
    }
    cp_async_commit();
    cp_async_wait_all_but_newest();
    __syncthreads();
    const uint4* sx = st & 1 ? sxb1 : sxb0;
    const int rbase = (st % nsl) * wrows;
#pragma unroll 1
    for (int tap = 0; tap < 27; ++tap) {
      const int off = ((tap / 9 - 1) * hy + ((tap / 3) % 3 - 1)) * hx + (tap % 3 - 1);
      unsigned a[kMT][4];
#pragma unroll
      for (int mt = 0; mt < kMT; ++mt)
        if (active[mt]) ldsm_x4(sx + chunk_at(cslot[mt] + off, lane >> 4), a[mt][0], a[mt][1], a[mt][2], a[mt][3]);
#pragma unroll
      for (int n = 0; n < CO_T / 8; ++n) {
        const int row = rbase + tap * CO_T + n * 8 + (lane & 7);
        unsigned b0, b1;
        ldsm_x2(sw + chunk_at(row, (lane >> 3) & 1), b0, b1);
#pragma unroll
        for (int mt = 0; mt < kMT; ++mt)
          if (active[mt]) mma_bf16(acc[mt][n], a[mt][0], a[mt][1], a[mt][2], a[mt][3], b0, b1);
      }
    }
    if (st % nsl == nsl - 1) {
      int x0, y0, z0;
      tile_origin(T, t0 + (st / nsl) * tstride, x0, y0, z0);
      store_tile<CO_T>(acc, active, in, out, T, x0, y0, z0, co0);
#pragma unroll
      for (int mt = 0; mt < kMT; ++mt)
#pragma unroll
        for (int n = 0; n < CO_T / 8; ++n) acc[mt][n][0] = acc[mt][n][1] = acc[mt][n][2] = acc[mt][n][3] = 0.f;
    }
    __syncthreads();  // the buffer just read is refilled by the next iteration's copies
  }
}

__global__ void __launch_bounds__(kWarps * 32) k_conv3_wgrad(const ConvIn in, const __nv_bfloat16* __restrict__ dy,
                                                             int Co, float* __restrict__ dw) {
  __shared__ __align__(16) uint4 sdy[2 * kTileVox];
  __shared__ __align__(16) uint4 sx[2 * kMaxHalo];
  const Tile T = make_tile(in.D, in.H, in.W);
  const int hx = T.tx + 2, hy = T.ty + 2;
  const int Ci = in.C1 + in.C2, nci = Ci / 16;
  const int co0 = (blockIdx.x / nci) * 16, ci0 = (blockIdx.x % nci) * 16;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int m = lane >> 3, r = lane & 7;
  float acc[7][2][4];
#pragma unroll
  for (int t = 0; t < 7; ++t)
#pragma unroll
    for (int n = 0; n < 2; ++n) acc[t][n][0] = acc[t][n][1] = acc[t][n][2] = acc[t][n][3] = 0.f;
  const int ntiles = T.nx * T.ny * T.nz;
  for (int tile = blockIdx.y; tile < ntiles; tile += gridDim.y) {
    int x0, y0, z0;
    tile_origin(T, tile, x0, y0, z0);
    __syncthreads();
    for (int v = threadIdx.x; v < T.vox; v += blockDim.x) {
      const int vx = x0 + v % T.tx, vy = y0 + (v / T.tx) % T.ty, vz = z0 + v / (T.tx * T.ty);
      const uint4* q = reinterpret_cast<const uint4*>(dy + (((size_t)vz * in.H + vy) * in.W + vx) * Co + co0);
      sdy[chunk_at(v, 0)] = __ldg(q);
      sdy[chunk_at(v, 1)] = __ldg(q + 1);
    }
    stage_halo(sx, T, in, x0, y0, z0, ci0);
    __syncthreads();
    for (int k0 = 0; k0 < T.vox; k0 += 16) {
      // A = dY^T (rows co, cols voxels): matrix m covers voxels k0 + 8 (m >> 1), channels 8 (m & 1)
      const int va = k0 + ((m >> 1) << 3) + r;
      unsigned a0, a1, a2, a3;
      ldsm_x4_t(sdy + chunk_at(va, m & 1), a0, a1, a2, a3);
      // B = X_tap (rows voxels, cols ci): matrix m covers voxels k0 + 8 (m & 1), channels 8 (m >> 1)
      const int cb = centre_slot(T, k0 + ((m & 1) << 3) + r);
#pragma unroll
      for (int ts = 0; ts < 7; ++ts) {
        const int tap = warp + 4 * ts;
        if (tap < 27) {
          const int off = ((tap / 9 - 1) * hy + ((tap / 3) % 3 - 1)) * hx + (tap % 3 - 1);
          unsigned b0, b1, b2, b3;
          ldsm_x4_t(sx + chunk_at(cb + off, m >> 1), b0, b1, b2, b3);
          mma_bf16(acc[ts][0], a0, a1, a2, a3, b0, b1);
          mma_bf16(acc[ts][1], a0, a1, a2, a3, b2, b3);
        }
      }
    }
  }
  // C rows = co (lane/4, +8), cols = ci (2 (lane % 4) + {0, 1}) within each n8 block
  const int g = lane >> 2, q2 = (lane & 3) * 2;
#pragma unroll
  for (int ts = 0; ts < 7; ++ts) {
    const int tap = warp + 4 * ts;
    if (tap >= 27) continue;
#pragma unroll
    for (int n = 0; n < 2; ++n)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        float* p = dw + ((size_t)tap * Co + co0 + g + 8 * h) * Ci + ci0 + n * 8 + q2;
        atomicAdd(p, acc[ts][n][2 * h]);
        atomicAdd(p + 1, acc[ts][n][2 * h + 1]);
      }
  }
}

// Set on every launch: the attribute is per device, and the call is cheap.
template <int CO_T>
void set_fwd_smem_attr() {
  cudaFuncSetAttribute(k_conv3_fwd<CO_T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (2 * kMaxHalo + 2 * 27 * CO_T) * 16);
}

}  // namespace

bool conv_shape_ok(int D, int H, int W, int C1, int C2, int Co) {
  if (D < 1 || H < 4 || W < 4 || C1 < 16 || C1 % 16 || C2 < 0 || C2 % 16 || Co < 16 || Co % 16) return false;
  const Tile T = make_tile(D, H, W);
  return W % T.tx == 0 && H % T.ty == 0 && D % T.tz == 0 && T.vox % 16 == 0;
}

size_t conv3_fwd_smem(int D, int H, int W, int co_t) {
  const Tile T = make_tile(D, H, W);
  const size_t nh = (size_t)(T.tx + 2) * (T.ty + 2) * (T.tz + 2);
  return (2 * nh + 2 * 27 * (size_t)co_t) * 16;
}

namespace {

constexpr size_t kResidentWeightBytes = 100 * 1024;

template <int CO_T>
vg_status launch_resident(Ctx* c, const ConvIn& in, const __nv_bfloat16* wt, const ConvOut& out) {
  const Tile T = make_tile(in.D, in.H, in.W);
  const int Ci = in.C1 + in.C2, ncog = out.Co / CO_T;
  const size_t nh = (size_t)(T.tx + 2) * (T.ty + 2) * (T.tz + 2);
  const size_t smem = (2 * 27 * (size_t)CO_T * (Ci / 16) + 4 * nh) * 16;
  VG_CUDA(c, cudaFuncSetAttribute(k_conv3_fwd_resident<CO_T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
  int per_sm = 0;
  VG_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_conv3_fwd_resident<CO_T>, kWarps * 32, smem));
  const long items = (long)T.nx * T.ny * T.nz * ncog;
  long grid = std::min<long>(items, (long)std::max(per_sm, 1) * sm_count());
  grid = std::max<long>(ncog, grid / ncog * ncog);
  k_conv3_fwd_resident<CO_T><<<(unsigned)grid, kWarps * 32, smem, c->stream>>>(in, wt, out, ncog);
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

}  // namespace

vg_status conv3_fwd(Ctx* c, const ConvIn& in, const __nv_bfloat16* wt, const ConvOut& out) {
  if (!conv_shape_ok(in.D, in.H, in.W, in.C1, in.C2, out.Co) || (in.up1 && (in.D % 2 || in.H % 2 || in.W % 2)) ||
      (!out.y && !out.yf))
    return fail(c, VG_INVALID, "conv3: unsupported shape");
  {
    bool handled = false;
    const vg_status st = conv3_fwd_umma(c, in, wt, out, &handled);
    if (handled || st != VG_OK) return st;
  }
  const Tile T = make_tile(in.D, in.H, in.W);
  const size_t Ci = (size_t)(in.C1 + in.C2);
  // weights resident in shared memory when one output-channel group's fit
  for (int co_t : {64, 32, 16}) {
    if (out.Co % co_t || 27 * (size_t)co_t * Ci * 2 > kResidentWeightBytes) continue;
    if (co_t == 64) return launch_resident<64>(c, in, wt, out);
    if (co_t == 32) return launch_resident<32>(c, in, wt, out);
    return launch_resident<16>(c, in, wt, out);
  }
  // otherwise weights stream with the halo, slice by slice; the group width is
  // the widest that still gives two CTAs per SM
  const long tiles = (long)T.nx * T.ny * T.nz;
  int co_t = 16;
  for (int w : {64, 32}) {
    if (out.Co % w == 0 && tiles * (out.Co / w) >= 2L * sm_count()) {
      co_t = w;
      break;
    }
  }
  if (out.Co % 32 && co_t != 16) co_t = 16;
  const size_t smem = conv3_fwd_smem(in.D, in.H, in.W, co_t);
  const dim3 grid((unsigned)tiles, (unsigned)(out.Co / co_t));
  if (co_t == 64) {
    set_fwd_smem_attr<64>();
    k_conv3_fwd<64><<<grid, kWarps * 32, smem, c->stream>>>(in, wt, out);
  } else if (co_t == 32) {
    set_fwd_smem_attr<32>();
    k_conv3_fwd<32><<<grid, kWarps * 32, smem, c->stream>>>(in, wt, out);
  } else {
    set_fwd_smem_attr<16>();
    k_conv3_fwd<16><<<grid, kWarps * 32, smem, c->stream>>>(in, wt, out);
  }
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

vg_status conv3_wgrad(Ctx* c, const ConvIn& in, const __nv_bfloat16* dy, int Co, float* dw) {
  if (!conv_shape_ok(in.D, in.H, in.W, in.C1, in.C2, Co) || (in.up1 && (in.D % 2 || in.H % 2 || in.W % 2)))
    return fail(c, VG_INVALID, "conv3 wgrad: unsupported shape");
  const Tile T = make_tile(in.D, in.H, in.W);
  const int ntiles = T.nx * T.ny * T.nz;
  const int blocks_cc = (Co / 16) * ((in.C1 + in.C2) / 16);
  int splits = (4 * sm_count() + blocks_cc - 1) / blocks_cc;
  if (splits > ntiles) splits = ntiles;
  if (splits < 1) splits = 1;
  k_conv3_wgrad<<<dim3((unsigned)blocks_cc, (unsigned)splits), kWarps * 32, 0, c->stream>>>(in, dy, Co, dw);
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

}  // namespace nn
}  // namespace vg
