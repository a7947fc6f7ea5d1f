// K6-K9: vector-potential Poisson solve  L a = b  (b = -vorticity) with
// Dirichlet boundary values, to a relative-residual tolerance.
//
// The reference solves the same equation with a fixed-work cascade
// (VortonFluid/vortonSim.cpp:2539-2571) that never targets a residual; this
// is a correction-scheme multigrid in iterative refinement:
//   * each cycle: r = b - L a (the residual of the current iterate, norms
//     accumulated in FP64 and reduced in a fixed order), then one FP32
//     V(2,2)-cycle on L e = r -- point red-black Gauss-Seidel (colour = parity
//     of x+y+z), 27-point full-weighting restriction fused with the residual
//     (the reference's SLOWER_MORE_ACCURATE weights, uniformGrid.h:1453-1585),
//     trilinear prolongation, an exact solve on the coarsest grid -- and
//     a += e;
//   * phase 1 iterates on the FP32 field with an FP32 residual while FP32 can
//     still represent it (relative residual above 1e-4);
//   * phase 2 (iterative refinement) keeps the iterate as the FP32 field plus
//     an FP32 correction field, evaluates r = b - L a to FP64-class accuracy
//     (float-pair sums with exact FMA-split products; GB300's FP64 pipe runs
//     at a small fraction of its FP32 rate), solves the correction L e = r
//     with FP32 cycles (the correction's residual is small, so FP32 tracks it
//     well), accumulates e and checks with another such residual -- reaching
//     residuals far below FP32's cancellation floor (~1e-4 at 128^3) with two
//     accurate residual evaluations per solve.
// FP64 is used for the norms (and the host-built tables of the coarsest
// solve).  The hierarchy stops at the finest level with at most 32,768
// interior points, which is solved exactly by sine transforms (over the whole
// GPU, or inside the small-level CTA when it has at most 512); levels of at
// most 17^3 points above such a small one run inside one CTA with their
// fields in shared memory; each cycle is captured once as a CUDA graph and
// replayed.
// Grids are float[3] per point (x fastest); the three components are three
// independent scalar problems solved together.
#include <float.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "vg_internal.cuh"

namespace vg {

namespace {

constexpr int kRedThreads = 256;

struct Lev {
  Geom g;
  float r2x, r2y, r2z, H;  // FP32 operator constants
  size_t base;             // offset (points) into level arrays
};

// Block reduction (kRedThreads threads, any 2D shape) of two sums into
// part[2 * b + {0, 1}], b the linear block index: 32-term warp sums in FP32
// (relative error ~1e-6, irrelevant for a norm), then FP64 across warps,
// blocks and the grid.
__device__ __forceinline__ void block_sum2(float a32, float b32, double* __restrict__ part) {
  __shared__ double s_a[kRedThreads / 32], s_b[kRedThreads / 32];
  const unsigned tid = threadIdx.x + blockDim.x * threadIdx.y;
  for (int o = 16; o > 0; o >>= 1) {
    a32 += __shfl_xor_sync(0xffffffffu, a32, o);
    b32 += __shfl_xor_sync(0xffffffffu, b32, o);
  }
  if ((tid & 31) == 0) {
    s_a[tid >> 5] = (double)a32;
    s_b[tid >> 5] = (double)b32;
  }
  __syncthreads();
  if (tid == 0) {
    double t1 = 0.0, t2 = 0.0;
    for (int w = 0; w < kRedThreads / 32; ++w) {
      t1 += s_a[w];
      t2 += s_b[w];
    }
    const unsigned b = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    part[2 * b] = t1;
    part[2 * b + 1] = t2;
  }
}

// Residual kernels run over interior points in rows: blocks of (bx, by) =
// kRedThreads threads over (x, y), each thread stepping through `zs` planes.
struct ResLaunch {
  dim3 grid, block;
  unsigned zs, nb;  // planes per thread, blocks (= partial sums)
};
static ResLaunch res_launch(const Geom& g) {
  const unsigned nxi = g.np[0] - 2, nyi = g.np[1] - 2, nzi = g.np[2] - 2;
  unsigned bx = 32;
  while (bx < nxi && bx < (unsigned)kRedThreads) bx <<= 1;
  const unsigned by = kRedThreads / bx;
  const unsigned gx = (nxi + bx - 1) / bx, gy = (nyi + by - 1) / by;
  const unsigned zs = (size_t)gx * gy * nzi >= 4096 ? 4 : 1;
  ResLaunch L;
  L.block = dim3(bx, by, 1);
  L.grid = dim3(gx, gy, (nzi + zs - 1) / zs);
  L.zs = zs;
  L.nb = L.grid.x * L.grid.y * L.grid.z;
  return L;
}

// Point arithmetic shared by the per-level kernels and the persistent batched
// solve, written as explicit round-to-nearest operations so that every caller
// compiles to the same float operations (no contraction left to the compiler).
// L v at a point: the 7-point Laplacian from the centre c0 and the neighbours
// along x, y and z.
__device__ __forceinline__ float lap7(float c0, float xp, float xm, float yp, float ym, float zp, float zm,
                                      float r2x, float r2y, float r2z) {
  const float tx = __fmaf_rn(-2.f, c0, __fadd_rn(xp, xm));
  const float ty = __fmaf_rn(-2.f, c0, __fadd_rn(yp, ym));
  const float tz = __fmaf_rn(-2.f, c0, __fadd_rn(zp, zm));
  return __fmaf_rn(tx, r2x, __fmaf_rn(ty, r2y, __fmul_rn(tz, r2z)));
}

// The Gauss-Seidel value of a point from its neighbour sums along x, y, z.
__device__ __forceinline__ float gs_value(float sx, float sy, float sz, float r, float r2x, float r2y, float r2z,
                                          float H) {
  return __fmul_rn(__fsub_rn(__fmaf_rn(sx, r2x, __fmaf_rn(sy, r2y, __fmul_rn(sz, r2z))), r), H);
}

// The smoother is over-relaxed red-black Gauss-Seidel: a point moves to
// e + omega (gs - e).  With omega = 1.3 a V(2,2)-cycle of this hierarchy
// (full-weighting restriction, trilinear prolongation, exact coarsest solve)
// contracts the residual by ~0.02 per cycle on the 7-point Laplacian instead
// of ~0.09 at omega = 1, at every grid size and for cell aspect ratios up to
// 3 (a V-cycle model in double precision on 33^3 and 65^3 grids, random
// right-hand sides), so a solve to 1e-6 takes about 4 cycles instead of 6.
// From e = 0 the update is omega gs.
constexpr float kSorOmega = 1.3f;
__device__ __forceinline__ float sor_value(float e_old, float gs) {
  return __fmaf_rn(kSorOmega, __fsub_rn(gs, e_old), e_old);
}

// Phase 1 residual: r = b - L a in FP32 from the FP32 iterate at interior
// points (boundary r is never read); per-block FP64 partial sums of r^2 and b^2.
__global__ void __launch_bounds__(kRedThreads) k_residual32n(Geom g, float r2x, float r2y, float r2z, unsigned zs,
                                                             const float* __restrict__ a, const float* __restrict__ b,
                                                             float* __restrict__ r, double* __restrict__ part) {
  pdl_entry();
  const unsigned x = blockIdx.x * blockDim.x + threadIdx.x + 1, y = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const unsigned nx = g.np[0], ny = g.np[1], nz = g.np[2];
  float rr = 0.f, bb = 0.f;
  if (x + 1 < nx && y + 1 < ny) {
    const unsigned sy = nx, sz = nx * ny;
    const unsigned z0 = 1 + blockIdx.z * zs, z1 = min(nz - 1, z0 + zs);
    for (unsigned z = z0; z < z1; ++z) {
      const unsigned k = x + sy * y + sz * z;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float lap = lap7(a[3 * k + c], a[3 * (k + 1) + c], a[3 * (k - 1) + c], a[3 * (k + sy) + c],
                               a[3 * (k - sy) + c], a[3 * (k + sz) + c], a[3 * (k - sz) + c], r2x, r2y, r2z);
        const float bv = b[3 * k + c];
        const float rv = __fsub_rn(bv, lap);
        r[3 * k + c] = rv;
        rr = fmaf(rv, rv, rr);
        bb = fmaf(bv, bv, bb);
      }
    }
  }
  block_sum2(rr, bb, part);
}

// Phase 2 residual: r = b - L (hi + lo) for the iterate kept as a pair of
// FP32 fields (hi: phase 1's FP32 iterate, fixed during refinement; lo: the
// accumulated corrections).  L hi, where b - L hi cancels to ~1e-6 of the
// terms, is summed as an unevaluated pair of floats: every product
// coefficient x value is split exactly by an FMA (the coefficients themselves
// carried as float pairs) and added with error-free TwoSum, so the sum keeps
// ~2^-46 relative accuracy -- the FP64-class residual of iterative refinement
// without GB300's low-rate FP64 pipe.  L lo is small and needs only FP32.
// Stored as FP32, with per-block FP64 partial sums of r^2 (b^2 slot unused).
struct PairCoef {
  float xh, xl, yh, yl, zh, zl, dh, dl;  // r2x, r2y, r2z and -2 (r2x + r2y + r2z) as float pairs
  float r2x, r2y, r2z;                   // the FP32 operator of the cycles
};

__device__ __forceinline__ void pair_add_prod(float ch, float cl, float v, float& sh, float& sl) {
  const float p = __fmul_rn(ch, v);
  const float pe = __fmaf_rn(ch, v, -p);  // ch v - p exactly
  const float t = __fadd_rn(sh, p);      // TwoSum(sh, p)
  const float bv = __fsub_rn(t, sh);
  const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bv)), __fsub_rn(p, bv));
  sh = t;
  sl = __fadd_rn(sl, __fadd_rn(err, __fmaf_rn(cl, v, pe)));
}

// r = b - L (hi + lo) at a point from the centre and neighbour values of hi
// and lo, in the order centre, x+, x-, y+, y-, z+, z-.
__device__ __forceinline__ float pair_residual(const float (&h)[7], const float (&l)[7], float bv, const PairCoef& cf) {
  float sh = 0.f, sl = 0.f;
  pair_add_prod(cf.dh, cf.dl, h[0], sh, sl);
  pair_add_prod(cf.xh, cf.xl, h[1], sh, sl);
  pair_add_prod(cf.xh, cf.xl, h[2], sh, sl);
  pair_add_prod(cf.yh, cf.yl, h[3], sh, sl);
  pair_add_prod(cf.yh, cf.yl, h[4], sh, sl);
  pair_add_prod(cf.zh, cf.zl, h[5], sh, sl);
  pair_add_prod(cf.zh, cf.zl, h[6], sh, sl);
  const float lap_lo = lap7(l[0], l[1], l[2], l[3], l[4], l[5], l[6], cf.r2x, cf.r2y, cf.r2z);
  // r = (b - sh) - sl - lap_lo, the first difference by TwoSum
  const float t = __fsub_rn(bv, sh);
  const float bb = __fsub_rn(t, bv);
  const float terr = __fadd_rn(__fsub_rn(bv, __fsub_rn(t, bb)), __fsub_rn(-sh, bb));
  return __fadd_rn(t, __fsub_rn(__fsub_rn(terr, sl), lap_lo));
}

// kLo false: lo is zero (not read); the result is the same as from a zero field.
template <bool kLo = true>
__global__ void __launch_bounds__(kRedThreads) k_residual_pair(Geom g, PairCoef cf, unsigned zs,
                                                               const float* __restrict__ hi,
                                                               const float* __restrict__ lo,
                                                               const float* __restrict__ b, float* __restrict__ r,
                                                               double* __restrict__ part) {
  pdl_entry();
  const unsigned x = blockIdx.x * blockDim.x + threadIdx.x + 1, y = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const unsigned nx = g.np[0], ny = g.np[1], nz = g.np[2];
  float rr = 0.f;
  if (x + 1 < nx && y + 1 < ny) {
    const unsigned sy = nx, sz = nx * ny;
    const unsigned z0 = 1 + blockIdx.z * zs, z1 = min(nz - 1, z0 + zs);
    for (unsigned z = z0; z < z1; ++z) {
      const unsigned k = x + sy * y + sz * z;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const unsigned o[7] = {k, k + 1, k - 1, k + sy, k - sy, k + sz, k - sz};
        float h[7], l[7];
#pragma unroll
        for (int i = 0; i < 7; ++i) {
          h[i] = hi[3 * o[i] + c];
          l[i] = kLo ? lo[3 * o[i] + c] : 0.f;
        }
        const float rv = pair_residual(h, l, b[3 * k + c], cf);
        r[3 * k + c] = rv;
        rr = fmaf(rv, rv, rr);
      }
    }
  }
  block_sum2(rr, 0.f, part);
}

// Sum the per-block partials in a fixed order (one block); with keep_b the
// ||b||^2 slot is left as phase 1's first residual wrote it.
__global__ void __launch_bounds__(1024) k_sum_partials(const double* __restrict__ part, int nb,
                                                       double* __restrict__ out2, int keep_b) {
  pdl_entry();
  __shared__ double s1[1024], s2[1024];
  double a1 = 0.0, a2 = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    a1 += part[2 * i];
    a2 += part[2 * i + 1];
  }
  s1[threadIdx.x] = a1;
  s2[threadIdx.x] = a2;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      s1[threadIdx.x] += s1[threadIdx.x + s];
      s2[threadIdx.x] += s2[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out2[0] = s1[0];
    if (!keep_b) out2[1] = s2[0];
  }
}

__device__ __forceinline__ void rbgs_point(const Geom& g, float r2x, float r2y, float r2z, float H,
                                           float* __restrict__ e, const float* __restrict__ r, size_t k,
                                           bool zero_first) {
  const size_t sy = g.np[0], sz = (size_t)g.np[0] * g.np[1];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    float v;
    if (zero_first) {
      v = sor_value(0.f, __fmul_rn(-r[3 * k + c], H));
    } else {
      const float sx = __fadd_rn(e[3 * (k + 1) + c], e[3 * (k - 1) + c]);
      const float syv = __fadd_rn(e[3 * (k + sy) + c], e[3 * (k - sy) + c]);
      const float szv = __fadd_rn(e[3 * (k + sz) + c], e[3 * (k - sz) + c]);
      v = sor_value(e[3 * k + c], gs_value(sx, syv, szv, r[3 * k + c], r2x, r2y, r2z, H));
    }
    e[3 * k + c] = v;
  }
}

// Point red-black Gauss-Seidel on L e = r (FP32).  One thread per component
// of an interior point of `color`: threadIdx.x runs along a row over
// (point j, component c) pairs -- x = 1 + parity + 2 j, components adjacent --
// so a warp reads ~11 points' worth of consecutive floats of the AoS field
// instead of 32 points 24 bytes apart; y and z come from the block index
// (launch_rows), so no thread divides by a grid size.  zero_first: e is zero
// before this sweep, so the red points take -r H directly.
__global__ void __launch_bounds__(256) k_rbgs(Geom g, float r2x, float r2y, float r2z, float H,
                                              float* __restrict__ e, const float* __restrict__ r, unsigned color,
                                              int zero_first) {
  pdl_entry();
  const unsigned nx = g.np[0], ny = g.np[1];
  const unsigned jc = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned y = blockIdx.y * blockDim.y + threadIdx.y + 1, z = blockIdx.z + 1;
  const unsigned j = jc / 3u, c = jc - 3u * j;
  const unsigned x = 1u + ((color + 1u + y + z) & 1u) + 2u * j;
  if (y + 1 >= ny || x + 1 >= nx) return;
  const unsigned k = x + nx * (y + ny * z);
  const unsigned sy = nx, sz = nx * ny;
  float v;
  if (zero_first) {
    v = sor_value(0.f, __fmul_rn(-r[3 * k + c], H));
  } else {
    const float sx = __fadd_rn(e[3 * (k + 1) + c], e[3 * (k - 1) + c]);
    const float syv = __fadd_rn(e[3 * (k + sy) + c], e[3 * (k - sy) + c]);
    const float szv = __fadd_rn(e[3 * (k + sz) + c], e[3 * (k - sz) + c]);
    v = sor_value(e[3 * k + c], gs_value(sx, syv, szv, r[3 * k + c], r2x, r2y, r2z, H));
  }
  e[3 * k + c] = v;
}

// The first pre-smoothing sweep from e = 0, both colours in one pass: red
// points take -r H, black points the Gauss-Seidel update from those red
// values (recomputed from r, the same float operations as the two half
// sweeps, so the result is identical).  Threads over every interior (point,
// component), as k_rbgs_add.
__global__ void __launch_bounds__(256) k_rbgs_first(Geom g, float r2x, float r2y, float r2z, float H,
                                                    float* __restrict__ e, const float* __restrict__ r) {
  pdl_entry();
  const unsigned nx = g.np[0], ny = g.np[1];
  const unsigned jc = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned y = blockIdx.y * blockDim.y + threadIdx.y + 1, z = blockIdx.z + 1;
  const unsigned j = jc / 3u, c = jc - 3u * j;
  const unsigned x = 1u + j;
  if (y + 1 >= ny || x + 1 >= nx) return;
  const unsigned k = x + nx * (y + ny * z), t = 3 * k + c;
  float v;
  if (((x + y + z) & 1u) == 0u) {
    v = sor_value(0.f, __fmul_rn(-r[t], H));
  } else {
    const unsigned sy = nx, sz = nx * ny;
    // red neighbours: omega (-r H) (boundary neighbours stay e = 0)
    auto red = [&](unsigned n, bool in) { return in ? sor_value(0.f, __fmul_rn(-r[3 * n + c], H)) : 0.f; };
    const float sx = __fadd_rn(red(k + 1, x + 2 < nx), red(k - 1, x > 1));
    const float syv = __fadd_rn(red(k + sy, y + 2 < ny), red(k - sy, y > 1));
    const float szv = __fadd_rn(red(k + sz, z + 2 < g.np[2]), red(k - sz, z > 1));
    v = sor_value(0.f, gs_value(sx, syv, szv, r[t], r2x, r2y, r2z, H));
  }
  e[t] = v;
}

// Fused FP32 residual + full-weighting restriction at coarse interior point
// (x, y, z): the fine residuals r - L e at the 27 fine points around
// (2x, 2y, 2z) with weights 8/4/2/1 / 64, recomputed instead of writing the
// fine residual field.  Levels halve exactly (fine n = 2 coarse n - 1 per
// axis), so those fine points are all interior.
__device__ __forceinline__ void residual_restrict_point(const Geom& F, const Geom& C, float r2x, float r2y,
                                                        float r2z, const float* __restrict__ e,
                                                        const float* __restrict__ r, unsigned x, unsigned y,
                                                        unsigned z, float* __restrict__ rc) {
  const unsigned sy = F.np[0], sz = F.np[0] * F.np[1];
  const unsigned f0 = 2 * x + sy * (2 * y) + sz * (2 * z);
  float acc[3] = {0.f, 0.f, 0.f};
#pragma unroll 1  // the 1024-thread CTA has 64 registers per thread
  for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
      for (int dx = -1; dx <= 1; ++dx) {
        const float wt = (float)(8 >> (abs(dx) + abs(dy) + abs(dz)));
        const unsigned o = f0 + dx + sy * dy + sz * dz;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float lap = lap7(e[3 * o + c], e[3 * (o + 1) + c], e[3 * (o - 1) + c], e[3 * (o + sy) + c],
                                 e[3 * (o - sy) + c], e[3 * (o + sz) + c], e[3 * (o - sz) + c], r2x, r2y, r2z);
          acc[c] = __fmaf_rn(wt, __fsub_rn(r[3 * o + c], lap), acc[c]);
        }
      }
  const float s = 1.0f / 64.0f;
  const unsigned k = x + C.np[0] * (y + C.np[1] * z);
  rc[3 * k] = __fmul_rn(acc[0], s);
  rc[3 * k + 1] = __fmul_rn(acc[1], s);
  rc[3 * k + 2] = __fmul_rn(acc[2], s);
}

// Global-memory form, tiled: a CTA owns kRTX x kRTY x kRTZ coarse points.  It
// first computes the fine residuals r - L e of the (2 kRTX + 1) x (2 kRTY + 1)
// x (2 kRTZ + 1) fine points around them into shared memory (coalesced along
// fine rows, each fine residual evaluated once per tile instead of once per
// coarse neighbour), then each (coarse point, component) sums its 27 fine
// residuals in the order of residual_restrict_point.  Coarse boundary points
// are never read, so they are not written.
constexpr int kRTX = 16, kRTY = 4, kRTZ = 2;
constexpr int kRFX = 2 * kRTX + 1, kRFY = 2 * kRTY + 1, kRFZ = 2 * kRTZ + 1;
__global__ void __launch_bounds__(256) k_residual_restrict(Geom F, Geom C, float r2x, float r2y, float r2z,
                                                           const float* __restrict__ e, const float* __restrict__ r,
                                                           float* __restrict__ rc) {
  pdl_entry();
  __shared__ float s_res[kRFX * kRFY * kRFZ * 3];
  const unsigned cx0 = 1 + blockIdx.x * kRTX, cy0 = 1 + blockIdx.y * kRTY, cz0 = 1 + blockIdx.z * kRTZ;
  const unsigned nx = F.np[0], ny = F.np[1], nz = F.np[2];
  const unsigned sy = nx, sz = nx * ny;
  // fine local (0, 0, 0) is fine (2 cx0 - 1, 2 cy0 - 1, 2 cz0 - 1)
  for (unsigned p = threadIdx.x; p < (unsigned)(kRFX * kRFY * kRFZ); p += blockDim.x) {
    const unsigned lx = p % kRFX, q = p / kRFX;
    const unsigned ly = q % kRFY, lz = q / kRFY;
    const unsigned fx = 2 * cx0 - 1 + lx, fy = 2 * cy0 - 1 + ly, fz = 2 * cz0 - 1 + lz;
    float v[3] = {0.f, 0.f, 0.f};
    if (fx + 1 < nx && fy + 1 < ny && fz + 1 < nz) {  // fx, fy, fz >= 1 by construction
      const unsigned o = fx + sy * fy + sz * fz;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float lap = lap7(e[3 * o + c], e[3 * (o + 1) + c], e[3 * (o - 1) + c], e[3 * (o + sy) + c],
                               e[3 * (o - sy) + c], e[3 * (o + sz) + c], e[3 * (o - sz) + c], r2x, r2y, r2z);
        v[c] = __fsub_rn(r[3 * o + c], lap);
      }
    }
    s_res[3 * p] = v[0];
    s_res[3 * p + 1] = v[1];
    s_res[3 * p + 2] = v[2];
  }
  __syncthreads();
  // levels halve exactly, so the 27 fine points of a coarse interior point
  // are all interior
  for (unsigned i = threadIdx.x; i < (unsigned)(kRTX * kRTY * kRTZ * 3); i += blockDim.x) {
    const unsigned c = i % 3u, p = i / 3u;
    const unsigned lx = p % kRTX, q = p / kRTX;
    const unsigned ly = q % kRTY, lz = q / kRTY;
    const unsigned x = cx0 + lx, y = cy0 + ly, z = cz0 + lz;
    if (x + 1 >= C.np[0] || y + 1 >= C.np[1] || z + 1 >= C.np[2]) continue;
    const float* sr = s_res + 3 * ((2 * lx + 1) + kRFX * ((2 * ly + 1) + kRFY * (2 * lz + 1))) + c;
    float acc = 0.f;
#pragma unroll
    for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
      for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
        for (int dx = -1; dx <= 1; ++dx) {
          const float wt = (float)(8 >> (abs(dx) + abs(dy) + abs(dz)));
          acc = __fmaf_rn(wt, sr[3 * (dx + kRFX * (dy + kRFY * dz))], acc);
        }
    rc[3 * (x + C.np[0] * (y + C.np[1] * z)) + c] = __fmul_rn(acc, 1.0f / 64.0f);
  }
}

// e_fine += trilinear(e_coarse) at fine interior point (x, y, z).
__device__ __forceinline__ void prolong_point(const Geom& F, const Geom& C, const float* __restrict__ ec,
                                              float* __restrict__ ef, unsigned x, unsigned y, unsigned z) {
  const unsigned ox = x & 1, oy = y & 1, oz = z & 1;
  const unsigned sy = C.np[0], sz = C.np[0] * C.np[1];
  const unsigned c0 = (x >> 1) + sy * (y >> 1) + sz * (z >> 1);
  float a0 = 0.f, a1 = 0.f, a2 = 0.f;
  const float wt = 1.0f / (float)(1u << (ox + oy + oz));
  for (unsigned iz = 0; iz <= oz; ++iz)
    for (unsigned iy = 0; iy <= oy; ++iy)
      for (unsigned ix = 0; ix <= ox; ++ix) {
        const unsigned o = c0 + ix + sy * iy + sz * iz;
        a0 += ec[3 * o];
        a1 += ec[3 * o + 1];
        a2 += ec[3 * o + 2];
      }
  const unsigned k = x + F.np[0] * (y + F.np[1] * z);
  ef[3 * k] += a0 * wt;
  ef[3 * k + 1] += a1 * wt;
  ef[3 * k + 2] += a2 * wt;
}

// Global-memory form for small levels: one thread per coarse cell (cx .. cx+1) x (cy .. cy+1) x
// (cz .. cz+1), all three components: it reads the cell's 8 corners once and
// updates the 8 fine points (2 cx + ox, 2 cy + oy, 2 cz + oz) with the same
// sums in the same order as prolong_point (fine boundary points skipped).
__global__ void __launch_bounds__(256) k_prolong_cells(Geom F, Geom C, const float* __restrict__ ec,
                                                     float* __restrict__ ef) {
  pdl_entry();
  const unsigned cx = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned cy = blockIdx.y * blockDim.y + threadIdx.y, cz = blockIdx.z;
  if (cx + 1 >= C.np[0] || cy + 1 >= C.np[1]) return;
  const unsigned sy = C.np[0], sz = C.np[0] * C.np[1];
  const unsigned c0 = cx + sy * cy + sz * cz;
  float v[2][2][2][3];  // [iz][iy][ix][component]
#pragma unroll
  for (int iz = 0; iz < 2; ++iz)
#pragma unroll
    for (int iy = 0; iy < 2; ++iy)
#pragma unroll
      for (int ix = 0; ix < 2; ++ix)
#pragma unroll
        for (int c = 0; c < 3; ++c) v[iz][iy][ix][c] = ec[3 * (c0 + ix + sy * iy + sz * iz) + c];
  const unsigned fsy = F.np[0], fsz = F.np[0] * F.np[1];
#pragma unroll
  for (int oz = 0; oz < 2; ++oz)
#pragma unroll
    for (int oy = 0; oy < 2; ++oy)
#pragma unroll
      for (int ox = 0; ox < 2; ++ox) {
        const unsigned X = 2 * cx + ox, Y = 2 * cy + oy, Z = 2 * cz + oz;
        if (X == 0 || Y == 0 || Z == 0) continue;  // X <= nx - 2 etc. always
        const float wt = 1.0f / (float)(1u << (ox + oy + oz));
        const unsigned k = X + fsy * Y + fsz * Z;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          float a = 0.f;
#pragma unroll
          for (int iz = 0; iz <= oz; ++iz)
#pragma unroll
            for (int iy = 0; iy <= oy; ++iy)
#pragma unroll
              for (int ix = 0; ix <= ox; ++ix) a += v[iz][iy][ix][c];
          ef[3 * k + c] += a * wt;
        }
      }
}

// Global-memory form: a CTA of kPCX x kPCY x kPCZ threads, one per coarse
// cell (cx .. cx+1) x (cy .. cy+1) x (cz .. cz+1).  Each thread reads its
// cell's 8 corners once and forms the increments of the 8 fine points
// (2 cx + ox, 2 cy + oy, 2 cz + oz), all three components, with the same sums
// in the same order as prolong_point; the increments go through shared memory
// so that the read-modify-write of the fine field runs along whole fine rows
// (per-thread 24-byte runs would write every sector in pieces).  Fine
// boundary points are skipped.
template <int kPCX, int kPCY, int kPCZ>
__global__ void __launch_bounds__(kPCX * kPCY * kPCZ) k_prolong_add(Geom F, Geom C, const float* __restrict__ ec,
                                                                   float* __restrict__ ef) {
  pdl_entry();
  constexpr int kPFX = 2 * kPCX * 3, kPFR = 2 * kPCY * 2 * kPCZ;  // floats per fine row, fine rows per CTA
  __shared__ float s_inc[kPFR * kPFX];
  const unsigned tx = threadIdx.x, ty = threadIdx.y, tz = threadIdx.z;
  const unsigned cx0 = blockIdx.x * kPCX, cy0 = blockIdx.y * kPCY, cz0 = blockIdx.z * kPCZ;
  const unsigned cx = cx0 + tx, cy = cy0 + ty, cz = cz0 + tz;
  if (cx + 1 < C.np[0] && cy + 1 < C.np[1] && cz + 1 < C.np[2]) {
    const unsigned sy = C.np[0], sz = C.np[0] * C.np[1];
    const unsigned c0 = cx + sy * cy + sz * cz;
    float v[2][2][2][3];  // [iz][iy][ix][component]
#pragma unroll
    for (int iz = 0; iz < 2; ++iz)
#pragma unroll
      for (int iy = 0; iy < 2; ++iy)
#pragma unroll
        for (int ix = 0; ix < 2; ++ix)
#pragma unroll
          for (int c = 0; c < 3; ++c) v[iz][iy][ix][c] = ec[3 * (c0 + ix + sy * iy + sz * iz) + c];
#pragma unroll
    for (int oz = 0; oz < 2; ++oz)
#pragma unroll
      for (int oy = 0; oy < 2; ++oy)
#pragma unroll
        for (int ox = 0; ox < 2; ++ox) {
          const float wt = 1.0f / (float)(1u << (ox + oy + oz));
          const unsigned row = (2 * ty + oy) + 2 * kPCY * (2 * tz + oz);
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            float a = 0.f;
#pragma unroll
            for (int iz = 0; iz <= oz; ++iz)
#pragma unroll
              for (int iy = 0; iy <= oy; ++iy)
#pragma unroll
                for (int ix = 0; ix <= ox; ++ix) a += v[iz][iy][ix][c];
            s_inc[row * kPFX + 3 * (2 * tx + ox) + c] = a * wt;
          }
        }
  }
  __syncthreads();
  // fine rows Y = 2 cy0 + (0 .. 2 kPCY - 1), Z = 2 cz0 + (0 .. 2 kPCZ - 1);
  // fine x = 2 cx0 + (0 .. 2 kPCX - 1)
  const unsigned nthreads = kPCX * kPCY * kPCZ, tid = tx + kPCX * (ty + kPCY * tz);
  const unsigned X0 = 2 * cx0, Y0 = 2 * cy0, Z0 = 2 * cz0;
  for (unsigned i = tid; i < (unsigned)(kPFR * kPFX); i += nthreads) {
    const unsigned row = i / kPFX, col = i - row * kPFX;
    const unsigned X = X0 + col / 3u, Y = Y0 + row % (2 * kPCY), Z = Z0 + row / (2 * kPCY);
    if (X == 0 || Y == 0 || Z == 0 || X + 1 >= F.np[0] || Y + 1 >= F.np[1] || Z + 1 >= F.np[2]) continue;
    ef[3 * (X + F.np[0] * (Y + F.np[1] * Z)) + col % 3u] += s_inc[i];
  }
}

// Launch shape of the row kernels above over `items` (point, component)
// pairs per row and the interior rows (ny - 2) x (nz - 2) of a level: rows of
// up to 256 threads, rounded to whole warps; short rows stack in y.
struct RowLaunch {
  dim3 grid, block;
};
static RowLaunch launch_rows(unsigned items, unsigned ny, unsigned nz) {
  const unsigned nb = (items + 255) / 256;
  const unsigned bx = ((items + nb - 1) / nb + 31) / 32 * 32;
  unsigned by = std::max(1u, 256u / bx);
  while (by > 1 && by / 2 >= ny - 2) by >>= 1;
  RowLaunch L;
  L.block = dim3(bx, by, 1);
  L.grid = dim3(nb, (ny - 2 + by - 1) / by, nz - 2);
  return L;
}

// The small levels of a V-cycle in one CTA, their e and r in shared memory:
// pre-smoothing and fused residual-restriction down to the coarsest grid, an
// exact sine-transform solve there (or FP64 Gauss-Seidel when the hierarchy
// ends above kDirectMax interior points, e.g. on odd point counts), then
// prolongation and post-smoothing back up.
// The first small level reads its r from global memory and writes its e back.
constexpr int kSmallMax = 8;
constexpr int kCoarseShared = 1536;  // doubles of the coarsest solve kept in shared memory
constexpr unsigned kDirectMax = 512;         // interior points of a coarsest level solved in the small-level CTA
constexpr unsigned kDirectGlobalMax = 32768;  // ... or by sine-transform passes over the whole GPU
constexpr size_t kSmallLevelPoints = 17 * 17 * 17;
struct SmallLevels {
  int n;  // levels handled here
  Geom g[kSmallMax];
  float r2x[kSmallMax], r2y[kSmallMax], r2z[kSmallMax], H[kSmallMax];
  unsigned off[kSmallMax];  // float offsets of e (r follows e) in shared memory
  // Interior rows of a level as work items: row r = t >> sh, lane t & mask.
  // shc: lanes for one colour's points of a row; sha: for all interior points.
  unsigned shc[kSmallMax], sha[kSmallMax];
  float inv_nyi[kSmallMax];  // 1 / (ny - 2): z = r / (ny - 2) by a float product
  const float* dst;         // coarsest level solved exactly: its sine-transform tables (direct_tables), or null
  const float* r_in;        // first small level's r (global)
  float* e_out;             // first small level's e (global)
  int pre, post, coarse_sweeps;
};

__device__ __forceinline__ float* sm_e(float* sm, const SmallLevels& S, int l) { return sm + S.off[l]; }
__device__ __forceinline__ float* sm_r(float* sm, const SmallLevels& S, int l) {
  return sm + S.off[l] + 3 * S.g[l].points();
}

// Work item t over the interior rows of small level l with 2^sh lanes per row:
// lane j, interior row (y, z).  z = r / (ny - 2) by a float product, exact for
// the row counts of these levels (r < 2^20, ny - 2 < 2^10).
__device__ __forceinline__ void row_item(const SmallLevels& S, int l, unsigned sh, unsigned t, unsigned& j,
                                         unsigned& y, unsigned& z) {
  const unsigned nyi = S.g[l].np[1] - 2;
  const unsigned r = t >> sh;
  j = t & ((1u << sh) - 1u);
  const unsigned zz = __float2uint_rz(((float)r + 0.5f) * S.inv_nyi[l]);
  y = 1 + r - zz * nyi;
  z = 1 + zz;
}

__device__ __forceinline__ unsigned row_items(const SmallLevels& S, int l, unsigned sh) {
  return ((S.g[l].np[1] - 2) * (S.g[l].np[2] - 2)) << sh;
}

__device__ void block_rb_sweep(float* sm, const SmallLevels& S, int l, unsigned color, bool zero_first) {
  const Geom& g = S.g[l];
  float* e = sm_e(sm, S, l);
  const float* r = sm_r(sm, S, l);
  const unsigned sh = S.shc[l], items = row_items(S, l, sh);
  for (unsigned t = threadIdx.x; t < items; t += blockDim.x) {
    unsigned j, y, z;
    row_item(S, l, sh, t, j, y, z);
    const unsigned x = 1u + ((color + 1u + y + z) & 1u) + 2u * j;
    if (x + 1 >= g.np[0]) continue;
    rbgs_point(g, S.r2x[l], S.r2y[l], S.r2z[l], S.H[l], e, r, x + g.np[0] * (y + g.np[1] * z), zero_first);
  }
  __syncthreads();
}

__global__ void __launch_bounds__(1024) k_vcycle_small(const __grid_constant__ SmallLevels S,
                                                       double* __restrict__ work) {
  pdl_entry();
  extern __shared__ float sm[];
  {  // e = 0 everywhere (boundaries stay 0), r of the first level from global
    const size_t total = S.off[S.n - 1] + 6 * S.g[S.n - 1].points();
    for (size_t k = threadIdx.x; k < total; k += blockDim.x) sm[k] = 0.f;
    __syncthreads();
    const size_t n0 = 3 * S.g[0].points();
    float* r0 = sm_r(sm, S, 0);
    for (size_t k = threadIdx.x; k < n0; k += blockDim.x) r0[k] = S.r_in[k];
    __syncthreads();
  }
  for (int l = 0; l < S.n - 1; ++l) {
    for (int s = 0; s < S.pre; ++s) {
      block_rb_sweep(sm, S, l, 0, s == 0);
      block_rb_sweep(sm, S, l, 1, false);
    }
    const Geom& C = S.g[l + 1];
    {  // coarse interior points only: boundary r is never read (and stays 0)
      const unsigned sh = S.sha[l + 1], items = row_items(S, l + 1, sh);
      for (unsigned t = threadIdx.x; t < items; t += blockDim.x) {
        unsigned j, y, z;
        row_item(S, l + 1, sh, t, j, y, z);
        if (j + 2 >= C.np[0]) continue;
        residual_restrict_point(S.g[l], C, S.r2x[l], S.r2y[l], S.r2z[l], sm_e(sm, S, l), sm_r(sm, S, l), 1 + j,
                                y, z, sm_r(sm, S, l + 1));
      }
    }
    __syncthreads();
  }
  if (S.dst) {
    // Coarsest grid solved exactly: L is diagonalised by the discrete sine
    // transform along each axis, so e = S (D^-1 (S r)) with S = Sx Sy Sz
    // (orthonormal DST-I, its own inverse) and D the eigenvalues.  Seven
    // passes over the interior, ping-ponging between this level's r and e
    // arrays in compact layout (3 (x + nx' (y + ny' z)) + c).
    const int l = S.n - 1;
    const Geom& g = S.g[l];
    const unsigned nxi = g.np[0] - 2, nyi = g.np[1] - 2, nzi = g.np[2] - 2, N = nxi * nyi * nzi;
    float* E = sm_e(sm, S, l);
    float* R = sm_r(sm, S, l);
    const float* Sx = S.dst;
    const float* Sy = Sx + nxi * nxi;
    const float* Sz = Sy + nyi * nyi;
    const float* Dinv = Sz + nzi * nzi;
    for (unsigned i = threadIdx.x; i < 3 * N; i += blockDim.x) {  // R (full) -> E (compact)
      const unsigned c = i % 3u, p = i / 3u;
      const unsigned x = p % nxi, q = p / nxi, y = q % nyi, z = q / nyi;
      E[i] = R[3 * ((x + 1) + g.np[0] * ((y + 1) + g.np[1] * (z + 1))) + c];
    }
    __syncthreads();
    // one transform pass along axis a (stride st, length n, table T): out = T in
    auto pass = [&](const float* in, float* out, const float* T, unsigned n, unsigned st, bool scale) {
      for (unsigned i = threadIdx.x; i < 3 * N; i += blockDim.x) {
        const unsigned c = i % 3u, p = i / 3u;
        const unsigned k = (p / st) % n, p0 = p - k * st;
        float acc = 0.f;
        for (unsigned m = 0; m < n; ++m) acc = fmaf(__ldg(T + k * n + m), in[3 * (p0 + m * st) + c], acc);
        out[i] = scale ? acc * __ldg(Dinv + p) : acc;
      }
      __syncthreads();
    };
    pass(E, R, Sx, nxi, 1, false);
    pass(R, E, Sy, nyi, nxi, false);
    pass(E, R, Sz, nzi, nxi * nyi, true);
    pass(R, E, Sz, nzi, nxi * nyi, false);
    pass(E, R, Sy, nyi, nxi, false);
    // last pass along x writes e in full layout (interior), zero on the boundary
    for (unsigned i = threadIdx.x; i < 3 * (unsigned)g.points(); i += blockDim.x) {
      const unsigned c = i % 3u, k = i / 3u;
      const unsigned x = k % g.np[0], q = k / g.np[0], y = q % g.np[1], z = q / g.np[1];
      float v = 0.f;
      if (x > 0 && y > 0 && z > 0 && x + 1 < g.np[0] && y + 1 < g.np[1] && z + 1 < g.np[2]) {
        const unsigned kx = x - 1, p0 = nxi * ((y - 1) + nyi * (z - 1));
        for (unsigned m = 0; m < nxi; ++m) v = fmaf(__ldg(Sx + kx * nxi + m), R[3 * (p0 + m) + c], v);
      }
      E[i] = v;
    }
    __syncthreads();
  } else {  // coarsest grid: FP64 red-black Gauss-Seidel from zero
    const int l = S.n - 1;
    const Geom& g = S.g[l];
    const size_t n = g.points();
    const double cx = 1.0 / ((double)g.cell[0] * g.cell[0]), cy = 1.0 / ((double)g.cell[1] * g.cell[1]),
                 cz = 1.0 / ((double)g.cell[2] * g.cell[2]);
    const double H = 0.5 / (cx + cy + cz);
    const size_t sy = g.np[0], sz = (size_t)g.np[0] * g.np[1];
    const float* r = sm_r(sm, S, l);
    __shared__ double s_work[kCoarseShared];
    if (3 * n <= kCoarseShared) work = s_work;  // the usual 3^3..7^3 coarsest grids
    for (size_t k = threadIdx.x; k < 3 * n; k += blockDim.x) work[k] = 0.0;
    __syncthreads();
    for (int it = 0; it < S.coarse_sweeps; ++it)
      for (unsigned color = 0; color < 2; ++color) {
        const unsigned sh = S.shc[l], items = row_items(S, l, sh);
        for (unsigned t = threadIdx.x; t < items; t += blockDim.x) {
          unsigned j, y, z;
          row_item(S, l, sh, t, j, y, z);
          const unsigned x = 1u + ((color + 1u + y + z) & 1u) + 2u * j;
          if (x + 1 >= g.np[0]) continue;
          const size_t k = x + (size_t)g.np[0] * (y + (size_t)g.np[1] * z);
          for (int c = 0; c < 3; ++c) {
            const double sv = (work[3 * (k + 1) + c] + work[3 * (k - 1) + c]) * cx +
                              (work[3 * (k + sy) + c] + work[3 * (k - sy) + c]) * cy +
                              (work[3 * (k + sz) + c] + work[3 * (k - sz) + c]) * cz;
            work[3 * k + c] = (sv - (double)r[3 * k + c]) * H;
          }
        }
        __syncthreads();
      }
    float* e = sm_e(sm, S, l);
    for (size_t k = threadIdx.x; k < 3 * n; k += blockDim.x) e[k] = (float)work[k];
    __syncthreads();
  }
  for (int l = S.n - 2; l >= 0; --l) {
    const Geom& F = S.g[l];
    {
      const unsigned sh = S.sha[l], items = row_items(S, l, sh);
      for (unsigned t = threadIdx.x; t < items; t += blockDim.x) {
        unsigned j, y, z;
        row_item(S, l, sh, t, j, y, z);
        if (j + 2 >= F.np[0]) continue;
        prolong_point(F, S.g[l + 1], sm_e(sm, S, l + 1), sm_e(sm, S, l), 1 + j, y, z);
      }
    }
    __syncthreads();
    for (int s = 0; s < S.post; ++s) {
      block_rb_sweep(sm, S, l, 0, false);
      block_rb_sweep(sm, S, l, 1, false);
    }
  }
  const size_t n0 = 3 * S.g[0].points();
  const float* e0 = sm_e(sm, S, 0);
  for (size_t k = threadIdx.x; k < n0; k += blockDim.x) S.e_out[k] = e0[k];
}


}  // namespace

__global__ void k_add_f32(float* __restrict__ a, const float* __restrict__ e, size_t n) {
  pdl_entry();
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) a[k] += e[k];
}

// a += e as float4 over the first n4 groups of 4 (both arrays 16-byte
// aligned), the n - 4 n4 remaining floats one by one.
__global__ void k_add_f32x4(float* __restrict__ a, const float* __restrict__ e, size_t n4, size_t n) {
  pdl_entry();
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n4) {
    float4 va = reinterpret_cast<float4*>(a)[k];
    const float4 ve = reinterpret_cast<const float4*>(e)[k];
    va.x += ve.x;
    va.y += ve.y;
    va.z += ve.z;
    va.w += ve.w;
    reinterpret_cast<float4*>(a)[k] = va;
  } else if (k - n4 < n - 4 * n4) {
    a[4 * n4 + (k - n4)] += e[4 * n4 + (k - n4)];
  }
}

// a[0, n) += e[0, n) on the stream (vectorised when both are 16-byte aligned).
static void add_f32(Ctx* c, float* a, const float* e, size_t n) {
  if ((((uintptr_t)a | (uintptr_t)e) & 15) == 0) {
    const size_t n4 = n / 4;
    pdl_launch(c->stream, blocks_for(n4 + 3, 256), 256, 0, k_add_f32x4, a, e, n4, n);
  } else {
    pdl_launch(c->stream, blocks_for(n, 256), 256, 0, k_add_f32, a, e, n);
  }
}

// The exact coarsest solve of k_vcycle_small as passes over the whole GPU,
// for a coarsest level of up to kDirectGlobalMax interior points: gather r
// into compact order (3 (x + nx' (y + ny' z)) + c), five sine-transform passes
// (the third scaled by 1 / eigenvalue), and the last x pass writing e in
// full layout (zero on the boundary).  Same operations as the CTA form.  T is
// the arithmetic of the transform (float, or double for the FP64 coarsest
// solve, whose tables and intermediate fields are double).
__device__ __forceinline__ float fma_t(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fma_t(double a, double b, double c) { return fma(a, b, c); }

template <typename T>
__global__ void __launch_bounds__(256) k_dst_gather(Geom g, const float* __restrict__ rfull, T* __restrict__ X) {
  pdl_entry();
  const unsigned nxi = g.np[0] - 2, nyi = g.np[1] - 2, N = nxi * nyi * (g.np[2] - 2);
  const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * N) return;
  const unsigned c = i % 3u, p = i / 3u;
  const unsigned x = p % nxi, q = p / nxi, y = q % nyi, z = q / nyi;
  X[i] = (T)rfull[3 * ((x + 1) + g.np[0] * ((y + 1) + g.np[1] * (z + 1))) + c];
}

template <typename T>
__global__ void __launch_bounds__(256) k_dst_pass(unsigned N, const T* __restrict__ in, T* __restrict__ out,
                                                  const T* __restrict__ Tab, unsigned n, unsigned st,
                                                  const T* __restrict__ Dinv) {
  pdl_entry();
  const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * N) return;
  const unsigned c = i % 3u, p = i / 3u;
  const unsigned k = (p / st) % n, p0 = p - k * st;
  T acc = 0;
  for (unsigned m = 0; m < n; ++m) acc = fma_t(__ldg(Tab + k * n + m), in[3 * (p0 + m * st) + c], acc);
  out[i] = Dinv ? acc * __ldg(Dinv + p) : acc;
}

constexpr unsigned kDstThreads = 1024;  // threads of the plane and column kernels

// The x and y passes of one (z, component) plane of the interior in shared
// memory, reading r in full layout: the same sums in the same order as
// k_dst_gather followed by k_dst_pass along x and along y.  A CTA per plane;
// dynamic shared memory: two planes of nxi x nyi values and the x table
// transposed (so that a warp's threads, on consecutive k, read consecutive
// words).
template <typename T>
__global__ void __launch_bounds__(kDstThreads) k_dst_xy(Geom g, const float* __restrict__ rfull, T* __restrict__ out,
                                                        const T* __restrict__ Sx, const T* __restrict__ Sy) {
  pdl_entry();
  extern __shared__ __align__(16) unsigned char plane_raw[];
  const unsigned nxi = g.np[0] - 2, nyi = g.np[1] - 2, np = nxi * nyi;
  T* a = reinterpret_cast<T*>(plane_raw);  // [y][m]: r
  T* b = a + np;                            // [y][k]: after the x pass
  T* sxt = b + np;                          // [m][k]: Sx transposed
  const unsigned z = blockIdx.x, c = blockIdx.y;
  for (unsigned it = threadIdx.x; it < np; it += blockDim.x) {
    const unsigned x = it % nxi, y = it / nxi;
    a[it] = (T)rfull[3 * ((x + 1) + g.np[0] * ((y + 1) + g.np[1] * (z + 1))) + c];
  }
  for (unsigned it = threadIdx.x; it < nxi * nxi; it += blockDim.x) sxt[(it % nxi) * nxi + it / nxi] = __ldg(Sx + it);
  __syncthreads();
  for (unsigned it = threadIdx.x; it < np; it += blockDim.x) {
    const unsigned k = it % nxi, y = it / nxi;
    T acc = 0;
    for (unsigned m = 0; m < nxi; ++m) acc = fma_t(sxt[m * nxi + k], a[y * nxi + m], acc);
    b[it] = acc;
  }
  __syncthreads();
  for (unsigned it = threadIdx.x; it < np; it += blockDim.x) {
    const unsigned x = it % nxi, k = it / nxi;
    T acc = 0;
    for (unsigned m = 0; m < nyi; ++m) acc = fma_t(__ldg(Sy + k * nyi + m), b[m * nxi + x], acc);
    out[3 * (it + np * z) + c] = acc;
  }
}

// The two z passes around the eigenvalue scaling, fused: a CTA owns whole z
// columns (32 x's, one y, one component), stages them in shared memory, keeps
// the first pass's results there and runs the second from them -- the same
// sums as two k_dst_pass launches.  Dynamic shared memory: 2 nzi x 32 values.
template <typename T>
__global__ void __launch_bounds__(kDstThreads) k_dst_zz(unsigned nxi, unsigned nyi, unsigned nzi, const T* __restrict__ in,
                                                T* __restrict__ out, const T* __restrict__ Sz,
                                                const T* __restrict__ Dinv) {
  pdl_entry();
  extern __shared__ __align__(16) unsigned char col_raw[];
  T* src = reinterpret_cast<T*>(col_raw);  // [m][x - x0]: the input columns
  T* col = src + nzi * 32;                  // [z][x - x0]: after the scaled first pass
  const unsigned x0 = blockIdx.x * 32, y = blockIdx.y, c = blockIdx.z, st = nxi * nyi;
  for (unsigned it = threadIdx.x; it < nzi * 32; it += blockDim.x) {
    const unsigned xl = it % 32, m = it / 32, x = x0 + xl;
    if (x < nxi) src[it] = in[3 * (x + nxi * y + m * st) + c];
  }
  __syncthreads();
  for (unsigned it = threadIdx.x; it < nzi * 32; it += blockDim.x) {
    const unsigned xl = it % 32, z = it / 32, x = x0 + xl;
    if (x >= nxi) continue;
    const unsigned p0 = x + nxi * y;
    T acc = 0;
    for (unsigned m = 0; m < nzi; ++m) acc = fma_t(__ldg(Sz + z * nzi + m), src[m * 32 + xl], acc);
    col[z * 32 + xl] = acc * __ldg(Dinv + p0 + z * st);
  }
  __syncthreads();
  for (unsigned it = threadIdx.x; it < nzi * 32; it += blockDim.x) {
    const unsigned xl = it % 32, z = it / 32, x = x0 + xl;
    if (x >= nxi) continue;
    T acc = 0;
    for (unsigned m = 0; m < nzi; ++m) acc = fma_t(__ldg(Sz + z * nzi + m), col[m * 32 + xl], acc);
    out[3 * (x + nxi * y + z * st) + c] = acc;
  }
}

// The inverse y and x passes of one (z, component) plane, writing e in full
// layout (zero on the boundary, whole boundary planes included): the same
// sums as k_dst_pass along y followed by k_dst_scatter.  A CTA per plane of
// the full grid; dynamic shared memory: two planes of nxi x nyi values and
// the x table transposed.
template <typename T>
__global__ void __launch_bounds__(kDstThreads) k_dst_yx(Geom g, const T* __restrict__ in, const T* __restrict__ Sx,
                                                        const T* __restrict__ Sy, float* __restrict__ efull) {
  pdl_entry();
  extern __shared__ __align__(16) unsigned char plane_raw[];
  const unsigned nx = g.np[0], ny = g.np[1], nxi = nx - 2, nyi = ny - 2, np = nxi * nyi;
  const unsigned z = blockIdx.x, c = blockIdx.y;
  float* ep = efull + 3 * (size_t)nx * ny * z + c;
  if (z == 0 || z + 1 >= g.np[2]) {
    for (unsigned it = threadIdx.x; it < nx * ny; it += blockDim.x) ep[3 * it] = 0.f;
    return;
  }
  T* a = reinterpret_cast<T*>(plane_raw);  // [m][x]: the plane
  T* b = a + np;                            // [y][x]: after the y pass
  T* sxt = b + np;                          // [m][k]: Sx transposed
  const unsigned zi = z - 1;
  for (unsigned it = threadIdx.x; it < np; it += blockDim.x) a[it] = in[3 * (it + np * zi) + c];
  for (unsigned it = threadIdx.x; it < nxi * nxi; it += blockDim.x) sxt[(it % nxi) * nxi + it / nxi] = __ldg(Sx + it);
  __syncthreads();
  for (unsigned it = threadIdx.x; it < np; it += blockDim.x) {
    const unsigned x = it % nxi, k = it / nxi;
    T acc = 0;
    for (unsigned m = 0; m < nyi; ++m) acc = fma_t(__ldg(Sy + k * nyi + m), a[m * nxi + x], acc);
    b[it] = acc;
  }
  __syncthreads();
  for (unsigned it = threadIdx.x; it < nx * ny; it += blockDim.x) {
    const unsigned x = it % nx, y = it / nx;
    T v = 0;
    if (x > 0 && y > 0 && x + 1 < nx && y + 1 < ny) {
      const unsigned kx = x - 1, row = nxi * (y - 1);
      for (unsigned m = 0; m < nxi; ++m) v = fma_t(sxt[m * nxi + kx], b[row + m], v);
    }
    ep[3 * it] = (float)v;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_dst_scatter(Geom g, const T* __restrict__ Y, const T* __restrict__ Sx,
                                                     float* __restrict__ efull) {
  pdl_entry();
  const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * (unsigned)g.points()) return;
  const unsigned nxi = g.np[0] - 2, nyi = g.np[1] - 2;
  const unsigned c = i % 3u, k = i / 3u;
  const unsigned x = k % g.np[0], q = k / g.np[0], y = q % g.np[1], z = q / g.np[1];
  T v = 0;
  if (x > 0 && y > 0 && z > 0 && x + 1 < g.np[0] && y + 1 < g.np[1] && z + 1 < g.np[2]) {
    const unsigned kx = x - 1, p0 = nxi * ((y - 1) + nyi * (z - 1));
    for (unsigned m = 0; m < nxi; ++m) v = fma_t(__ldg(Sx + kx * nxi + m), Y[3 * (p0 + m) + c], v);
  }
  efull[i] = (float)v;
}

// Shared memory of the plane and column kernels above (their attribute is
// raised to this once); larger coarsest levels take the pass-per-axis form.
constexpr size_t kDstSmemMax = 96 * 1024;

struct MgPlan {
  int nlev;
  Lev lev[kMaxLayers];
  size_t total;
  int first_small;    // first level run by k_vcycle_small
  size_t small_smem;  // its dynamic shared memory (bytes)
  bool direct;        // the coarsest level is solved exactly (sine transforms)
  bool direct_global;  // ... by kernels over the whole GPU instead of in the small-level CTA
};

static MgPlan plan_levels(const Geom& g) {
  MgPlan P;
  P.nlev = 0;
  Geom cur = g;
  size_t total = 0;
  for (;;) {
    Lev L;
    L.g = cur;
    const float rs[3] = {1.0f / cur.cell[0], 1.0f / cur.cell[1], 1.0f / cur.cell[2]};
    L.r2x = rs[0] * rs[0];
    L.r2y = rs[1] * rs[1];
    L.r2z = rs[2] * rs[2];
    L.H = 0.5f / (L.r2x + L.r2y + L.r2z);
    L.base = total;
    total += cur.points();
    P.lev[P.nlev++] = L;
    bool can = P.nlev < kMaxLayers;
    // coarsen while every axis keeps an even cell count and at least 2 cells
    for (int a = 0; a < 3; ++a) can = can && ((cur.np[a] - 1) % 2 == 0) && cur.np[a] >= 5;
    if (!can) break;
    cur = decimate(cur, 2);
  }
  // Stop at the finest level with at most kDirectMax interior points and solve
  // it exactly there by sine transforms: the levels below it would cost a
  // V-cycle of short barrier-bound phases.
  P.direct = P.direct_global = false;
  for (int l = 0; l < P.nlev; ++l) {
    const Geom& lg = P.lev[l].g;
    const size_t interior = (size_t)(lg.np[0] - 2) * (lg.np[1] - 2) * (lg.np[2] - 2);
    if (interior <= kDirectGlobalMax) {
      P.nlev = l + 1;
      P.direct = true;
      // a few thousand interior points: seven passes over the GPU cost less
      // than the single-CTA V-cycle (or transform) of that level
      P.direct_global = interior > kDirectMax;
      break;
    }
  }
  total = 0;
  for (int l = 0; l < P.nlev; ++l) total += P.lev[l].g.points();
  P.total = total;
  int fs = P.nlev - 1;  // the coarsest level runs in the CTA kernel (or the global transform)
  if (!P.direct_global)
    while (fs > 1 && P.lev[fs - 1].g.points() <= kSmallLevelPoints && P.nlev - (fs - 1) <= kSmallMax) --fs;
  if (P.nlev == 1) fs = 0;
  P.first_small = fs;
  size_t floats = 0;
  if (!P.direct_global)
    for (int l = fs; l < P.nlev; ++l) floats += 6 * P.lev[l].g.points();
  P.small_smem = floats * sizeof(float);
  return P;
}

struct MgBufs {
  float* E;
  float* R;
  float* lo;  // refinement: corrections accumulated on top of the FP32 iterate
  double* part;
  double* sums;
  double* cwork;
  const void* dst;  // the coarsest level's sine-transform tables when P.direct (float, or double with dst64)
  bool dst64;       // FP64 coarsest solve: double tables, and double ping-pong fields d64a, d64b (3 N each)
  double* d64a;
  double* d64b;
  unsigned nb0;  // residual blocks (partial sums)
  ResLaunch rl;   // the residual kernels' launch over level 0
};

// One V(pre, post)-cycle on L e = R[level 0] (level 0's e and r in B; e
// starts from zero).
static vg_status enqueue_vcycle(Ctx* c, const MgPlan& P, const MgBufs& B, unsigned* nl) {
  const int pre = 2, post = 2;
  const int fs = P.first_small;
  for (int l = 0; l < fs; ++l) {
    const Lev& L = P.lev[l];
    float* e = B.E + 3 * L.base;
    float* r = B.R + 3 * L.base;
    const RowLaunch sw = launch_rows(3 * ((L.g.np[0] - 1) / 2), L.g.np[1], L.g.np[2]);  // one colour's points
    const RowLaunch all = launch_rows(3 * (L.g.np[0] - 2), L.g.np[1], L.g.np[2]);     // every interior point
    pdl_launch(c->stream, all.grid, all.block, 0, k_rbgs_first, L.g, L.r2x, L.r2y, L.r2z, L.H, e, r);
    ++*nl;
    for (int s = 1; s < pre; ++s)
      for (unsigned col = 0; col < 2; ++col) {
        pdl_launch(c->stream, sw.grid, sw.block, 0, k_rbgs, L.g, L.r2x, L.r2y, L.r2z, L.H, e, r, col, 0);
        ++*nl;
      }
    const Lev& Cn = P.lev[l + 1];
    const dim3 rg((Cn.g.np[0] - 2 + kRTX - 1) / kRTX, (Cn.g.np[1] - 2 + kRTY - 1) / kRTY,
                  (Cn.g.np[2] - 2 + kRTZ - 1) / kRTZ);
    pdl_launch(c->stream, rg, 256, 0, k_residual_restrict, L.g, Cn.g, L.r2x, L.r2y, L.r2z, e, r, B.R + 3 * Cn.base);
    ++*nl;
  }
  if (P.direct_global) {
    const Lev& L = P.lev[fs];
    const Geom& g = L.g;
    const unsigned nxi = g.np[0] - 2, nyi = g.np[1] - 2, nzi = g.np[2] - 2, N = nxi * nyi * nzi;
    float* E = B.E + 3 * L.base;  // ping-pong buffers in compact layout (3 N <= 3 points)
    float* R = B.R + 3 * L.base;
    const unsigned nb = blocks_for(3 * N, 256);
    auto transform = [&](auto* X, auto* Y, auto* tab) {
      using T = typename std::remove_const<typename std::remove_pointer<decltype(tab)>::type>::type;
      const T* Sx = tab;
      const T* Sy = Sx + nxi * nxi;
      const T* Sz = Sy + nyi * nyi;
      const T* Dinv = Sz + nzi * nzi;
      const size_t plane_smem = (2 * (size_t)nxi * nyi + (size_t)nxi * nxi) * sizeof(T);
      const size_t col_smem = 2 * (size_t)nzi * 32 * sizeof(T);
      if (plane_smem <= kDstSmemMax && col_smem <= kDstSmemMax) {
        // x and y passes per plane from r (full layout) -> X, z (scaled) z -> Y, y and x per plane -> e (full)
        pdl_launch(c->stream, dim3(nzi, 3), kDstThreads, plane_smem, k_dst_xy<T>, g, (const float*)R, X, Sx, Sy);
        pdl_launch(c->stream, dim3((nxi + 31) / 32, nyi, 3), kDstThreads, col_smem, k_dst_zz<T>, nxi, nyi, nzi,
                   (const T*)X, Y, Sz, Dinv);
        pdl_launch(c->stream, dim3(g.np[2], 3), kDstThreads, plane_smem, k_dst_yx<T>, g, (const T*)Y, Sx, Sy, E);
        *nl += 3;
        return;
      } else {
        pdl_launch(c->stream, nb, 256, 0, k_dst_gather<T>, g, (const float*)R, X);
        pdl_launch(c->stream, nb, 256, 0, k_dst_pass<T>, N, (const T*)X, Y, Sx, nxi, 1u, (const T*)nullptr);
        pdl_launch(c->stream, nb, 256, 0, k_dst_pass<T>, N, (const T*)Y, X, Sy, nyi, nxi, (const T*)nullptr);
        pdl_launch(c->stream, nb, 256, 0, k_dst_pass<T>, N, (const T*)X, Y, Sz, nzi, nxi * nyi, Dinv);
        pdl_launch(c->stream, nb, 256, 0, k_dst_pass<T>, N, (const T*)Y, X, Sz, nzi, nxi * nyi, (const T*)nullptr);
        pdl_launch(c->stream, nb, 256, 0, k_dst_pass<T>, N, (const T*)X, Y, Sy, nyi, nxi, (const T*)nullptr);
        *nl += 6;
      }
      pdl_launch(c->stream, blocks_for(3 * g.points(), 256), 256, 0, k_dst_scatter<T>, g, (const T*)Y, Sx, E);
      ++*nl;
    };
    if (B.dst64)
      transform(B.d64a, B.d64b, (const double*)B.dst);
    else
      transform(E, R, (const float*)B.dst);
  } else {
    SmallLevels S;
    S.n = P.nlev - fs;
    unsigned off = 0;
    for (int i = 0; i < S.n; ++i) {
      const Lev& L = P.lev[fs + i];
      S.g[i] = L.g;
      S.r2x[i] = L.r2x;
      S.r2y[i] = L.r2y;
      S.r2z[i] = L.r2z;
      S.H[i] = L.H;
      S.off[i] = off;
      unsigned shc = 0, sha = 0;
      while ((1u << shc) < (L.g.np[0] - 1) / 2) ++shc;
      while ((1u << sha) < L.g.np[0] - 2) ++sha;
      S.shc[i] = shc;
      S.sha[i] = sha;
      S.inv_nyi[i] = 1.0f / (float)(L.g.np[1] - 2);
      off += (unsigned)(6 * L.g.points());
    }
    S.dst = P.direct ? (const float*)B.dst : nullptr;
    S.r_in = B.R + 3 * P.lev[fs].base;
    S.e_out = B.E + 3 * P.lev[fs].base;
    S.pre = pre;
    S.post = post;
    const Geom& cg = P.lev[P.nlev - 1].g;
    // Gauss-Seidel on m interior points per axis contracts by about
    // cos^2(pi / (m + 1)) per sweep; 3 (m + 1)^2 sweeps reach ~1e-13.
    const unsigned m = std::max(cg.np[0], std::max(cg.np[1], cg.np[2])) - 2;
    // one interior point: a single sweep solves it exactly
    S.coarse_sweeps = m == 1 ? 1 : (int)std::min(3u * m * m + 2u, 4000u);
    pdl_launch(c->stream, 1, 1024, P.small_smem, k_vcycle_small, S, B.cwork);
    ++*nl;
  }
  for (int l = fs - 1; l >= 0; --l) {
    const Lev& L = P.lev[l];
    const Lev& Cn = P.lev[l + 1];
    float* e = B.E + 3 * L.base;
    float* r = B.R + 3 * L.base;
    const RowLaunch sw = launch_rows(3 * ((L.g.np[0] - 1) / 2), L.g.np[1], L.g.np[2]);
    // large levels through the shared-memory tile; small ones (few CTAs per
    // tile) one thread per cell with direct updates, which measured faster there
    if (Cn.g.points() >= (size_t)1 << 18) {
      const dim3 pg((Cn.g.np[0] - 1 + 31) / 32, (Cn.g.np[1] - 1 + 3) / 4, (Cn.g.np[2] - 1 + 1) / 2);
      pdl_launch(c->stream, pg, dim3(32, 4, 2), 0, k_prolong_add<32, 4, 2>, L.g, Cn.g, B.E + 3 * Cn.base, e);
    } else {
      const unsigned cells_x = Cn.g.np[0] - 1, pbx = cells_x >= 64 ? 64 : 32, pby = 256 / pbx;
      const dim3 pg((cells_x + pbx - 1) / pbx, (Cn.g.np[1] - 1 + pby - 1) / pby, Cn.g.np[2] - 1);
      pdl_launch(c->stream, pg, dim3(pbx, pby), 0, k_prolong_cells, L.g, Cn.g, B.E + 3 * Cn.base, e);
    }
    ++*nl;
    for (int s = 0; s < post; ++s)
      for (unsigned col = 0; col < 2; ++col) {
        pdl_launch(c->stream, sw.grid, sw.block, 0, k_rbgs, L.g, L.r2x, L.r2y, L.r2z, L.H, e, r, col, 0);
        ++*nl;
      }
  }
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

// One cycle on L x = rhs: V-cycle on the current residual R, x += e, then
// R = rhs - L x in FP32 with its FP64-accumulated norm.
// Cycle tails: the residual with its norm (the adaptive solve reads it), the
// residual alone (a fixed schedule's next cycle needs R, not its norm), or
// nothing (a fixed schedule's last cycle of a phase: the next step replaces R).
enum CycleTail { TAIL_NORM, TAIL_RESIDUAL, TAIL_NONE };

static vg_status enqueue_cycle(Ctx* c, const MgPlan& P, const Geom& g, const MgBufs& B, float* x, const float* rhs,
                               unsigned* nl, CycleTail tail = TAIL_NORM) {
  vg_status st = enqueue_vcycle(c, P, B, nl);
  if (st != VG_OK) return st;
  const size_t n3 = 3 * g.points();
  const Lev& L0 = P.lev[0];
  // x += e as a separate streaming pass: fused into the last half sweep it
  // measured slower (x is not in L2 by then, and the sweep's gathers wait on it).
  // x NULL: the correction stays in B.E (level 0) for the caller.
  if (x) {
    add_f32(c, x, B.E, n3);
    ++*nl;
  }
  if (tail != TAIL_NONE) {
    pdl_launch(c->stream, B.rl.grid, B.rl.block, 0, k_residual32n, g, L0.r2x, L0.r2y, L0.r2z, B.rl.zs, x, rhs, B.R, B.part);
    ++*nl;
  }
  if (tail == TAIL_NORM) {
    pdl_launch(c->stream, 1, 1024, 0, k_sum_partials, B.part, (int)B.nb0, B.sums, 1);
    ++*nl;
  }
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

// Capture (or reuse) the cycle graph for (x, rhs) in cache slot `slot`.
static void cycle_graph(Ctx* c, const MgPlan& P, const Geom& g, const MgBufs& B, float* x, const float* rhs,
                        int slot) {
  MgGraphCache& G = c->mg_graph[slot];
  const void* key[4] = {B.E, B.R, rhs, x};
  if (G.exec && memcmp(&G.g, &g, sizeof(Geom)) == 0 && memcmp(G.key, key, sizeof(key)) == 0) return;
  if (G.exec) {
    cudaGraphExecDestroy(G.exec);
    G.exec = nullptr;
  }
  cudaGraph_t graph = nullptr;
  unsigned nl = 0;
  if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
    const vg_status cst = enqueue_cycle(c, P, g, B, x, rhs, &nl);
    const cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
    if (cst == VG_OK && ce == cudaSuccess && graph && cudaGraphInstantiate(&G.exec, graph, 0) == cudaSuccess) {
      G.g = g;
      memcpy(G.key, key, sizeof(key));
      G.launches = nl;
    } else {
      G.exec = nullptr;
    }
    if (graph) cudaGraphDestroy(graph);
  }
  cudaGetLastError();  // capture unavailable (e.g. the legacy stream): launch directly instead
}

static vg_status run_cycle(Ctx* c, const MgPlan& P, const Geom& g, const MgBufs& B, float* x, const float* rhs,
                           int slot) {
  cycle_graph(c, P, g, B, x, rhs, slot);
  MgGraphCache& G = c->mg_graph[slot];
  if (G.exec) {
    VG_CUDA(c, cudaGraphLaunch(G.exec, c->stream));
    c->launches += G.launches;
    return VG_OK;
  }
  unsigned nl = 0;
  const vg_status st = enqueue_cycle(c, P, g, B, x, rhs, &nl);
  c->launches += nl;
  return st;
}

static vg_status read_norm(Ctx* c, const MgBufs& B, double* rr, double* bb) {
  double h[2];
  VG_CUDA(c, cudaMemcpyAsync(h, B.sums, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  VG_CUDA(c, cudaStreamSynchronize(c->stream));
  *rr = h[0];
  if (bb) *bb = h[1];
  if (!(h[0] == h[0])) return fail(c, VG_NONFINITE, "multigrid: non-finite residual");
  return VG_OK;
}

// Tables of the exact coarsest-level solve: per axis the orthonormal DST-I
// matrix S[k][m] = sqrt(2 / (n + 1)) sin(pi (m + 1) (k + 1) / (n + 1)) of its
// n interior points, then 1 / eigenvalue of L for every transformed point,
// eig = -(r2x lx + r2y ly + r2z lz) with l(k) = 2 - 2 cos(pi (k + 1) / (n + 1))
// (FP64 on the host, stored as FP32).  Uploaded when the level's shape or
// spacing changes; never during stream capture, which the calibrated
// schedules guarantee by running the same grid uncaptured first.
static vg_status direct_tables(Ctx* c, const Geom& lg, bool fp64, const void** out, double** d64a, double** d64b) {
  const double r2[3] = {1.0 / ((double)lg.cell[0] * lg.cell[0]), 1.0 / ((double)lg.cell[1] * lg.cell[1]),
                        1.0 / ((double)lg.cell[2] * lg.cell[2])};
  const unsigned n[3] = {lg.np[0] - 2, lg.np[1] - 2, lg.np[2] - 2};
  const size_t N = (size_t)n[0] * n[1] * n[2];
  const size_t count = (size_t)n[0] * n[0] + (size_t)n[1] * n[1] + (size_t)n[2] * n[2] + N;
  const size_t tab_bytes = ((count * (fp64 ? sizeof(double) : sizeof(float)) + 255) / 256) * 256;
  auto fields = [&](void* base) {
    if (!fp64) return;
    *d64a = (double*)((char*)base + tab_bytes);
    *d64b = *d64a + 3 * N;
  };
  if (c->mginv_np[0] == lg.np[0] && c->mginv_np[1] == lg.np[1] && c->mginv_np[2] == lg.np[2] &&
      c->mginv_r2[0] == r2[0] && c->mginv_r2[1] == r2[1] && c->mginv_r2[2] == r2[2] && c->mginv_fp64 == fp64 &&
      c->buf[S_MGINV].p) {
    *out = c->buf[S_MGINV].p;
    fields(c->buf[S_MGINV].p);
    return VG_OK;
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  VG_CUDA(c, cudaStreamIsCapturing(c->stream, &cap));
  if (cap != cudaStreamCaptureStatusNone)
    return fail(c, VG_INVALID, "multigrid: the coarsest-level tables are not ready (run this grid uncaptured first)");
  const double pi = 3.14159265358979323846;
  std::vector<double> h;
  std::vector<double> lam[3];
  for (int a = 0; a < 3; ++a) {
    const double f = std::sqrt(2.0 / (n[a] + 1));
    for (unsigned k = 0; k < n[a]; ++k)
      for (unsigned m = 0; m < n[a]; ++m) h.push_back(f * std::sin(pi * (m + 1) * (k + 1) / (n[a] + 1)));
    for (unsigned k = 0; k < n[a]; ++k) lam[a].push_back(2.0 - 2.0 * std::cos(pi * (k + 1) / (n[a] + 1)));
  }
  for (unsigned z = 0; z < n[2]; ++z)
    for (unsigned y = 0; y < n[1]; ++y)
      for (unsigned x = 0; x < n[0]; ++x)
        h.push_back(-1.0 / (r2[0] * lam[0][x] + r2[1] * lam[1][y] + r2[2] * lam[2][z]));
  vg_status st = VG_OK;
  void* d = ws(c, S_MGINV, tab_bytes + (fp64 ? 2 * 3 * N * sizeof(double) : 0), &st);
  if (st != VG_OK) return st;
  if (fp64) {
    VG_CUDA(c, cudaMemcpyAsync(d, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    VG_CUDA(c, cudaStreamSynchronize(c->stream));  // h is released on return
  } else {
    std::vector<float> hf(h.begin(), h.end());
    VG_CUDA(c, cudaMemcpyAsync(d, hf.data(), hf.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    VG_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  for (int a = 0; a < 3; ++a) {
    c->mginv_np[a] = lg.np[a];
    c->mginv_r2[a] = r2[a];
  }
  c->mginv_fp64 = fp64;
  *out = d;
  fields(d);
  return VG_OK;
}

// Buffers of a solve on grid g (grow-only workspace slot S_MG).
static vg_status setup_bufs(Ctx* c, const Geom& g, const MgPlan& P, MgBufs& B, float** etot, float** rir) {
  const size_t n0 = g.points();
  const ResLaunch rl = res_launch(g);
  const unsigned nb0 = rl.nb;
  const size_t coarse_pts = P.lev[P.nlev - 1].g.points();
  const size_t bytes = 2 * P.total * 3 * sizeof(float) + n0 * 3 * sizeof(double) + (size_t)nb0 * 2 * sizeof(double) +
                       4 * sizeof(double) + coarse_pts * 3 * sizeof(double) + 2 * n0 * 3 * sizeof(float) + 4096;
  if (P.small_smem > 200 * 1024) return fail(c, VG_TOO_LARGE, "multigrid: coarse levels exceed shared memory");
  vg_status st = VG_OK;
  char* mem = (char*)ws(c, S_MG, bytes, &st);
  if (st != VG_OK) return st;
  B.E = (float*)mem;
  B.R = B.E + 3 * P.total;
  B.lo = (float*)(((uintptr_t)(B.R + 3 * P.total) + 255) & ~(uintptr_t)255);
  B.part = (double*)(((uintptr_t)(B.lo + 3 * n0) + 255) & ~(uintptr_t)255);
  B.sums = B.part + 2 * (size_t)nb0;
  B.cwork = B.sums + 4;
  B.nb0 = nb0;
  B.rl = rl;
  B.dst = nullptr;
  B.dst64 = P.direct_global && c->mg_coarse_fp64;
  B.d64a = B.d64b = nullptr;
  if (P.direct && (st = direct_tables(c, P.lev[P.nlev - 1].g, B.dst64, &B.dst, &B.d64a, &B.d64b)) != VG_OK)
    return st;
  *etot = (float*)(((uintptr_t)(B.cwork + 3 * coarse_pts) + 255) & ~(uintptr_t)255);  // IR correction
  *rir = *etot + 3 * n0;                                                                 // IR right-hand side
  // kernel attributes are per device: set once for each device used
  static unsigned long long smem_set = 0;
  const unsigned long long dev_bit = 1ull << (c->cfg.device & 63);
  if (!(smem_set & dev_bit)) {
    cudaFuncSetAttribute(k_vcycle_small, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_dst_xy<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDstSmemMax);
    cudaFuncSetAttribute(k_dst_xy<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDstSmemMax);
    cudaFuncSetAttribute(k_dst_zz<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDstSmemMax);
    cudaFuncSetAttribute(k_dst_zz<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDstSmemMax);
    cudaFuncSetAttribute(k_dst_yx<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDstSmemMax);
    cudaFuncSetAttribute(k_dst_yx<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDstSmemMax);
    smem_set |= dev_bit;
  }
  return VG_OK;
}

// out = sqrt(sums[0] / sums[1]) (sums[1] = ||b||^2 from the solve's first residual)
__global__ void k_relres(const double* __restrict__ sums, double* __restrict__ out) {
  pdl_entry();
  if (threadIdx.x == 0 && blockIdx.x == 0) *out = sums[1] > 0.0 ? sqrt(sums[0] / sums[1]) : sqrt(sums[0]);
}

// The adaptive solve's steps with the cycle counts fixed in advance (k1 FP32
// cycles, then one refinement round of k2 cycles) and no host round trip; the
// relative residuals go to mg_relres_dev ([0] final, [1] initial).
// The refinement residual's operator constants: FP64 values split into float
// pairs (hi = nearest float, lo = the rest), and the cycles' FP32 operator.
static PairCoef pair_coef(const Geom& g, const Lev& L0) {
  const double r2x = 1.0 / ((double)g.cell[0] * g.cell[0]), r2y = 1.0 / ((double)g.cell[1] * g.cell[1]),
               r2z = 1.0 / ((double)g.cell[2] * g.cell[2]);
  const double d = -2.0 * (r2x + r2y + r2z);
  PairCoef cf;
  cf.xh = (float)r2x;
  cf.xl = (float)(r2x - (double)cf.xh);
  cf.yh = (float)r2y;
  cf.yl = (float)(r2y - (double)cf.yh);
  cf.zh = (float)r2z;
  cf.zl = (float)(r2z - (double)cf.zh);
  cf.dh = (float)d;
  cf.dl = (float)(d - (double)cf.dh);
  cf.r2x = L0.r2x;
  cf.r2y = L0.r2y;
  cf.r2z = L0.r2z;
  return cf;
}

vg_status run_multigrid_fixed(Ctx* c, const Geom& g, float* soln3, const float* rhs3) {
  const MgPlan P = plan_levels(g);
  MgBufs B;
  float *etot = nullptr, *rir = nullptr;
  vg_status st = setup_bufs(c, g, P, B, &etot, &rir);
  if (st != VG_OK) return st;
  if (!c->mg_relres_dev) return fail(c, VG_INVALID, "multigrid: no device slot for the residual");
  const size_t n0 = g.points();
  const unsigned nb0 = B.nb0;
  const Lev& L0 = P.lev[0];
  const PairCoef cf = pair_coef(g, L0);
  unsigned nl = 0;
  VG_CUDA(c, cudaMemsetAsync(B.E, 0, P.total * 3 * sizeof(float), c->stream));
  pdl_launch(c->stream, B.rl.grid, B.rl.block, 0, k_residual32n, g, L0.r2x, L0.r2y, L0.r2z, B.rl.zs, soln3, rhs3, B.R,
                                                         B.part);
  pdl_launch(c->stream, 1, 1024, 0, k_sum_partials, B.part, (int)nb0, B.sums, 0);
  pdl_launch(c->stream, 1, 32, 0, k_relres, B.sums, c->mg_relres_dev + 1);
  nl += 3;
  for (int k = 0; k < c->mg_fixed_k1; ++k)
    if ((st = enqueue_cycle(c, P, g, B, soln3, rhs3, &nl, k + 1 < c->mg_fixed_k1 ? TAIL_RESIDUAL : TAIL_NONE)) != VG_OK)
      return st;
  if (c->mg_fixed_k2 <= 1) {
    // No refinement cycle, or one: the general round below with its zero lo
    // and etot, its copy of the residual and its two additions collapses to
    // r = b - L soln straight into the cycle's residual, the cycle's
    // correction e left in B.E, the check of soln + e and soln += e -- the
    // same float operations on the same values (0 + e = e exactly).
    pdl_launch(c->stream, B.rl.grid, B.rl.block, 0, k_residual_pair<false>, g, cf, B.rl.zs, (const float*)soln3,
               (const float*)nullptr, rhs3, c->mg_fixed_k2 ? B.R : rir, B.part);
    pdl_launch(c->stream, 1, 1024, 0, k_sum_partials, B.part, (int)nb0, B.sums, 1);
    nl += 2;
    if (c->mg_fixed_k2 == 1) {
      if ((st = enqueue_cycle(c, P, g, B, nullptr, rhs3, &nl, TAIL_NONE)) != VG_OK) return st;
      pdl_launch(c->stream, B.rl.grid, B.rl.block, 0, k_residual_pair<true>, g, cf, B.rl.zs, (const float*)soln3,
                 (const float*)B.E, rhs3, rir, B.part);
      pdl_launch(c->stream, 1, 1024, 0, k_sum_partials, B.part, (int)nb0, B.sums, 1);
      nl += 2;
    }
    pdl_launch(c->stream, 1, 32, 0, k_relres, B.sums, c->mg_relres_dev);
    ++nl;
    if (c->mg_fixed_k2 == 1) {
      add_f32(c, soln3, B.E, 3 * n0);
      ++nl;
    }
    c->launches += nl;
    VG_CUDA(c, cudaGetLastError());
    return VG_OK;
  }
  VG_CUDA(c, cudaMemsetAsync(B.lo, 0, 3 * n0 * sizeof(float), c->stream));
  pdl_launch(c->stream, B.rl.grid, B.rl.block, 0, k_residual_pair<true>, g, cf, B.rl.zs, soln3, B.lo, rhs3, rir, B.part);
  pdl_launch(c->stream, 1, 1024, 0, k_sum_partials, B.part, (int)nb0, B.sums, 1);
  nl += 3;
  if (c->mg_fixed_k2 > 0) {
    VG_CUDA(c, cudaMemsetAsync(etot, 0, 3 * n0 * sizeof(float), c->stream));
    VG_CUDA(c, cudaMemcpyAsync(B.R, rir, 3 * n0 * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
    for (int k = 0; k < c->mg_fixed_k2; ++k)
      if ((st = enqueue_cycle(c, P, g, B, etot, rir, &nl, k + 1 < c->mg_fixed_k2 ? TAIL_RESIDUAL : TAIL_NONE)) !=
          VG_OK)
        return st;
    add_f32(c, B.lo, etot, 3 * n0);
    pdl_launch(c->stream, B.rl.grid, B.rl.block, 0, k_residual_pair<true>, g, cf, B.rl.zs, soln3, B.lo, rhs3, rir, B.part);
    pdl_launch(c->stream, 1, 1024, 0, k_sum_partials, B.part, (int)nb0, B.sums, 1);
    nl += 3;
  }
  pdl_launch(c->stream, 1, 32, 0, k_relres, B.sums, c->mg_relres_dev);
  add_f32(c, soln3, B.lo, 3 * n0);
  nl += 2;
  c->launches += nl;
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

vg_status run_multigrid(Ctx* c, const Geom& g, float* soln3, const float* rhs3, double tol, int max_cycles,
                        int* cycles_out, double* relres0_out, double* relres_out) {
  const MgPlan P = plan_levels(g);
  const size_t n0 = g.points();
  MgBufs B;
  float *etot = nullptr, *rir = nullptr;
  vg_status st = setup_bufs(c, g, P, B, &etot, &rir);
  if (st != VG_OK) return st;
  const unsigned nb0 = B.nb0;
  // e must be zero on every level's boundary (Dirichlet correction); the
  // kernels only ever write interior points.
  VG_CUDA(c, cudaMemsetAsync(B.E, 0, P.total * 3 * sizeof(float), c->stream));
  const Lev& L0 = P.lev[0];
  const PairCoef cf = pair_coef(g, L0);
  pdl_launch(c->stream, B.rl.grid, B.rl.block, 0, k_residual32n, g, L0.r2x, L0.r2y, L0.r2z, B.rl.zs, soln3, rhs3, B.R,
                                                         B.part);
  pdl_launch(c->stream, 1, 1024, 0, k_sum_partials, B.part, (int)nb0, B.sums, 0);
  c->launches += 2;
  double rr = 0.0, bnorm2 = 0.0;
  if ((st = read_norm(c, B, &rr, &bnorm2)) != VG_OK) return st;
  const double bn = bnorm2 > 0.0 ? std::sqrt(bnorm2) : 1.0;
  double relres = std::sqrt(rr) / bn;
  const double relres0 = relres;
  int cyc = 0;
  // Phase 1: FP32 cycles on the field itself while FP32 can represent the
  // residual (relative residual above 1e-4).
  const double switch_tol = std::max(tol, 1e-4);
  while (relres > switch_tol && cyc < max_cycles) {
    if ((st = run_cycle(c, P, g, B, soln3, rhs3, 0)) != VG_OK) return st;
    ++cyc;
    if ((st = read_norm(c, B, &rr, nullptr)) != VG_OK) return st;
    relres = std::sqrt(rr) / bn;
  }
  const int k1 = cyc;
  // Phase 2: iterative refinement.  The iterate is soln3 + lo (lo from zero);
  // the residual b - L (soln3 + lo) is evaluated to FP64-class accuracy by
  // k_residual_pair, FP32 cycles solve the correction equation L e = r (its
  // residual updated in FP32, accurate because r is already small), lo += e,
  // and another such residual checks.
  VG_CUDA(c, cudaMemsetAsync(B.lo, 0, 3 * n0 * sizeof(float), c->stream));
  for (;;) {
    pdl_launch(c->stream, B.rl.grid, B.rl.block, 0, k_residual_pair<true>, g, cf, B.rl.zs, soln3, B.lo, rhs3, rir, B.part);
    pdl_launch(c->stream, 1, 1024, 0, k_sum_partials, B.part, (int)nb0, B.sums, 1);
    c->launches += 2;
    if ((st = read_norm(c, B, &rr, nullptr)) != VG_OK) return st;
    relres = std::sqrt(rr) / bn;
    if (relres <= tol || cyc >= max_cycles) break;
    // The FP32 residual of the correction equation tracks the accurate residual
    // of soln3 + lo + e to ~1e-11 relative (its right-hand side is already below 1e-4),
    // so a tenth of the tolerance is margin enough for the FP64 check that follows.
    const double inner_tol = std::max(0.9 * tol, 1e-4 * relres);
    VG_CUDA(c, cudaMemsetAsync(etot, 0, 3 * n0 * sizeof(float), c->stream));
    VG_CUDA(c, cudaMemcpyAsync(B.R, rir, 3 * n0 * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
    double inner = relres;
    while (inner > inner_tol && cyc < max_cycles) {
      if ((st = run_cycle(c, P, g, B, etot, rir, 1)) != VG_OK) return st;
      ++cyc;
      if ((st = read_norm(c, B, &rr, nullptr)) != VG_OK) return st;
      inner = std::sqrt(rr) / bn;
    }
    add_f32(c, B.lo, etot, 3 * n0);
    VG_LAUNCHED(c);
  }
  add_f32(c, soln3, B.lo, 3 * n0);
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  c->mg_last_k1 = k1;
  c->mg_last_k2 = cyc - k1;
  if (cycles_out) *cycles_out = cyc;
  if (relres0_out) *relres0_out = relres0;
  if (relres_out) *relres_out = relres;
  if (relres > tol) return fail(c, VG_NOT_CONVERGED, "multigrid: cycle limit reached above tolerance");
  return VG_OK;
}

// ------------------------------------------------------- persistent batched solve
//
// Many simulations' fixed-schedule solves in one cooperative launch.  The
// CTAs form teams of T; a team takes its simulations (assigned on the host,
// longest first) one after another and runs every phase of the schedule of
// run_multigrid_fixed -- zeroing, residuals, smoothing sweeps, residual +
// restriction, sine-transform passes, prolongation, updates -- as loops over
// the team's threads, with a team barrier between phases.  The point
// arithmetic is the shared lap7 / gs_value / pair_residual code, so the
// result is bit-identical to the per-level launches; only the norm sums
// (statistics) are accumulated in another order.  Fields written during the
// launch are read with weak loads (never the non-coherent read-only path),
// which the barrier's fences order after the writes.

namespace {

constexpr int kPThreads = 512;  // threads per CTA
constexpr int kPU = 3;          // items a lane has in flight per step of the streaming phases
constexpr int kPMaxLev = 8;     // levels above and including the sine-transform solve

struct PLev {
  unsigned np[3];
  float r2x, r2y, r2z, H;
  unsigned base;  // points before this level in E and R
};

struct PSim {
  PLev lev[kPMaxLev];
  int nlev;
  int k1, k2;
  PairCoef cf;
  float *E, *R, *x, *lo, *etot, *rir;
  const float* rhs;
  const float* dst;  // coarsest level: Sx, Sy, Sz, 1 / eigenvalue (direct_tables)
  double* relres;    // [0] final, [1] initial relative residual
  double* acc;       // [0] sum r^2, [1] sum b^2
  unsigned n0;       // level-0 points
  unsigned total;    // points over all levels
};

struct Team {
  unsigned* ctr;  // arrivals at this team's barriers (cleared before the launch)
  int* err;       // set when any barrier gives up
  unsigned T, rank, target;
  unsigned long long limit_ns;  // a barrier wait gives up after this long
  __device__ unsigned tid() const { return rank * blockDim.x + threadIdx.x; }
  __device__ unsigned size() const { return T * blockDim.x; }
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

constexpr unsigned long long kBarrierNs = 2000000000ull;  // the solve's barrier waits give up after 2 s
constexpr unsigned kBarrierPolls = 1u << 26;              // ... or after this many polls

// Team barrier: each CTA's writes are fenced before it arrives, and after
// the wait, so the team's next phase sees them.  False (err set) when a wait
// gives up or another barrier already has; the caller then returns.
__device__ bool team_sync(Team& tm) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    tm.target += tm.T;
    __threadfence();
    atomicAdd(tm.ctr, 1u);
    int ok = 1;
    const unsigned long long t0 = global_ns();
    for (unsigned it = 0;; ++it) {
      if ((int)(*(volatile unsigned*)tm.ctr - tm.target) >= 0) break;
      if (*(volatile int*)tm.err) {
        ok = 0;
        break;
      }
      if (it >= kBarrierPolls || ((it & 255u) == 255u && global_ns() - t0 > tm.limit_ns)) {
        atomicExch(tm.err, 1);
        ok = 0;
        break;
      }
      if (it >= 4096) __nanosleep(64);  // long waits back off
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Loads of fields written earlier in the launch: weak loads, cached in L1
// (the stencils re-read each value up to seven times).  The team barrier's
// fences order them after the other CTAs' writes; the non-coherent read-only
// path (ld.global.nc) is never used for these fields.
__device__ __forceinline__ float ld(const float* p) { return __ldca(p); }

// Interior rows (y, z) of a level taken by the team's warps in turn; the
// lanes run along the row over `items` (point, component) pairs.
template <class F>
__device__ __forceinline__ void team_rows(const Team& tm, unsigned ny, unsigned nz, unsigned items, F f) {
  const unsigned lane = threadIdx.x & 31u, nyi = ny - 2, rows = nyi * (nz - 2);
  for (unsigned row = tm.tid() >> 5; row < rows; row += tm.size() >> 5) {
    const unsigned zz = row / nyi;
    const unsigned y = 1 + row - zz * nyi, z = 1 + zz;
    for (unsigned jc = lane; jc < items; jc += 32) f(jc, y, z);
  }
}

__device__ void warp_add2(double* a, double* b, float va, float vb) {
  for (int o = 16; o > 0; o >>= 1) {
    va += __shfl_xor_sync(0xffffffffu, va, o);
    vb += __shfl_xor_sync(0xffffffffu, vb, o);
  }
  if ((threadIdx.x & 31u) == 0) {
    if (a) atomicAdd(a, (double)va);
    if (b) atomicAdd(b, (double)vb);
  }
}

// Streaming loops, as float4 where the arrays are 16-byte aligned.
__device__ __forceinline__ bool aligned16(const void* a, const void* b) {
  return (((uintptr_t)a | (uintptr_t)b) & 15u) == 0;
}

__device__ void p_zero(const Team& tm, float* p, unsigned n) {
  const unsigned n4 = aligned16(p, p) ? n / 4 : 0;
  for (unsigned i = tm.tid(); i < n4; i += tm.size()) reinterpret_cast<float4*>(p)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  for (unsigned i = 4 * n4 + tm.tid(); i < n; i += tm.size()) p[i] = 0.f;
}

__device__ void p_add(const Team& tm, float* a, const float* e, unsigned n) {  // a += e
  const unsigned n4 = aligned16(a, e) ? n / 4 : 0;
  const unsigned step = tm.size();
  for (unsigned i = tm.tid(); i < n4; i += kPU * step) {
    float4 va[kPU], ve[kPU];
#pragma unroll
    for (int u = 0; u < kPU; ++u) {
      const unsigned q = min(i + u * step, n4 - 1);  // past the end: reload the last group, not stored
      va[u] = __ldcg(reinterpret_cast<const float4*>(a) + q);
      ve[u] = __ldcg(reinterpret_cast<const float4*>(e) + q);
    }
#pragma unroll
    for (int u = 0; u < kPU; ++u) {
      if (i + u * step >= n4) break;
      va[u].x = __fadd_rn(va[u].x, ve[u].x);
      va[u].y = __fadd_rn(va[u].y, ve[u].y);
      va[u].z = __fadd_rn(va[u].z, ve[u].z);
      va[u].w = __fadd_rn(va[u].w, ve[u].w);
      reinterpret_cast<float4*>(a)[i + u * step] = va[u];
    }
  }
  for (unsigned i = 4 * n4 + tm.tid(); i < n; i += tm.size()) a[i] = __fadd_rn(ld(a + i), ld(e + i));
}

__device__ void p_copy(const Team& tm, float* d, const float* s, unsigned n) {
  const unsigned n4 = aligned16(d, s) ? n / 4 : 0;
  for (unsigned i = tm.tid(); i < n4; i += tm.size())
    reinterpret_cast<float4*>(d)[i] = __ldcg(reinterpret_cast<const float4*>(s) + i);
  for (unsigned i = 4 * n4 + tm.tid(); i < n; i += tm.size()) d[i] = ld(s + i);
}

// The team's share of the flattened (interior row, item) space of a level:
// each warp a contiguous slice of whole warps' worth of items, each lane every
// 32nd item of it, kPU items per step.  A step first computes all kPU
// positions, then issues every load (items past the end read a safe interior
// point), then computes and stores, so each lane keeps kPU items' loads in
// flight instead of one (the stores would otherwise keep the compiler from
// hoisting the next item's loads).
struct Slice {
  unsigned t, t1;   // this lane's next item and the end of the warp's slice
  unsigned y, z, jc;  // the item's row and index within the row
};

__device__ __forceinline__ bool slice_begin(const Team& tm, unsigned ny, unsigned nz, unsigned ipr, Slice& s) {
  const unsigned nyi = ny - 2, total = nyi * (nz - 2) * ipr;
  const unsigned nw = tm.size() >> 5, w = tm.tid() >> 5;
  const unsigned chunk = ((total + nw - 1) / nw + 31u) & ~31u;
  s.t = w * chunk + (threadIdx.x & 31u);
  s.t1 = min(total, w * chunk + chunk);
  if (s.t >= s.t1) return false;
  const unsigned row = s.t / ipr;
  s.jc = s.t - row * ipr;
  s.z = 1 + row / nyi;
  s.y = 1 + row - (s.z - 1) * nyi;
  return true;
}

// The positions of this lane's next kPU items (32 apart); s moves past them.
__device__ __forceinline__ void slice_step(Slice& s, unsigned ipr, unsigned ny, unsigned (&y)[kPU],
                                           unsigned (&z)[kPU], unsigned (&jc)[kPU], bool (&in)[kPU]) {
#pragma unroll
  for (int u = 0; u < kPU; ++u) {
    y[u] = s.y;
    z[u] = s.z;
    jc[u] = s.jc;
    in[u] = s.t + 32u * u < s.t1;
    s.jc += 32u;
    while (s.jc >= ipr) {
      s.jc -= ipr;
      if (++s.y == ny - 1) {
        s.y = 1;
        ++s.z;
      }
    }
  }
  s.t += 32u * kPU;
}

// One colour's Gauss-Seidel half sweep (k_rbgs).
__device__ void p_rbgs(const Team& tm, const PLev& L, float* e, const float* r, unsigned col) {
  const unsigned nx = L.np[0], ny = L.np[1], sy = 3 * nx, sz = 3 * nx * ny;
  const unsigned ipr = 3 * ((nx - 1) / 2), safe = 3 * (1 + nx * (1 + ny));
  Slice s;
  if (!slice_begin(tm, ny, L.np[2], ipr, s)) return;
  while (s.t < s.t1) {
    unsigned y[kPU], z[kPU], jc[kPU], k[kPU];
    bool in[kPU];
    slice_step(s, ipr, ny, y, z, jc, in);
#pragma unroll
    for (int u = 0; u < kPU; ++u) {
      const unsigned j = jc[u] / 3u, c = jc[u] - 3u * j;
      const unsigned x = 1u + ((col + 1u + y[u] + z[u]) & 1u) + 2u * j;
      in[u] = in[u] && x + 1 < nx;
      k[u] = in[u] ? 3 * (x + nx * (y[u] + ny * z[u])) + c : safe;
    }
    float vx[kPU], vy[kPU], vz[kPU], vr[kPU], ve[kPU];
#pragma unroll
    for (int u = 0; u < kPU; ++u) {
      vx[u] = __fadd_rn(ld(e + k[u] + 3), ld(e + k[u] - 3));
      vy[u] = __fadd_rn(ld(e + k[u] + sy), ld(e + k[u] - sy));
      vz[u] = __fadd_rn(ld(e + k[u] + sz), ld(e + k[u] - sz));
      vr[u] = ld(r + k[u]);
      ve[u] = ld(e + k[u]);
    }
#pragma unroll
    for (int u = 0; u < kPU; ++u)
      if (in[u]) e[k[u]] = sor_value(ve[u], gs_value(vx[u], vy[u], vz[u], vr[u], L.r2x, L.r2y, L.r2z, L.H));
  }
}

// The first sweep from e = 0, both colours (k_rbgs_first).  Red items load
// their own r in place of the neighbours they do not use.
__device__ void p_rbgs_first(const Team& tm, const PLev& L, float* e, const float* r) {
  const unsigned nx = L.np[0], ny = L.np[1], nz = L.np[2], sy = 3 * nx, sz = 3 * nx * ny;
  const unsigned ipr = 3 * (nx - 2);
  const float H = L.H;
  Slice s;
  if (!slice_begin(tm, ny, nz, ipr, s)) return;
  while (s.t < s.t1) {
    unsigned y[kPU], z[kPU], jc[kPU], k[kPU];
    bool in[kPU], black[kPU];
    unsigned m[kPU];  // bit i: neighbour i (x+, x-, y+, y-, z+, z-) is a red interior point
    slice_step(s, ipr, ny, y, z, jc, in);
#pragma unroll
    for (int u = 0; u < kPU; ++u) {
      const unsigned j = jc[u] / 3u, c = jc[u] - 3u * j, x = 1u + j;
      k[u] = in[u] ? 3 * (x + nx * (y[u] + ny * z[u])) + c : 3 * (1 + nx * (1 + ny));
      black[u] = in[u] && ((x + y[u] + z[u]) & 1u);
      m[u] = black[u] ? (x + 2 < nx) | (x > 1) << 1 | (y[u] + 2 < ny) << 2 | (y[u] > 1) << 3 |
                            (z[u] + 2 < nz) << 4 | (z[u] > 1) << 5
                      : 0u;
    }
    float nb[kPU][6], vr[kPU];
#pragma unroll
    for (int u = 0; u < kPU; ++u) {
      const int off[6] = {3, -3, (int)sy, -(int)sy, (int)sz, -(int)sz};
      vr[u] = ld(r + k[u]);
#pragma unroll
      for (int i = 0; i < 6; ++i) nb[u][i] = ld(r + k[u] + ((m[u] >> i) & 1u ? off[i] : 0));
    }
#pragma unroll
    for (int u = 0; u < kPU; ++u) {
      if (!in[u]) continue;
      float v;
      if (!black[u]) {
        v = sor_value(0.f, __fmul_rn(-vr[u], H));
      } else {
        float red[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) red[i] = (m[u] >> i) & 1u ? sor_value(0.f, __fmul_rn(-nb[u][i], H)) : 0.f;
        v = sor_value(0.f, gs_value(__fadd_rn(red[0], red[1]), __fadd_rn(red[2], red[3]), __fadd_rn(red[4], red[5]),
                                    vr[u], L.r2x, L.r2y, L.r2z, H));
      }
      e[k[u]] = v;
    }
  }
}

// r = b - L a at level 0 (k_residual32n); sums of r^2 and b^2 into *arr, *abb when given.
__device__ void p_residual32(const Team& tm, const PLev& L, const float* a, const float* b, float* r, double* arr,
                             double* abb) {
  const unsigned nx = L.np[0], ny = L.np[1], sy = 3 * nx, sz = 3 * nx * ny;
  const unsigned ipr = 3 * (nx - 2);
  float rr = 0.f, bb = 0.f;
  Slice s;
  if (slice_begin(tm, ny, L.np[2], ipr, s)) {
    while (s.t < s.t1) {
      unsigned y[kPU], z[kPU], jc[kPU], k[kPU];
      bool in[kPU];
      slice_step(s, ipr, ny, y, z, jc, in);
#pragma unroll
      for (int u = 0; u < kPU; ++u) {
        const unsigned j = jc[u] / 3u, c = jc[u] - 3u * j, x = 1u + j;
        k[u] = in[u] ? 3 * (x + nx * (y[u] + ny * z[u])) + c : 3 * (1 + nx * (1 + ny));
      }
      float v[kPU][7], vb[kPU];
#pragma unroll
      for (int u = 0; u < kPU; ++u) {
        v[u][0] = ld(a + k[u]);
        v[u][1] = ld(a + k[u] + 3);
        v[u][2] = ld(a + k[u] - 3);
        v[u][3] = ld(a + k[u] + sy);
        v[u][4] = ld(a + k[u] - sy);
        v[u][5] = ld(a + k[u] + sz);
        v[u][6] = ld(a + k[u] - sz);
        vb[u] = ld(b + k[u]);
      }
#pragma unroll
      for (int u = 0; u < kPU; ++u) {
        if (!in[u]) continue;
        const float lap = lap7(v[u][0], v[u][1], v[u][2], v[u][3], v[u][4], v[u][5], v[u][6], L.r2x, L.r2y, L.r2z);
        const float rv = __fsub_rn(vb[u], lap);
        r[k[u]] = rv;
        rr = fmaf(rv, rv, rr);
        bb = fmaf(vb[u], vb[u], bb);
      }
    }
  }
  if (arr || abb) warp_add2(arr, abb, rr, bb);
}

// r = b - L (x + lo) to FP64-class accuracy (k_residual_pair); r^2 into *arr when given.
__device__ void p_residual_pair(const Team& tm, const PSim& S, float* r, double* arr) {
  const PLev& L = S.lev[0];
  const unsigned nx = L.np[0], ny = L.np[1], sy = nx, sz = nx * ny;
  float rr = 0.f;
  team_rows(tm, ny, L.np[2], 3 * (nx - 2), [&](unsigned jc, unsigned y, unsigned z) {
    const unsigned j = jc / 3u, c = jc - 3u * j, x = 1u + j;
    const unsigned k = x + nx * (y + ny * z);
    const unsigned o[7] = {k, k + 1, k - 1, k + sy, k - sy, k + sz, k - sz};
    float h[7], l[7];
#pragma unroll
    for (int i = 0; i < 7; ++i) {
      h[i] = ld(S.x + 3 * o[i] + c);
      l[i] = ld(S.lo + 3 * o[i] + c);
    }
    const float rv = pair_residual(h, l, ld(S.rhs + 3 * k + c), S.cf);
    r[3 * k + c] = rv;
    rr = fmaf(rv, rv, rr);
  });
  if (arr) warp_add2(arr, nullptr, rr, 0.f);
}

// Fused residual + full-weighting restriction (k_residual_restrict), the
// team's CTAs taking its tiles in turn.
__device__ void p_restrict(const Team& tm, const PLev& F, const PLev& C, const float* e, const float* r, float* rc,
                           float* s_res) {
  const unsigned gx = (C.np[0] - 2 + kRTX - 1) / kRTX, gy = (C.np[1] - 2 + kRTY - 1) / kRTY,
                 gz = (C.np[2] - 2 + kRTZ - 1) / kRTZ;
  const unsigned nx = F.np[0], ny = F.np[1], nz = F.np[2], sy = nx, sz = nx * ny;
  for (unsigned tile = tm.rank; tile < gx * gy * gz; tile += tm.T) {
    const unsigned bx = tile % gx, q = tile / gx, by = q % gy, bz = q / gy;
    const unsigned cx0 = 1 + bx * kRTX, cy0 = 1 + by * kRTY, cz0 = 1 + bz * kRTZ;
    for (unsigned p = threadIdx.x; p < (unsigned)(kRFX * kRFY * kRFZ); p += blockDim.x) {
      const unsigned lx = p % kRFX, qq = p / kRFX;
      const unsigned ly = qq % kRFY, lz = qq / kRFY;
      const unsigned fx = 2 * cx0 - 1 + lx, fy = 2 * cy0 - 1 + ly, fz = 2 * cz0 - 1 + lz;
      float v[3] = {0.f, 0.f, 0.f};
      if (fx + 1 < nx && fy + 1 < ny && fz + 1 < nz) {
        const unsigned o = fx + sy * fy + sz * fz;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float lap = lap7(ld(e + 3 * o + c), ld(e + 3 * (o + 1) + c), ld(e + 3 * (o - 1) + c),
                                 ld(e + 3 * (o + sy) + c), ld(e + 3 * (o - sy) + c), ld(e + 3 * (o + sz) + c),
                                 ld(e + 3 * (o - sz) + c), F.r2x, F.r2y, F.r2z);
          v[c] = __fsub_rn(ld(r + 3 * o + c), lap);
        }
      }
      s_res[3 * p] = v[0];
      s_res[3 * p + 1] = v[1];
      s_res[3 * p + 2] = v[2];
    }
    __syncthreads();
    for (unsigned i = threadIdx.x; i < (unsigned)(kRTX * kRTY * kRTZ * 3); i += blockDim.x) {
      const unsigned c = i % 3u, pp = i / 3u;
      const unsigned lx = pp % kRTX, qq = pp / kRTX;
      const unsigned ly = qq % kRTY, lz = qq / kRTY;
      const unsigned x = cx0 + lx, y = cy0 + ly, z = cz0 + lz;
      if (x + 1 >= C.np[0] || y + 1 >= C.np[1] || z + 1 >= C.np[2]) continue;
      const float* sr = s_res + 3 * ((2 * lx + 1) + kRFX * ((2 * ly + 1) + kRFY * (2 * lz + 1))) + c;
      float acc = 0.f;
#pragma unroll
      for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
        for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
          for (int dx = -1; dx <= 1; ++dx) {
            const float wt = (float)(8 >> (abs(dx) + abs(dy) + abs(dz)));
            acc = __fmaf_rn(wt, sr[3 * (dx + kRFX * (dy + kRFY * dz))], acc);
          }
      rc[3 * (x + C.np[0] * (y + C.np[1] * z)) + c] = __fmul_rn(acc, 1.0f / 64.0f);
    }
    __syncthreads();
  }
}

// e_fine += trilinear(e_coarse), one thread per coarse cell (k_prolong_cells).
__device__ void p_prolong(const Team& tm, const PLev& F, const PLev& C, const float* ec, float* ef) {
  const unsigned ncx = C.np[0] - 1, ncy = C.np[1] - 1, cells = ncx * ncy * (C.np[2] - 1);
  const unsigned sy = C.np[0], sz = C.np[0] * C.np[1], fsy = F.np[0], fsz = F.np[0] * F.np[1];
  for (unsigned i = tm.tid(); i < cells; i += tm.size()) {
    const unsigned cx = i % ncx, q = i / ncx, cy = q % ncy, cz = q / ncy;
    const unsigned c0 = cx + sy * cy + sz * cz;
    float v[2][2][2][3];
#pragma unroll
    for (int iz = 0; iz < 2; ++iz)
#pragma unroll
      for (int iy = 0; iy < 2; ++iy)
#pragma unroll
        for (int ix = 0; ix < 2; ++ix)
#pragma unroll
          for (int c = 0; c < 3; ++c) v[iz][iy][ix][c] = ld(ec + 3 * (c0 + ix + sy * iy + sz * iz) + c);
#pragma unroll
    for (int oz = 0; oz < 2; ++oz)
#pragma unroll
      for (int oy = 0; oy < 2; ++oy)
#pragma unroll
        for (int ox = 0; ox < 2; ++ox) {
          const unsigned X = 2 * cx + ox, Y = 2 * cy + oy, Z = 2 * cz + oz;
          if (X == 0 || Y == 0 || Z == 0) continue;
          const float wt = 1.0f / (float)(1u << (ox + oy + oz));
          const unsigned k = X + fsy * Y + fsz * Z;
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            float a = 0.f;
#pragma unroll
            for (int iz = 0; iz <= oz; ++iz)
#pragma unroll
              for (int iy = 0; iy <= oy; ++iy)
#pragma unroll
                for (int ix = 0; ix <= ox; ++ix) a += v[iz][iy][ix][c];
            ef[3 * k + c] = __fadd_rn(ld(ef + 3 * k + c), __fmul_rn(a, wt));
          }
        }
  }
}

// The exact coarsest solve (k_dst_gather, k_dst_pass, k_dst_scatter).
__device__ bool p_direct(Team& tm, const PSim& S) {
  const PLev& L = S.lev[S.nlev - 1];
  const unsigned nx = L.np[0], ny = L.np[1], nz = L.np[2];
  const unsigned nxi = nx - 2, nyi = ny - 2, nzi = nz - 2, N = nxi * nyi * nzi;
  float* E = S.E + 3 * L.base;
  float* R = S.R + 3 * L.base;
  const float* Sx = S.dst;
  const float* Sy = Sx + nxi * nxi;
  const float* Sz = Sy + nyi * nyi;
  const float* Dinv = Sz + nzi * nzi;
  for (unsigned i = tm.tid(); i < 3 * N; i += tm.size()) {  // R (full) -> E (compact)
    const unsigned c = i % 3u, p = i / 3u;
    const unsigned x = p % nxi, q = p / nxi, y = q % nyi, z = q / nyi;
    E[i] = ld(R + 3 * ((x + 1) + nx * ((y + 1) + ny * (z + 1))) + c);
  }
  if (!team_sync(tm)) return false;
  auto pass = [&](const float* in, float* out, const float* T, unsigned n, unsigned st, const float* scale) {
    for (unsigned i = tm.tid(); i < 3 * N; i += tm.size()) {
      const unsigned c = i % 3u, p = i / 3u;
      const unsigned k = (p / st) % n, p0 = p - k * st;
      float acc = 0.f;
      for (unsigned m = 0; m < n; ++m) acc = fmaf(__ldg(T + k * n + m), ld(in + 3 * (p0 + m * st) + c), acc);
      out[i] = scale ? acc * __ldg(scale + p) : acc;
    }
    return team_sync(tm);
  };
  if (!pass(E, R, Sx, nxi, 1, nullptr) || !pass(R, E, Sy, nyi, nxi, nullptr) ||
      !pass(E, R, Sz, nzi, nxi * nyi, Dinv) || !pass(R, E, Sz, nzi, nxi * nyi, nullptr) ||
      !pass(E, R, Sy, nyi, nxi, nullptr))
    return false;
  const unsigned pts = nx * ny * nz;
  for (unsigned i = tm.tid(); i < 3 * pts; i += tm.size()) {  // x pass into e (full layout)
    const unsigned c = i % 3u, k = i / 3u;
    const unsigned x = k % nx, q = k / nx, y = q % ny, z = q / ny;
    float v = 0.f;
    if (x > 0 && y > 0 && z > 0 && x + 1 < nx && y + 1 < ny && z + 1 < nz) {
      const unsigned kx = x - 1, p0 = nxi * ((y - 1) + nyi * (z - 1));
      for (unsigned m = 0; m < nxi; ++m) v = fmaf(__ldg(Sx + kx * nxi + m), ld(R + 3 * (p0 + m) + c), v);
    }
    E[i] = v;
  }
  return team_sync(tm);
}

// One V(2,2)-cycle on L e = R[level 0] (enqueue_vcycle).
__device__ bool p_vcycle(Team& tm, const PSim& S, float* s_res) {
  const int nl = S.nlev;
  for (int l = 0; l + 1 < nl; ++l) {
    const PLev& L = S.lev[l];
    float* e = S.E + 3 * L.base;
    const float* r = S.R + 3 * L.base;
    p_rbgs_first(tm, L, e, r);
    if (!team_sync(tm)) return false;
    for (unsigned col = 0; col < 2; ++col) {
      p_rbgs(tm, L, e, r, col);
      if (!team_sync(tm)) return false;
    }
    p_restrict(tm, L, S.lev[l + 1], e, r, S.R + 3 * S.lev[l + 1].base, s_res);
    if (!team_sync(tm)) return false;
  }
  if (!p_direct(tm, S)) return false;
  for (int l = nl - 2; l >= 0; --l) {
    const PLev& L = S.lev[l];
    float* e = S.E + 3 * L.base;
    const float* r = S.R + 3 * L.base;
    p_prolong(tm, L, S.lev[l + 1], S.E + 3 * S.lev[l + 1].base, e);
    if (!team_sync(tm)) return false;
    for (int s = 0; s < 2; ++s)
      for (unsigned col = 0; col < 2; ++col) {
        p_rbgs(tm, L, e, r, col);
        if (!team_sync(tm)) return false;
      }
  }
  return true;
}

// V-cycle, x += e, R = b - L x unless it is the phase's last cycle (enqueue_cycle).
__device__ bool p_cycle(Team& tm, const PSim& S, float* xv, const float* b, float* s_res, bool residual) {
  if (!p_vcycle(tm, S, s_res)) return false;
  p_add(tm, xv, S.E, 3 * S.n0);
  if (!team_sync(tm)) return false;
  if (!residual) return true;
  p_residual32(tm, S.lev[0], xv, b, S.R, nullptr, nullptr);
  return team_sync(tm);
}

__device__ double relres_of(const double* acc) {
  const double rr = __ldcg(acc), bb = __ldcg(acc + 1);
  return bb > 0.0 ? sqrt(rr / bb) : sqrt(rr);
}

// run_multigrid_fixed's schedule for one simulation.
__device__ bool p_solve(Team& tm, const PSim& S, float* s_res) {
  const unsigned n3 = 3 * S.n0;
  const bool lead = tm.tid() == 0;
  p_zero(tm, S.E, 3 * S.total);  // e is zero on every level's boundary
  p_zero(tm, S.lo, n3);
  if (S.k2 > 0) p_zero(tm, S.etot, n3);
  if (lead) {
    S.acc[0] = 0.0;
    S.acc[1] = 0.0;
  }
  if (!team_sync(tm)) return false;
  p_residual32(tm, S.lev[0], S.x, S.rhs, S.R, S.acc, S.acc + 1);
  if (!team_sync(tm)) return false;
  if (lead) {
    S.relres[1] = relres_of(S.acc);
    S.acc[0] = 0.0;
  }
  for (int k = 0; k < S.k1; ++k)
    if (!p_cycle(tm, S, S.x, S.rhs, s_res, k + 1 < S.k1)) return false;
  p_residual_pair(tm, S, S.rir, S.k2 > 0 ? nullptr : S.acc);
  if (!team_sync(tm)) return false;
  if (S.k2 > 0) {
    p_copy(tm, S.R, S.rir, n3);
    if (!team_sync(tm)) return false;
    for (int k = 0; k < S.k2; ++k)
      if (!p_cycle(tm, S, S.etot, S.rir, s_res, k + 1 < S.k2)) return false;
    p_add(tm, S.lo, S.etot, n3);
    if (!team_sync(tm)) return false;
    p_residual_pair(tm, S, S.rir, S.acc);
    if (!team_sync(tm)) return false;
  }
  if (lead) S.relres[0] = relres_of(S.acc);
  p_add(tm, S.x, S.lo, n3);
  return true;
}

__global__ void __launch_bounds__(kPThreads, 2) k_mg_persistent(const PSim* __restrict__ sims,
                                                                const int* __restrict__ order,
                                                                const int* __restrict__ team_first, unsigned T,
                                                                unsigned* bar, int* err) {
  __shared__ float s_res[kRFX * kRFY * kRFZ * 3];
  const unsigned team = blockIdx.x / T;
  Team tm;
  tm.ctr = bar + 32 * team;
  tm.err = err;
  tm.T = T;
  tm.rank = blockIdx.x - team * T;
  tm.target = 0;
  tm.limit_ns = kBarrierNs;
  for (int j = team_first[team]; j < team_first[team + 1]; ++j)
    if (!p_solve(tm, sims[order[j]], s_res)) return;
}

// The team barrier alone: one team of T CTAs of which the last `missing`
// never arrive; the others pass two barriers (counted in *passed) or give up
// after limit_ns and set *err.
__global__ void k_team_barrier_check(unsigned T, unsigned missing, unsigned long long limit_ns, unsigned* bar,
                                     int* err, int* passed) {
  Team tm;
  tm.ctr = bar;
  tm.err = err;
  tm.T = T;
  tm.rank = blockIdx.x;
  tm.target = 0;
  tm.limit_ns = limit_ns;
  if (blockIdx.x + missing >= T) return;
  const bool ok = team_sync(tm) && team_sync(tm);
  if (ok && threadIdx.x == 0) atomicAdd(passed, 1);
}

}  // namespace

struct MgBatch {
  int device = 0;
  unsigned T = 0, teams = 0, nsims = 0;
  PSim* d_sims = nullptr;
  int* d_order = nullptr;
  int* d_first = nullptr;
  unsigned* d_bar = nullptr;
  int* d_err = nullptr;
  double* d_acc = nullptr;
};

bool mg_batch_eligible(const Geom& g) {
  const MgPlan P = plan_levels(g);
  return P.direct && P.direct_global && P.nlev <= kPMaxLev && 3 * P.total < 0xffffffffull;
}

void mg_batch_destroy(MgBatch* mb) {
  if (!mb) return;
  cudaFree(mb->d_sims);
  cudaFree(mb->d_order);
  cudaFree(mb->d_first);
  cudaFree(mb->d_bar);
  cudaFree(mb->d_err);
  cudaFree(mb->d_acc);
  delete mb;
}

vg_status mg_batch_build(const std::vector<MgBatchItem>& items, int device, int team_ctas, MgBatch** out,
                         std::string* err) {
  *out = nullptr;
  if (items.empty()) {
    *err = "persistent solve: no simulations";
    return VG_EMPTY;
  }
  std::vector<PSim> hs(items.size());
  std::vector<double> cost(items.size());
  for (size_t i = 0; i < items.size(); ++i) {
    const MgBatchItem& it = items[i];
    Ctx* c = it.c;
    const MgPlan P = plan_levels(it.g);
    if (!(P.direct && P.direct_global && P.nlev <= kPMaxLev) || c->mg_fixed_k1 < 1 || !c->mg_relres_dev) {
      *err = "persistent solve: a simulation without a calibrated schedule ending in the global sine-transform solve";
      return VG_INVALID;
    }
    MgBufs B;
    float *etot = nullptr, *rir = nullptr;
    vg_status st = setup_bufs(c, it.g, P, B, &etot, &rir);
    if (st != VG_OK) {
      *err = "persistent solve: " + c->err;
      return st;
    }
    PSim& S = hs[i];
    memset(&S, 0, sizeof(S));
    S.nlev = P.nlev;
    for (int l = 0; l < P.nlev; ++l) {
      const Lev& L = P.lev[l];
      for (int a = 0; a < 3; ++a) S.lev[l].np[a] = L.g.np[a];
      S.lev[l].r2x = L.r2x;
      S.lev[l].r2y = L.r2y;
      S.lev[l].r2z = L.r2z;
      S.lev[l].H = L.H;
      S.lev[l].base = (unsigned)L.base;
    }
    S.k1 = c->mg_fixed_k1;
    S.k2 = c->mg_fixed_k2;
    S.cf = pair_coef(it.g, P.lev[0]);
    S.E = B.E;
    S.R = B.R;
    S.x = it.soln;
    S.lo = B.lo;
    S.etot = etot;
    S.rir = rir;
    S.rhs = it.rhs;
    if (B.dst64) {
      *err = "persistent solve: the coarsest level must be solved in FP32 (vg_set_coarsest_fp64 off)";
      return VG_INVALID;
    }
    S.dst = (const float*)B.dst;
    S.relres = c->mg_relres_dev;
    S.n0 = (unsigned)it.g.points();
    S.total = (unsigned)P.total;
    // work ~ level-0 points per cycle plus a fixed cost per barrier (~27 a cycle)
    cost[i] = (double)(S.k1 + S.k2 + 1) * ((double)P.total + 27.0 * 4096.0);
  }
  int sms = 0, occ = 0;
  cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_mg_persistent, kPThreads, 0);
  if (e != cudaSuccess || occ < 1) {
    cudaGetLastError();
    *err = std::string("persistent solve: occupancy query: ") + cudaGetErrorString(e);
    return VG_CUDA_ERROR;
  }
  const unsigned max_ctas = (unsigned)(sms * occ);
  unsigned T = team_ctas > 0 ? (unsigned)team_ctas : 8u;
  T = std::min(T, max_ctas);
  const unsigned teams = std::max(1u, std::min(max_ctas / T, (unsigned)items.size()));
  // longest first, each to the least-loaded team
  std::vector<int> idx(items.size());
  for (size_t i = 0; i < idx.size(); ++i) idx[i] = (int)i;
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return cost[a] > cost[b]; });
  std::vector<double> load(teams, 0.0);
  std::vector<std::vector<int>> per(teams);
  for (int i : idx) {
    const size_t t = std::min_element(load.begin(), load.end()) - load.begin();
    load[t] += cost[i];
    per[t].push_back(i);
  }
  std::vector<int> order, first(1, 0);
  for (unsigned t = 0; t < teams; ++t) {
    order.insert(order.end(), per[t].begin(), per[t].end());
    first.push_back((int)order.size());
  }
  MgBatch* mb = new MgBatch();
  mb->device = device;
  mb->T = T;
  mb->teams = teams;
  mb->nsims = (unsigned)items.size();
  e = cudaMalloc(&mb->d_sims, hs.size() * sizeof(PSim));
  if (e == cudaSuccess) e = cudaMalloc(&mb->d_order, order.size() * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&mb->d_first, first.size() * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&mb->d_bar, (size_t)teams * 32 * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMalloc(&mb->d_err, sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&mb->d_acc, hs.size() * 2 * sizeof(double));
  if (e == cudaSuccess) {
    for (size_t i = 0; i < hs.size(); ++i) hs[i].acc = mb->d_acc + 2 * i;
    e = cudaMemcpy(mb->d_sims, hs.data(), hs.size() * sizeof(PSim), cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) e = cudaMemcpy(mb->d_order, order.data(), order.size() * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(mb->d_first, first.data(), first.size() * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(mb->d_err, 0, sizeof(int));
  if (e != cudaSuccess) {
    cudaGetLastError();
    mg_batch_destroy(mb);
    *err = std::string("persistent solve: ") + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? VG_OOM : VG_CUDA_ERROR;
  }
  *out = mb;
  return VG_OK;
}

vg_status mg_batch_enqueue(MgBatch* mb, cudaStream_t s, std::string* err) {
  cudaError_t e = cudaMemsetAsync(mb->d_bar, 0, (size_t)mb->teams * 32 * sizeof(unsigned), s);
  if (e == cudaSuccess) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(mb->teams * mb->T);
    cfg.blockDim = dim3(kPThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;  // every CTA resident at once: the team barriers need it
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, k_mg_persistent, (const PSim*)mb->d_sims, (const int*)mb->d_order,
                           (const int*)mb->d_first, mb->T, mb->d_bar, mb->d_err);
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    *err = std::string("persistent solve launch: ") + cudaGetErrorString(e);
    return VG_CUDA_ERROR;
  }
  return VG_OK;
}

bool mg_batch_failed(MgBatch* mb) {
  int h = 0;
  if (cudaMemcpy(&h, mb->d_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) {
    cudaGetLastError();
    return true;
  }
  if (h) cudaMemset(mb->d_err, 0, sizeof(int));
  return h != 0;
}

void mg_batch_info(const MgBatch* mb, int* teams, int* team_ctas, int* ctas) {
  if (teams) *teams = mb ? (int)mb->teams : 0;
  if (team_ctas) *team_ctas = mb ? (int)mb->T : 0;
  if (ctas) *ctas = mb ? (int)(mb->teams * mb->T) : 0;
}

}  // namespace vg

extern "C" vg_status vg_team_barrier_check(int device, int ctas, int missing, float limit_ms, int* completed,
                                           int* gave_up) {
  using namespace vg;
  if (ctas < 1 || missing < 0 || missing > ctas || !(limit_ms > 0.f) || limit_ms > 10000.f || !completed || !gave_up)
    return VG_INVALID;
  int sms = 0;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess && ctas > sms) return set_noctx_error(VG_INVALID, "vg_team_barrier_check: more CTAs than SMs");
  int* d = nullptr;  // [0] err, [1] passed, [2..] barrier counter
  if (e == cudaSuccess) e = cudaMalloc(&d, 4 * sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(d, 0, 4 * sizeof(int));
  if (e == cudaSuccess) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)ctas);
    cfg.blockDim = dim3(kPThreads);
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, k_team_barrier_check, (unsigned)ctas, (unsigned)missing,
                           (unsigned long long)((double)limit_ms * 1e6), (unsigned*)(d + 2), d, d + 1);
  }
  int h[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  if (d) cudaFree(d);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_noctx_error(VG_CUDA_ERROR, std::string("vg_team_barrier_check: ") + cudaGetErrorString(e));
  }
  *gave_up = h[0] != 0;
  *completed = h[1];
  return VG_OK;
}
