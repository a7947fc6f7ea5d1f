// K1: direct mollified Biot-Savart / vector-potential sums.
//
// Replaces ComputeVelocity_Direct / ComputeVectorPotential_Direct
// (VortonFluid/vortonSim.cpp:1113-1158), the per-pair laws of
// VortonFluid/vorton.h:118-179.
//
// Fast path (FP32-FMA bound):
//   * a CTA owns TPT * THREADS query points (TPT per thread in registers) and
//     one of KSPLIT equal chunks of the sources, so that a 40k-target,
//     4k-source problem still fills 152 SMs;
//   * sources are staged through shared memory in tiles as two float4 per
//     vorton -- (position, 1/radius) and (2/3 r^3 * angvel * circulation
//     factor) -- and read by every warp as broadcasts;
//   * per pair: law = min(rsqrt(|d|^2), 1/r)^3 (one MUFU.RSQ), 18 FP32 pipe
//     instructions for the 26 algorithmic flops;
//   * the KSPLIT partial sums per target go to a scratch buffer and are summed
//     in a fixed order by a second kernel, so results are run-to-run
//     deterministic.
// Reference path: one thread per query, sources in index order, the
// reference's operation order (bit-identical to the CPU).
#include <float.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <string>

#include "vg_internal.cuh"

namespace vg {

namespace {

constexpr int kThreads = 128;
constexpr int kTPT = 8;        // targets per thread
constexpr int kTile = 256;     // sources per shared-memory tile

// One MUFU.RSQ: approximate reciprocal square root with denormals flushed
// (rsqrt(0) = +inf, which the min(., 1/r) below turns into the core law).
__device__ __forceinline__ float rsqrt_ftz(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Precompute per-source constants for the fast law.
template <int KIND>
__global__ void __launch_bounds__(256) k_prep_sources(const float4* __restrict__ ps, const float4* __restrict__ w,
                                                      int n, float sr, float sc, float4* __restrict__ s0,
                                                      float4* __restrict__ s1) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p = ps[i];
  const float4 a = w[i];
  const float radius = p.w * 0.5f * sr;
  const float s = VG_TWO_THIRDS * radius * radius * radius * sc;
  const float invr = 1.0f / radius;
  s0[i] = make_float4(p.x, p.y, p.z, invr);
  s1[i] = make_float4(a.x * s, a.y * s, a.z * s, radius * radius);
}

template <int KIND>
__global__ void __launch_bounds__(kThreads) k_direct_fast(const float4* __restrict__ s0, const float4* __restrict__ s1,
                                                           int n, int chunk, const float4* __restrict__ q, int m,
                                                           float* __restrict__ partial) {
  __shared__ float4 sh0[kTile];
  __shared__ float4 sh1[kTile];
  const int base = blockIdx.x * (kThreads * kTPT) + threadIdx.x;
  float qx[kTPT], qy[kTPT], qz[kTPT];
  float ax[kTPT], ay[kTPT], az[kTPT];
#pragma unroll
  for (int t = 0; t < kTPT; ++t) {
    const int j = base + t * kThreads;
    const float4 v = (j < m) ? q[j] : make_float4(0.f, 0.f, 0.f, 0.f);
    qx[t] = v.x; qy[t] = v.y; qz[t] = v.z;
    ax[t] = 0.f; ay[t] = 0.f; az[t] = 0.f;
  }
  const int k0 = blockIdx.y * chunk;
  const int k1 = min(n, k0 + chunk);
  for (int tile = k0; tile < k1; tile += kTile) {
    const int cnt = min(kTile, k1 - tile);
    __syncthreads();
    for (int i = threadIdx.x; i < cnt; i += kThreads) {
      sh0[i] = s0[tile + i];
      sh1[i] = s1[tile + i];
    }
    __syncthreads();
#pragma unroll 4
    for (int i = 0; i < cnt; ++i) {
      const float4 p = sh0[i];
      const float4 a = sh1[i];
#pragma unroll
      for (int t = 0; t < kTPT; ++t) {
        const float d0 = qx[t] - p.x, d1 = qy[t] - p.y, d2 = qz[t] - p.z;
        const float dist2 = fmaf(d0, d0, fmaf(d1, d1, d2 * d2));
        if (KIND == 0) {
          const float inv = fminf(rsqrt_ftz(dist2), p.w);
          const float law = inv * inv * inv;
          const float b0 = d0 * law, b1 = d1 * law, b2 = d2 * law;
          ax[t] = fmaf(a.y, b2, fmaf(-a.z, b1, ax[t]));
          ay[t] = fmaf(a.z, b0, fmaf(-a.x, b2, ay[t]));
          az[t] = fmaf(a.x, b1, fmaf(-a.y, b0, az[t]));
        } else {
          const float law = (dist2 < a.w) ? dist2 * p.w * p.w * p.w : rsqrt_ftz(dist2);
          ax[t] = fmaf(a.x, law, ax[t]);
          ay[t] = fmaf(a.y, law, ay[t]);
          az[t] = fmaf(a.z, law, az[t]);
        }
      }
    }
  }
  float* out = partial + (size_t)blockIdx.y * m * 3;
#pragma unroll
  for (int t = 0; t < kTPT; ++t) {
    const int j = base + t * kThreads;
    if (j < m) {
      out[3 * j] = ax[t];
      out[3 * j + 1] = ay[t];
      out[3 * j + 2] = az[t];
    }
  }
}

constexpr int kPairTPT = 8;
constexpr int kPairThreads = 256;

// How a k_direct_pair launch divides its targets and sources.  Targets
// [0, pts) may be the points of a grid: in the first `rows` grid rows (as
// many as whole CTAs of row threads hold), the first xs = 8 floor(np0 / 8)
// points of a row are row targets (8 consecutive points of one row per
// thread); the last r0 = np0 - xs points of those rows (nrem in all), every
// point of the later rows (nrest) and the targets [pts, m) (points
// qg[0, m - pts)) form the general class (8 per thread, strided by the CTA
// width).  Each class has its own
// source split (ks chunks of `chunk` sources), chosen so that the CTAs of both
// classes take about as long; CTA b < row_ctas * row_ks is a row CTA.
struct PairPlan {
  Geom g;                 // the grid whose points are targets [0, pts)
  int rows, tpr;          // rows of the row class (whole CTAs of row threads), row threads per row (xs / 8)
  int xs, r0, nrem;       // first remainder column, remainder columns, remainder points of those rows
  int nrest;              // points of the grid rows past the row class (general targets after the remainders)
  int row_ctas, row_ks, row_chunk;
  int pts, m;             // targets: grid points [0, pts), then qg[0, m - pts)
  int gen_ctas, gen_ks, gen_chunk;
};

// Position of the gridpoint (x, y, z): the velocity step's gridpoint positions,
// min + i spacing (1 - 2 FLT_EPSILON).
__device__ __forceinline__ float grid_coord(const Geom& g, int a, int i) {
  return __fadd_rn(g.mn[a], __fmul_rn((float)i, __fmul_rn(g.cell[a], 1.0f - 2.0f * FLT_EPSILON)));
}

// Stages sources [tile, tile + cnt) as five float4 per source, each value
// duplicated for the packed operations: (-p, 1/R, w, -w) with w scaled as in
// k_prep_sources<0>.
__device__ __forceinline__ void stage_pair_tile(const float4* __restrict__ ps, const float4* __restrict__ w,
                                                int tile, int cnt, float sr, float sc, float4* sh) {
  for (int i = threadIdx.x; i < cnt; i += kPairThreads) {
    const float4 p = ps[tile + i], a0 = w[tile + i];
    // k_prep_sources<0>: 1/R and the scaled angular velocity
    const float radius = p.w * 0.5f * sr;
    const float s = VG_TWO_THIRDS * radius * radius * radius * sc;
    const float invr = 1.0f / radius;
    const float4 a = make_float4(a0.x * s, a0.y * s, a0.z * s, 0.f);
    sh[5 * i + 0] = make_float4(-p.x, -p.x, -p.y, -p.y);
    sh[5 * i + 1] = make_float4(-p.z, -p.z, invr, invr);
    sh[5 * i + 2] = make_float4(a.x, a.x, a.y, a.y);
    sh[5 * i + 3] = make_float4(a.z, a.z, -a.x, -a.x);
    sh[5 * i + 4] = make_float4(-a.y, -a.y, -a.z, -a.z);
  }
}

// General targets t of the class (remainder gridpoints, then qg): its
// position, and where its sum goes (target index j).
__device__ __forceinline__ float4 general_target(const PairPlan& P, const float4* __restrict__ qg, int t, int* j) {
  const int np0 = (int)P.g.np[0], np1 = (int)P.g.np[1];
  int row, x;
  if (t < P.nrem) {
    row = t / P.r0, x = P.xs + (t - row * P.r0);
  } else if (t < P.nrem + P.nrest) {
    const int u = t - P.nrem;
    row = P.rows + u / np0, x = u % np0;
  } else {
    *j = P.pts + (t - P.nrem - P.nrest);
    return qg[t - P.nrem - P.nrest];
  }
  *j = row * np0 + x;
  return make_float4(grid_coord(P.g, 0, x), grid_coord(P.g, 1, row % np1), grid_coord(P.g, 2, row / np1), 0.f);
}

// Arbitrary targets: each operation advances two targets (a float2 pair) of
// the thread's eight.  17 packed operations per pair and source: d (3), |d|^2
// (3), the cubed law (2), b = d law (3), w x b accumulated (6).
__device__ __forceinline__ void pair_general(const float4* __restrict__ ps, const float4* __restrict__ w, int n,
                                             float sr, float sc, const float4* __restrict__ qg, const PairPlan& P,
                                             int b, float4* sh, float* __restrict__ partial,
                                             float4* __restrict__ out) {
  constexpr int kPairs = kPairTPT / 2;
  const int tb = b / P.gen_ks, kc = b - tb * P.gen_ks;
  const int base = tb * (kPairThreads * kPairTPT) + threadIdx.x;
  const int count = P.nrem + P.nrest + (P.m - P.pts);
  float2 qx[kPairs], qy[kPairs], qz[kPairs], ax[kPairs], ay[kPairs], az[kPairs];
  int jt[kPairTPT];
#pragma unroll
  for (int pr = 0; pr < kPairs; ++pr) {
    const int t0 = base + 2 * pr * kPairThreads, t1 = t0 + kPairThreads;
    jt[2 * pr] = jt[2 * pr + 1] = -1;
    const float4 v0 = (t0 < count) ? general_target(P, qg, t0, &jt[2 * pr]) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 v1 = (t1 < count) ? general_target(P, qg, t1, &jt[2 * pr + 1]) : make_float4(0.f, 0.f, 0.f, 0.f);
    qx[pr] = make_float2(v0.x, v1.x);
    qy[pr] = make_float2(v0.y, v1.y);
    qz[pr] = make_float2(v0.z, v1.z);
    ax[pr] = ay[pr] = az[pr] = make_float2(0.f, 0.f);
  }
  const int k0 = kc * P.gen_chunk;
  const int k1 = min(n, k0 + P.gen_chunk);
  for (int tile = k0; tile < k1; tile += kTile) {
    const int cnt = min(kTile, k1 - tile);
    __syncthreads();
    stage_pair_tile(ps, w, tile, cnt, sr, sc, sh);
    __syncthreads();
#pragma unroll 4
    for (int i = 0; i < cnt; ++i) {
      const float4 e0 = sh[5 * i], e1 = sh[5 * i + 1], e2 = sh[5 * i + 2], e3 = sh[5 * i + 3], e4 = sh[5 * i + 4];
      const float2 np0 = make_float2(e0.x, e0.y), np1 = make_float2(e0.z, e0.w), np2 = make_float2(e1.x, e1.y);
      const float invr = e1.z;
      const float2 wx = make_float2(e2.x, e2.y), wy = make_float2(e2.z, e2.w), wz = make_float2(e3.x, e3.y);
      const float2 nwx = make_float2(e3.z, e3.w), nwy = make_float2(e4.x, e4.y), nwz = make_float2(e4.z, e4.w);
#pragma unroll
      for (int pr = 0; pr < kPairs; ++pr) {
        const float2 d0 = __fadd2_rn(qx[pr], np0), d1 = __fadd2_rn(qy[pr], np1), d2 = __fadd2_rn(qz[pr], np2);
        const float2 r2 = __ffma2_rn(d0, d0, __ffma2_rn(d1, d1, __fmul2_rn(d2, d2)));
        const float2 inv = make_float2(fminf(rsqrt_ftz(r2.x), invr), fminf(rsqrt_ftz(r2.y), invr));
        const float2 law = __fmul2_rn(__fmul2_rn(inv, inv), inv);
        const float2 b0 = __fmul2_rn(d0, law), b1 = __fmul2_rn(d1, law), b2 = __fmul2_rn(d2, law);
        ax[pr] = __ffma2_rn(wy, b2, __ffma2_rn(nwz, b1, ax[pr]));
        ay[pr] = __ffma2_rn(wz, b0, __ffma2_rn(nwx, b2, ay[pr]));
        az[pr] = __ffma2_rn(wx, b1, __ffma2_rn(nwy, b0, az[pr]));
      }
    }
  }
  float* mine = partial ? partial + (size_t)kc * (size_t)count * 3 : nullptr;
#pragma unroll
  for (int pr = 0; pr < kPairs; ++pr) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int t = base + (2 * pr + h) * kPairThreads, j = jt[2 * pr + h];
      if (j < 0) continue;
      const float vx = h ? ax[pr].y : ax[pr].x, vy = h ? ay[pr].y : ay[pr].x, vz = h ? az[pr].y : az[pr].x;
      if (!mine) {  // one chunk: the sums are final (0 + sum, as the reduction would give)
        out[j] = make_float4(0.f + vx, 0.f + vy, 0.f + vz, 0.f);
      } else {
        float* o = mine + 3 * (size_t)t;
        o[0] = vx, o[1] = vy, o[2] = vz;
      }
    }
  }
}

// Grid points: a thread holds 8 consecutive points of one grid row, which
// share y and z, so per source the y and z terms are formed once -- d1, d2,
// d1^2 + d2^2, (w x d)_x and the w d2 and w d1 products (8 packed operations)
// -- and each target pair needs 9: d0, |d|^2 = d0^2 + (d1^2 + d2^2) (the
// general path's rounding order, so the same bits), the cubed law (2), the
// (w x d)_y and _z components that depend on d0 (2), and law (w x d)
// accumulated (3).
__device__ __forceinline__ void pair_rows(const float4* __restrict__ ps, const float4* __restrict__ w, int n,
                                          float sr, float sc, const PairPlan& P, int b, float4* sh,
                                          float* __restrict__ partial, float4* __restrict__ out) {
  constexpr int kPairs = kPairTPT / 2;
  const int tb = b / P.row_ks, kc = b - tb * P.row_ks;
  const int t = tb * kPairThreads + threadIdx.x;
  const int r = t / P.tpr, seg = t - r * P.tpr;
  const bool live = r < P.rows;
  const int rr = live ? r : P.rows - 1;
  const int np0 = (int)P.g.np[0], np1 = (int)P.g.np[1];
  const int iy = rr % np1, iz = rr / np1;
  const int x0 = seg * kPairTPT;
  float2 qx[kPairs], ax[kPairs], ay[kPairs], az[kPairs];
#pragma unroll
  for (int pr = 0; pr < kPairs; ++pr) {
    qx[pr] = make_float2(grid_coord(P.g, 0, x0 + 2 * pr), grid_coord(P.g, 0, x0 + 2 * pr + 1));
    ax[pr] = ay[pr] = az[pr] = make_float2(0.f, 0.f);
  }
  const float qyv = grid_coord(P.g, 1, iy), qzv = grid_coord(P.g, 2, iz);
  const float2 qy = make_float2(qyv, qyv), qz = make_float2(qzv, qzv);
  const int k0 = kc * P.row_chunk;
  const int k1 = min(n, k0 + P.row_chunk);
  for (int tile = k0; tile < k1; tile += kTile) {
    const int cnt = min(kTile, k1 - tile);
    __syncthreads();
    stage_pair_tile(ps, w, tile, cnt, sr, sc, sh);
    __syncthreads();
#pragma unroll 4
    for (int i = 0; i < cnt; ++i) {
      const float4 e0 = sh[5 * i], e1 = sh[5 * i + 1], e2 = sh[5 * i + 2], e3 = sh[5 * i + 3], e4 = sh[5 * i + 4];
      const float2 np0d = make_float2(e0.x, e0.y), np1d = make_float2(e0.z, e0.w), np2d = make_float2(e1.x, e1.y);
      const float invr = e1.z;
      const float2 wx = make_float2(e2.x, e2.y), wy = make_float2(e2.z, e2.w), wz = make_float2(e3.x, e3.y);
      const float2 nwx = make_float2(e3.z, e3.w), nwy = make_float2(e4.x, e4.y), nwz = make_float2(e4.z, e4.w);
      const float2 d1 = __fadd2_rn(qy, np1d), d2 = __fadd2_rn(qz, np2d);
      const float2 yz2 = __ffma2_rn(d1, d1, __fmul2_rn(d2, d2));
      const float2 cx = __ffma2_rn(nwz, d1, __fmul2_rn(wy, d2));  // wy d2 - wz d1
      const float2 nwxd2 = __fmul2_rn(nwx, d2), wxd1 = __fmul2_rn(wx, d1);
#pragma unroll
      for (int pr = 0; pr < kPairs; ++pr) {
        const float2 d0 = __fadd2_rn(qx[pr], np0d);
        const float2 r2 = __ffma2_rn(d0, d0, yz2);
        const float2 inv = make_float2(fminf(rsqrt_ftz(r2.x), invr), fminf(rsqrt_ftz(r2.y), invr));
        const float2 law = __fmul2_rn(__fmul2_rn(inv, inv), inv);
        const float2 cy = __ffma2_rn(wz, d0, nwxd2);  // wz d0 - wx d2
        const float2 cz = __ffma2_rn(nwy, d0, wxd1);  // wx d1 - wy d0
        ax[pr] = __ffma2_rn(law, cx, ax[pr]);
        ay[pr] = __ffma2_rn(law, cy, ay[pr]);
        az[pr] = __ffma2_rn(law, cz, az[pr]);
      }
    }
  }
  if (!live) return;
  float4* mine = partial ? reinterpret_cast<float4*>(partial) + (size_t)kc * (size_t)P.pts : nullptr;
  const size_t jrow = (size_t)rr * np0 + x0;
#pragma unroll
  for (int pr = 0; pr < kPairs; ++pr) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const size_t j = jrow + 2 * pr + h;
      const float vx = h ? ax[pr].y : ax[pr].x, vy = h ? ay[pr].y : ay[pr].x, vz = h ? az[pr].y : az[pr].x;
      if (!mine)
        out[j] = make_float4(0.f + vx, 0.f + vy, 0.f + vz, 0.f);
      else
        mine[j] = make_float4(vx, vy, vz, 0.f);
    }
  }
}

// Velocity (KIND 0) with packed FP32x2 arithmetic (FADD2 / FMUL2 / FFMA2):
// every source is staged in shared memory already duplicated into pairs, so
// each operation advances two targets in one instruction.  Row CTAs (grid
// points) and general CTAs (arbitrary points) run in the same launch, each
// class with its own source split.  With one chunk per class the sums are
// written to out; otherwise the partial sums go to a scratch buffer per class
// ([chunk][target][3]) and k_reduce_pair adds them in chunk order, so results
// are run-to-run deterministic.
// 8 targets per thread (126 registers) was the fastest of the shapes measured
// on GB300 for the general path (4 to 16 targets); CTAs of 256 threads, 2 per
// SM, beat 4 CTAs of 128 by ~4%: the tile barriers keep a CTA's warps
// together, whereas independent small CTAs on one SM finish far apart and
// leave the SM short of warps at the end.
__global__ void __launch_bounds__(kPairThreads, 2)
    k_direct_pair(const float4* __restrict__ ps, const float4* __restrict__ w, int n, float sr, float sc,
                  const float4* __restrict__ qg, PairPlan P, float* __restrict__ partial_rows,
                  float* __restrict__ partial_gen, float4* __restrict__ out) {
  pdl_entry();
  __shared__ float4 sh[5 * kTile];
  const int row_total = P.row_ctas * P.row_ks;
  if ((int)blockIdx.x < row_total)
    pair_rows(ps, w, n, sr, sc, P, (int)blockIdx.x, sh, partial_rows, out);
  else
    pair_general(ps, w, n, sr, sc, qg, P, (int)blockIdx.x - row_total, sh, partial_gen, out);
}

// Sums each target's partial sums in chunk order -- row targets from the
// row partials (float4, indexed by target), general targets (remainder and
// later-row gridpoints, targets past the grid) from the general partials
// (float[3], indexed by class position) -- with up to 16 chunks' loads issued
// before the first add: the sum is bound by the latency of these loads, not
// by their bytes.
// With evolve_pos, the vortons' positions also move by their velocity x dt
// (PclOpEvolve's Euler step, as k_evolve would do next).
__global__ void __launch_bounds__(128) k_reduce_pair(const float4* __restrict__ partial_rows,
                                                     const float* __restrict__ partial_gen, PairPlan P,
                                                     float4* __restrict__ out, float* __restrict__ grid3, int pts,
                                                     float4* __restrict__ vel, float4* __restrict__ evolve_pos,
                                                     float dt) {
  pdl_entry();
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= P.m) return;
  constexpr int kBatch = 16;
  float sx = 0.f, sy = 0.f, sz = 0.f;
  const int np0 = (int)P.g.np[0];
  const int row = j < P.pts ? j / np0 : 0, x = j < P.pts ? j - row * np0 : 0;
  if (j < P.pts && row < P.rows && x < P.xs) {  // row partials: float4 per target
    const float4* src = partial_rows + j;
    for (int k0 = 0; k0 < P.row_ks; k0 += kBatch) {
      float4 v[kBatch];
#pragma unroll
      for (int k = 0; k < kBatch; ++k)
        if (k0 + k < P.row_ks) v[k] = src[(size_t)(k0 + k) * P.pts];
#pragma unroll
      for (int k = 0; k < kBatch; ++k)
        if (k0 + k < P.row_ks) {
          sx += v[k].x;
          sy += v[k].y;
          sz += v[k].z;
        }
    }
  } else {  // general partials: float[3] per target
    const int t = j >= P.pts ? P.nrem + P.nrest + (j - P.pts)
                             : (row < P.rows ? row * P.r0 + (x - P.xs) : P.nrem + (row - P.rows) * np0 + x);
    const float* src = partial_gen + 3 * (size_t)t;
    const size_t stride = 3 * (size_t)(P.nrem + P.nrest + (P.m - P.pts));
    for (int k0 = 0; k0 < P.gen_ks; k0 += kBatch) {
      float v[kBatch][3];
#pragma unroll
      for (int k = 0; k < kBatch; ++k)
        if (k0 + k < P.gen_ks) {
          const float* p = src + (size_t)(k0 + k) * stride;
          v[k][0] = p[0];
          v[k][1] = p[1];
          v[k][2] = p[2];
        }
#pragma unroll
      for (int k = 0; k < kBatch; ++k)
        if (k0 + k < P.gen_ks) {
          sx += v[k][0];
          sy += v[k][1];
          sz += v[k][2];
        }
    }
  }
  if (!grid3) {
    out[j] = make_float4(sx, sy, sz, 0.f);
  } else if (j < pts) {  // the velocity step's split: gridpoints as float[3], vortons as records
    grid3[3 * j] = sx;
    grid3[3 * j + 1] = sy;
    grid3[3 * j + 2] = sz;
  } else {
    vel[j - pts] = make_float4(sx, sy, sz, 0.f);
    if (evolve_pos) {
      float4 p = evolve_pos[j - pts];
      p.x = __fadd_rn(p.x, __fmul_rn(sx, dt));
      p.y = __fadd_rn(p.y, __fmul_rn(sy, dt));
      p.z = __fadd_rn(p.z, __fmul_rn(sz, dt));
      evolve_pos[j - pts] = p;
    }
  }
}

__global__ void k_reduce_partials(const float* __restrict__ partial, int ksplit, int m, float4* __restrict__ out) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  float x = 0.f, y = 0.f, z = 0.f;
  for (int k = 0; k < ksplit; ++k) {
    const float* p = partial + ((size_t)k * m + j) * 3;
    x += p[0];
    y += p[1];
    z += p[2];
  }
  out[j] = make_float4(x, y, z, 0.f);
}

// Reference order: each thread sums all sources for one query in index order.
template <int KIND>
__global__ void __launch_bounds__(kThreads) k_direct_ref(const float4* __restrict__ ps, const float4* __restrict__ w,
                                                          int n, const float4* __restrict__ q, int m, float sr,
                                                          float sc, float4* __restrict__ out) {
  __shared__ float4 sh0[kTile];
  __shared__ float4 sh1[kTile];
  const int j = blockIdx.x * kThreads + threadIdx.x;
  const float4 v = (j < m) ? q[j] : make_float4(0.f, 0.f, 0.f, 0.f);
  float3 acc = make_float3(0.f, 0.f, 0.f);
  for (int tile = 0; tile < n; tile += kTile) {
    const int cnt = min(kTile, n - tile);
    __syncthreads();
    for (int i = threadIdx.x; i < cnt; i += kThreads) {
      sh0[i] = ps[tile + i];
      sh1[i] = w[tile + i];
    }
    __syncthreads();
    for (int i = 0; i < cnt; ++i) ref_accum<KIND>(acc, v.x, v.y, v.z, sh0[i], sh1[i], sr, sc);
  }
  if (j < m) out[j] = make_float4(acc.x, acc.y, acc.z, 0.f);
}

// Resident CTAs of k_direct_fast across the device (SMs x occupancy), queried once.
unsigned direct_slots(int kind) {
  static unsigned cached[2] = {0, 0};
  if (!cached[kind]) {
    int dev = 0, sms = sm_count(), per_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (kind == 0)
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_direct_pair, kPairThreads, 0);
    else
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_direct_fast<1>, kThreads, 0);
    cudaGetLastError();
    cached[kind] = (unsigned)std::max(1, sms) * (unsigned)std::max(1, per_sm);
  }
  return cached[kind];
}

// Split the sources into `ksplit` chunks so that target blocks x chunks
// fills the resident CTA slots of the GPU (SMs x CTAs per SM) once, with no
// partial second wave; every CTA then does the same amount of work.  Returns
// the chunk length.
int direct_split(int kind, size_t n, size_t m, unsigned* tblocks_out, unsigned* ksplit_out) {
  const unsigned tblocks = blocks_for(m, kind == 0 ? kPairThreads * kPairTPT : kThreads * kTPT);
  const unsigned slots = direct_slots(kind);
  unsigned ksplit = std::max(1u, slots / tblocks);
  const size_t min_chunk = 64;  // keep each CTA's source loop long enough to amortise its set-up
  if (n / ksplit < min_chunk) ksplit = (unsigned)std::max<size_t>(1, n / min_chunk);
  const int chunk = (int)((n + ksplit - 1) / ksplit);
  *ksplit_out = (unsigned)((n + chunk - 1) / chunk);
  *tblocks_out = tblocks;
  return chunk;
}

// The source split of a k_direct_pair launch.  Each class of targets (grid
// rows, general points) gets its own number of source chunks, chosen to
// minimise the estimated time: the CTAs of both classes run in one wave
// where possible (SMs x CTAs per SM), and the slowest CTA sets the time.  A
// CTA's time is its chunk length times the class's packed operations per
// source and thread (row CTAs 8 + 4 x 9 = 44, general CTAs 4 x 17 = 68), plus
// a fixed set-up; more chunks cost more partial sums to reduce.
PairPlan plan_pair(size_t n, size_t m, const Geom* grid) {
  PairPlan P = {};
  if (grid) {
    P.g = *grid;
    const int all_rows = (int)(grid->np[1] * grid->np[2]);
    P.xs = (int)(grid->np[0] / kPairTPT) * kPairTPT;
    P.r0 = (int)grid->np[0] - P.xs;
    P.tpr = P.xs / kPairTPT;
    // whole CTAs of row threads only: the rows they cannot hold go to the general class
    P.row_ctas = P.tpr ? (int)(((size_t)all_rows * P.tpr) / kPairThreads) : 0;
    P.rows = P.row_ctas ? std::min(all_rows, P.row_ctas * kPairThreads / P.tpr) : 0;
    if (!P.rows) P.row_ctas = 0;
    P.nrem = P.rows * P.r0;
    P.nrest = (all_rows - P.rows) * (int)grid->np[0];
    P.pts = (int)grid->points();
  }
  P.m = (int)m;
  const size_t gcount = (size_t)P.nrem + (size_t)P.nrest + (m - (size_t)P.pts);
  P.gen_ctas = (int)blocks_for(gcount, kPairThreads * kPairTPT);
  struct Key {
    size_t n, m;
    int pts, rows, tpr, nrem, nrest, pad;
  };
  thread_local Key cached_key = {0, 0, 0, 0, 0, 0, 0, 0};
  thread_local int cached_ks[2] = {0, 0};
  const Key key = {n, m, P.pts, P.rows, P.tpr, P.nrem, P.nrest, 0};
  int kr = 1, kg = 1;
  if (cached_ks[0] && memcmp(&key, &cached_key, sizeof(Key)) == 0) {
    kr = cached_ks[0], kg = cached_ks[1];
  } else {
    const double slots = direct_slots(0), c_row = 44.0, c_gen = 68.0, setup = 24.0, reduce = 0.002;
    const int kmax = (int)std::max<size_t>(1, std::min<size_t>(256, n / 64));
    double best = 1e300;
    for (int a = 1; a <= (P.row_ctas ? kmax : 1); ++a)
      for (int b = 1; b <= (P.gen_ctas ? kmax : 1); ++b) {
        const size_t cr = (n + a - 1) / a, cg = (n + b - 1) / b;
        const double ctas = (double)P.row_ctas * a + (double)P.gen_ctas * b;
        const double waves = std::ceil(ctas / slots);
        const double slow = std::max(P.row_ctas ? c_row * (cr + setup) : 0.0, P.gen_ctas ? c_gen * (cg + setup) : 0.0);
        const double t =
            waves * slow + ((a > 1 || b > 1) ? reduce * ((double)a * P.pts + (double)b * (double)gcount) : 0.0);
        if (t < best) best = t, kr = a, kg = b;
      }
    cached_key = key;
    cached_ks[0] = kr, cached_ks[1] = kg;
  }
  P.row_chunk = (int)((n + kr - 1) / kr);
  P.row_ks = P.row_ctas ? (int)((n + P.row_chunk - 1) / P.row_chunk) : 1;
  P.gen_chunk = (int)((n + kg - 1) / kg);
  P.gen_ks = P.gen_ctas ? (int)((n + P.gen_chunk - 1) / P.gen_chunk) : 1;
  return P;
}

// Launches k_direct_pair (and, with more than one chunk in either class,
// k_reduce_pair) for plan P; partial has room for the plan's partial sums.
template <typename Launch>
cudaError_t launch_pair_plan(Launch launch, const PairPlan& P, const float4* ps, const float4* w, int n, float sr,
                             float sc, const float4* qg, float* partial, float4* out, const DirectSplit* split) {
  const bool reduce = P.row_ks > 1 || P.gen_ks > 1;
  float* pr = reduce ? partial : nullptr;
  float* pg = reduce ? partial + (P.row_ctas ? (size_t)P.row_ks * P.pts * 4 : 0) : nullptr;
  const unsigned ctas = (unsigned)(P.row_ctas * P.row_ks + P.gen_ctas * P.gen_ks);
  cudaError_t e = launch(dim3(ctas), dim3(kPairThreads), k_direct_pair, ps, w, n, sr, sc, qg, P, pr, pg, out);
  if (e != cudaSuccess || !reduce) return e;
  return launch(dim3(blocks_for((size_t)P.m, 128)), dim3(128), k_reduce_pair, (const float4*)pr, (const float*)pg,
                P, out, split ? split->grid3 : (float*)nullptr, split ? (int)split->pts : 0,
                split ? split->vel : (float4*)nullptr, split ? split->evolve_pos : (float4*)nullptr,
                split ? split->evolve_dt : 0.f);
}

// Partial sums of a plan: per chunk, float4 per gridpoint (row class), float[3] per general target.
size_t pair_partial_floats(const PairPlan& P) {
  const size_t rows = P.row_ctas ? (size_t)P.row_ks * (size_t)P.pts * 4 : 0;
  return rows + 3 * (size_t)P.gen_ks * ((size_t)P.nrem + (size_t)P.nrest + (size_t)(P.m - P.pts));
}

}  // namespace

vg_status launch_direct(Ctx* c, int kind, bool ref, const float4* ps, const float4* w, size_t n, const float4* q,
                        size_t m, float sr, float sc, float4* out, const DirectSplit* split, bool* split_done) {
  if (m == 0) return VG_OK;
  if (n == 0) {
    VG_CUDA(c, cudaMemsetAsync(out, 0, m * sizeof(float4), c->stream));
    return VG_OK;
  }
  if (n > 0x7fffffff || m > 0x7fffffff) return fail(c, VG_TOO_LARGE, "direct: more than 2^31 sources or targets");
  if (ref) {
    dim3 grid(blocks_for(m, kThreads));
    if (kind == 0)
      k_direct_ref<0><<<grid, kThreads, 0, c->stream>>>(ps, w, (int)n, q, (int)m, sr, sc, out);
    else
      k_direct_ref<1><<<grid, kThreads, 0, c->stream>>>(ps, w, (int)n, q, (int)m, sr, sc, out);
    VG_LAUNCHED(c);
    VG_CUDA(c, cudaGetLastError());
    return VG_OK;
  }
  vg_status st = VG_OK;
  if (kind == 0) {
    // grid rows for the step's gridpoint targets, when they are the grid's points
    const Geom* grid = (split && split->grid && split->grid->points() == split->pts && split->pts <= m &&
                        split->grid->np[0] >= 1)
                           ? split->grid
                           : nullptr;
    const PairPlan P = plan_pair(n, m, grid);
    const bool reduce = P.row_ks > 1 || P.gen_ks > 1;
    float* partial = nullptr;
    if (reduce) {
      partial = (float*)ws(c, S_DIRECT, pair_partial_floats(P) * sizeof(float), &st);
      if (st != VG_OK) return st;
    }
    cudaStream_t s = c->stream;
    auto launch = [s](dim3 g, dim3 b, auto kernel, auto... args) { return pdl_launch(s, g, b, 0, kernel, args...); };
    const float4* qg = (grid && split->after_grid) ? split->after_grid : q + P.pts;
    VG_CUDA(c, launch_pair_plan(launch, P, ps, w, (int)n, sr, sc, qg, partial, out, split));
    c->launches += reduce ? 2 : 1;
    if (split_done) *split_done = reduce && split != nullptr;
    if (reduce && split && split->evolve_pos) c->step_evolved = true;
    VG_CUDA(c, cudaGetLastError());
    return VG_OK;
  }
  unsigned tblocks = 0, ksplit = 0;
  const int chunk = direct_split(kind, n, m, &tblocks, &ksplit);
  const size_t srcb = ((n * sizeof(float4) + 255) / 256) * 256;
  char* scratch = (char*)ws(c, S_DIRECT, 2 * srcb + (size_t)ksplit * m * 3 * sizeof(float), &st);
  if (st != VG_OK) return st;
  float4* s0 = (float4*)scratch;
  float4* s1 = (float4*)(scratch + srcb);
  float* partial = (float*)(scratch + 2 * srcb);
  k_prep_sources<1><<<blocks_for(n, 256), 256, 0, c->stream>>>(ps, w, (int)n, sr, sc, s0, s1);
  VG_LAUNCHED(c);
  dim3 grid(tblocks, ksplit);
  k_direct_fast<1><<<grid, kThreads, 0, c->stream>>>(s0, s1, (int)n, chunk, q, (int)m, partial);
  VG_LAUNCHED(c);
  k_reduce_partials<<<blocks_for(m, 256), 256, 0, c->stream>>>(partial, (int)ksplit, (int)m, out);
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

}  // namespace vg

// ---------------------------------------------------------------------------
// Allocation-free direct sum (vg_direct_noalloc).
//
// Some callers cannot allocate device memory at the moment they need the
// velocity: a host application that hands this library a fixed memory budget
// up front, code running inside a real-time frame where an allocation's
// implicit device synchronisation would stall the frame, or an embedding that
// forbids the CUDA allocator altogether.  For them the scratch that the
// split-source direct sum needs (per-target partial sums, and for the vector
// potential the per-source constants) lives in one file-scope device array.
// It is reserved when this library's device code is loaded on a device --
// with lazy module loading, at the first call that needs it there -- and is
// held by that device until the process exits.
namespace vg {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(8) << 20;  // 8 MiB
constexpr size_t kNoAllocMaxSources = 32768;              // 1 MiB of per-source constants
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// A plain launch whose own error code is returned (no stream-wide error query
// that could report, and clear, an error some other code left behind).
template <typename... KArgs, typename... Args>
cudaError_t launch_plain(cudaStream_t s, dim3 grid, dim3 block, void (*kernel)(KArgs...), Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.stream = s;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

vg_status noalloc_fail(cudaError_t e, const char* what) {
  return set_noctx_error(VG_CUDA_ERROR, std::string("vg_direct_noalloc: ") + what + ": " + cudaGetErrorString(e));
}

}  // namespace

}  // namespace vg

extern "C" vg_status vg_direct_noalloc(void* stream, int kind, const float* pos_size, const float* angvel, size_t n,
                                       const float* q4, size_t m, float spread_range, float spread_circ,
                                       float* out4) {
  using namespace vg;
  if (kind != 0 && kind != 1) return set_noctx_error(VG_INVALID, "vg_direct_noalloc: kind must be 0 or 1");
  if (m == 0) return VG_OK;
  if (!q4 || !out4 || (n && (!pos_size || !angvel)))
    return set_noctx_error(VG_INVALID, "vg_direct_noalloc: NULL pointer");
  if (n > kNoAllocMaxSources)
    return set_noctx_error(VG_TOO_LARGE, "vg_direct_noalloc: more than 32768 sources (the fixed scratch holds "
                                         "32768 sources' constants); use vg_direct_device");
  if (m > 0x7fffffff) return set_noctx_error(VG_TOO_LARGE, "vg_direct_noalloc: more than 2^31 targets");
  const size_t src_bytes = ((n * sizeof(float4) + 255) / 256) * 256;
  const size_t room = kNoAllocScratchBytes - 2 * src_bytes;
  if (m * 3 * sizeof(float) > room)
    return set_noctx_error(VG_TOO_LARGE, "vg_direct_noalloc: too many targets for the fixed 8 MiB scratch "
                                         "(at most (8 MiB - 32 n) / 12 targets); use vg_direct_device");
  // The array's device address on the current device.  Host code holds only
  // a stand-in for the symbol; the address is looked up on every call (it
  // allocates nothing), so it stays right after cudaDeviceReset or a change
  // of context.  On a device where this library's device code is not loaded
  // yet, the lookup loads it: make the first call on each device before any
  // stream capture.
  void* base = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&base, g_noalloc_scratch);
  if (e != cudaSuccess || !base) return noalloc_fail(e, "cudaGetSymbolAddress");
  cudaStream_t st = (cudaStream_t)stream;
  if (n == 0) {
    e = cudaMemsetAsync(out4, 0, m * sizeof(float4), st);
    return e == cudaSuccess ? VG_OK : noalloc_fail(e, "cudaMemsetAsync");
  }
  // The kernels and the split of vg_direct_device, with the split capped so
  // the partial sums fit the array: wherever the cap does not bind, the
  // results are bit-identical to vg_direct_device's.
  unsigned tblocks = 0, ksplit = 0;
  int chunk = 0;
  PairPlan P = {};
  if (kind == 0) {
    P = plan_pair(n, m, nullptr);
    while (P.gen_ks > 1 && (size_t)P.gen_ks * m * 3 * sizeof(float) > room) {
      const int k = P.gen_ks - 1;
      P.gen_chunk = (int)((n + k - 1) / k);
      P.gen_ks = (int)((n + P.gen_chunk - 1) / P.gen_chunk);
    }
  } else {
    chunk = direct_split(kind, n, m, &tblocks, &ksplit);
    while (ksplit > 1 && (size_t)ksplit * m * 3 * sizeof(float) > room) {
      const unsigned k = ksplit - 1;
      chunk = (int)((n + k - 1) / k);
      ksplit = (unsigned)((n + chunk - 1) / chunk);
    }
  }
  float4* s0 = (float4*)base;
  float4* s1 = (float4*)((char*)base + src_bytes);
  float* partial = (float*)((char*)base + 2 * src_bytes);
  // Every scratch byte read below is written earlier in this call, so nothing
  // needs clearing between calls.
  const float4* ps = (const float4*)pos_size;
  const float4* w = (const float4*)angvel;
  const float4* q = (const float4*)q4;
  float4* out = (float4*)out4;
  if (kind == 0) {
    auto launch = [st](dim3 g, dim3 b, auto kernel, auto... args) { return launch_plain(st, g, b, kernel, args...); };
    e = launch_pair_plan(launch, P, ps, w, (int)n, spread_range, spread_circ, q, partial, out, nullptr);
    if (e != cudaSuccess) return noalloc_fail(e, "k_direct_pair / k_reduce_pair launch");
    return VG_OK;
  }
  e = launch_plain(st, dim3(blocks_for(n, 256)), dim3(256), k_prep_sources<1>, ps, w, (int)n, spread_range,
                   spread_circ, s0, s1);
  if (e != cudaSuccess) return noalloc_fail(e, "k_prep_sources launch");
  e = launch_plain(st, dim3(tblocks, ksplit), dim3(kThreads), k_direct_fast<1>, (const float4*)s0, (const float4*)s1,
                   (int)n, chunk, q, (int)m, partial);
  if (e != cudaSuccess) return noalloc_fail(e, "k_direct_fast launch");
  e = launch_plain(st, dim3(blocks_for(m, 256)), dim3(256), k_reduce_partials, (const float*)partial, (int)ksplit,
                   (int)m, out);
  if (e != cudaSuccess) return noalloc_fail(e, "k_reduce_partials launch");
  return VG_OK;
}
