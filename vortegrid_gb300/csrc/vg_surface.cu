// Density grid, its gradient, baroclinic generation and the signed distance
// grid of a heavy fluid: the reference's grid path for buoyancy and surface
// tracking.
//
//  * k_density      -- VortonSim::PopulateDensityAndMassFractionGrids,
//                      density part (VortonFluid/vortonSim.cpp:2911-3016):
//                      gather form of UniformGrid<float>::Accumulate
//                      (uniformGrid.h:1278-1342) -- each point merges the
//                      vortons of its 8 cells in ascending index, the order
//                      in which the reference's loop adds them -- for the
//                      density and for the unit contribution grid, then the
//                      ambient fill of that point;
//  * k_gradient     -- ComputeGradient (Core/SpatialPartition/
//                      uniformGridMath.cpp:468-503, 650-800): centred
//                      differences inside, one-sided on the faces;
//  * k_baroclinic   -- GenerateBaroclinicVorticitySlice (vortonSim.cpp:
//                      3318-3392) on the density-grid path of
//                      GenerateBaroclinicVorticity (vortonSim.cpp:3520-3547);
//  * signed distance -- PopulateSignedDistanceGridFromDensityGrid
//                      (vortonSim.cpp:3266-3290) with
//                      ComputeImmediateSDFFromDensity_Nearest and
//                      ComputeRemainingSDFFromImmediateSDF_Nearest
//                      (Particles/Operation/pclOpEmit.cpp:696-1060).  The
//                      immediate pass is a gather: each point applies the
//                      candidates of its incident crossing edges in the order
//                      the reference's cell loop visits them.  Each sweep of
//                      the remaining pass updates a point from its three
//                      backward neighbours only, which all lie on the
//                      previous diagonal plane (x + y + z one less), so tiles
//                      on one diagonal of tiles run in parallel, each walking
//                      its own diagonal planes in order: the serial sweep's
//                      result, bit for bit.
// Arithmetic the reference performs in FP32 is written with round-to-nearest
// intrinsics in its order.
#include <float.h>

#include "vg_internal.cuh"

namespace vg {

namespace {

// Clamp0to1 (vec3.h:565-571).
__device__ __forceinline__ float clamp01(float t) {
  const float lo = t > 0.0f ? t : 0.0f;
  return lo < 1.0f ? lo : 1.0f;
}

// kDeviation: the density deviation grid of PopulateDensityDeviationGridFromParticles
// (Particles/Operation/pclOpEmit.cpp:29-57) instead -- each vorton's density minus the
// ambient, accumulated alone, with no contribution grid and no fill.
template <bool kDeviation>
__global__ void __launch_bounds__(128) k_density(Geom g, const float4* __restrict__ ps,
                                                 const float* __restrict__ dens, const unsigned* __restrict__ start,
                                                 const unsigned* __restrict__ items, float ambient,
                                                 float* __restrict__ out) {
  pdl_entry();
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= g.points()) return;
  // volume ratio: first vorton's volume pi/6 size^3 (Particles/particle.h:225-228) / cell volume
  const float s0 = ps[0].w;
  const float pi_over_6 = __fdiv_rn(3.1415926535897932384626433832795f, 6.0f);
  const float vorton_volume = __fmul_rn(__fmul_rn(__fmul_rn(pi_over_6, s0), s0), s0);
  const float one_over_cell_volume = __fdiv_rn(1.0f, __fmul_rn(__fmul_rn(g.cell[0], g.cell[1]), g.cell[2]));
  const float volume_ratio = __fmul_rn(vorton_volume, one_over_cell_volume);
  const unsigned nx = g.np[0], ny = g.np[1];
  const unsigned X = (unsigned)(k % nx), Y = (unsigned)((k / nx) % ny), Z = (unsigned)(k / ((size_t)nx * ny));
  unsigned cur[8], end[8];
#pragma unroll
  for (int o = 0; o < 8; ++o) {
    const unsigned ox = o & 1, oy = (o >> 1) & 1, oz = (o >> 2) & 1;
    cur[o] = end[o] = 0;
    if (X >= ox && Y >= oy && Z >= oz) {
      const size_t c = (X - ox) + (size_t)nx * ((Y - oy) + (size_t)ny * (Z - oz));
      cur[o] = start[c];
      end[o] = start[c + 1];
    }
  }
  float d = 0.f, contrib = 0.f;
  for (;;) {
    unsigned best = 0xffffffffu;
    int bo = -1;
#pragma unroll
    for (int o = 0; o < 8; ++o) {
      if (cur[o] < end[o]) {
        const unsigned v = items[cur[o]];
        if (v < best) {
          best = v;
          bo = o;
        }
      }
    }
    if (bo < 0) break;
    cur[bo]++;
    const float4 p = ps[best];
    const float pp[3] = {p.x, p.y, p.z};
    float tw[3], om[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const unsigned idx = bin_axis(pp[a], g.mn[a], g.cpe[a]);
      const float cmin = __fadd_rn(g.mn[a], __fmul_rn((float)idx, g.cell[a]));
      tw[a] = clamp01(__fmul_rn(__fsub_rn(pp[a], cmin), g.cpe[a]));
      om[a] = __fsub_rn(1.0f, tw[a]);
    }
    // this point is corner `bo` of the vorton's cell
    const float wt = __fmul_rn(__fmul_rn((bo & 1) ? tw[0] : om[0], (bo & 2) ? tw[1] : om[1]), (bo & 4) ? tw[2] : om[2]);
    const float item = kDeviation ? __fsub_rn(dens[best], ambient) : __fmul_rn(dens[best], volume_ratio);
    d = __fadd_rn(d, __fmul_rn(wt, item));
    contrib = __fadd_rn(contrib, __fmul_rn(wt, 1.0f));
  }
  if (kDeviation) {
    out[k] = d;
    return;
  }
  // ambient fills what the vortons do not (vortonSim.cpp:3010-3014)
  const float pcls = __fmul_rn(contrib, volume_ratio);
  const float clamped = pcls < 1.0f ? pcls : 1.0f;
  out[k] = __fadd_rn(d, __fmul_rn(__fsub_rn(1.0f, clamped), ambient));
}

__global__ void k_density_ambient(size_t pts, float ambient, float* __restrict__ out) {
  pdl_entry();
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < pts) out[k] = __fmul_rn(1.0f, ambient);
}

__global__ void k_gradient(Geom g, const float* __restrict__ v, float* __restrict__ grad3) {
  pdl_entry();
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= g.points()) return;
  const unsigned nx = g.np[0], ny = g.np[1];
  const unsigned id[3] = {(unsigned)(k % nx), (unsigned)((k / nx) % ny), (unsigned)(k / ((size_t)nx * ny))};
  const size_t st[3] = {1, nx, (size_t)nx * ny};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float rs = (a < 2 || g.cell[2] > FLT_EPSILON) ? __fdiv_rn(1.0f, g.cell[a]) : 0.0f;
    const float hrs = __fmul_rn(rs, 0.5f);
    float d;
    if (id[a] == 0)
      d = __fmul_rn(__fsub_rn(v[k + st[a]], v[k]), rs);
    else if (id[a] == g.np[a] - 1)
      d = __fmul_rn(__fsub_rn(v[k], v[k - st[a]]), rs);
    else
      d = __fmul_rn(__fsub_rn(v[k + st[a]], v[k - st[a]]), hrs);
    grad3[3 * k + a] = d;
  }
}

__global__ void k_baroclinic(Geom g, const float* __restrict__ grad3, const float4* __restrict__ ps,
                             float4* __restrict__ w, int n, float pgx, float pgy, float pgz, float dt,
                             int* __restrict__ flag) {
  pdl_entry();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p = ps[i];
  if (!inside_cells(g, p.x, p.y, p.z)) {
    atomicOr(flag, (int)DF_OUT_OF_GRID);
    return;
  }
  float d[3];
  interp<3>(g, grad3, p.x, p.y, p.z, d);
  if (!(isfinite(d[0]) && isfinite(d[1]) && isfinite(d[2]))) return;
  // densityGradient ^ (gravAccel * (1 / ambient density)), then angvel += 0.5 b dt (vortonSim.cpp:3372-3378)
  const float bx = __fsub_rn(__fmul_rn(d[1], pgz), __fmul_rn(d[2], pgy));
  const float by = __fsub_rn(__fmul_rn(d[2], pgx), __fmul_rn(d[0], pgz));
  const float bz = __fsub_rn(__fmul_rn(d[0], pgy), __fmul_rn(d[1], pgx));
  float4 a = w[i];
  a.x = __fadd_rn(a.x, __fmul_rn(__fmul_rn(bx, 0.5f), dt));
  a.y = __fadd_rn(a.y, __fmul_rn(__fmul_rn(by, 0.5f), dt));
  a.z = __fadd_rn(a.z, __fmul_rn(__fmul_rn(bz, 0.5f), dt));
  w[i] = a;
}

// ------------------------------------------------------------ signed distance

// FindValueStats (uniformGridMath.cpp:554-590) with the reference's float sums
// in point order: one thread, the exact rounding of the serial loop.
__global__ void k_stats_serial(const float* __restrict__ v, size_t n, float* __restrict__ st) {
  pdl_entry();
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  float lo = FLT_MAX, hi = -FLT_MAX, s = 0.f, s2 = 0.f;
  for (size_t i = 0; i < n; ++i) {
    const float x = v[i];
    lo = x < lo ? x : lo;  // Min2(value, valMin)
    hi = x > hi ? x : hi;
    s = __fadd_rn(s, x);
    s2 = __fadd_rn(s2, __fmul_rn(x, x));
  }
  st[0] = lo;
  st[1] = hi;
  st[2] = s;
  st[3] = s2;
  st[5] = 0.0f;  // the serial float sums
}

// The same statistics from a parallel reduction: min and max exactly, the sums
// in FP64 (one partial per block, added in block order by k_stats_finish).
constexpr int kStatThreads = 256;
__global__ void __launch_bounds__(kStatThreads) k_stats_blocks(const float* __restrict__ v, size_t n,
                                                              double* __restrict__ part) {
  pdl_entry();
  __shared__ double sh_s[kStatThreads], sh_s2[kStatThreads];
  __shared__ float sh_lo[kStatThreads], sh_hi[kStatThreads];
  float lo = FLT_MAX, hi = -FLT_MAX;
  double s = 0.0, s2 = 0.0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float x = v[i];
    lo = fminf(lo, x);
    hi = fmaxf(hi, x);
    s += (double)x;
    s2 += (double)x * (double)x;
  }
  sh_s[threadIdx.x] = s;
  sh_s2[threadIdx.x] = s2;
  sh_lo[threadIdx.x] = lo;
  sh_hi[threadIdx.x] = hi;
  __syncthreads();
  for (int h = kStatThreads / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) {
      sh_s[threadIdx.x] += sh_s[threadIdx.x + h];
      sh_s2[threadIdx.x] += sh_s2[threadIdx.x + h];
      sh_lo[threadIdx.x] = fminf(sh_lo[threadIdx.x], sh_lo[threadIdx.x + h]);
      sh_hi[threadIdx.x] = fmaxf(sh_hi[threadIdx.x], sh_hi[threadIdx.x + h]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[4 * blockIdx.x] = sh_s[0];
    part[4 * blockIdx.x + 1] = sh_s2[0];
    part[4 * blockIdx.x + 2] = sh_lo[0];
    part[4 * blockIdx.x + 3] = sh_hi[0];
  }
}

__global__ void k_stats_finish(const double* __restrict__ part, int nb, size_t n, float* __restrict__ st) {
  pdl_entry();
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double s = 0.0, s2 = 0.0;
  float lo = FLT_MAX, hi = -FLT_MAX;
  for (int b = 0; b < nb; ++b) {
    s += part[4 * b];
    s2 += part[4 * b + 1];
    lo = fminf(lo, (float)part[4 * b + 2]);
    hi = fmaxf(hi, (float)part[4 * b + 3]);
  }
  st[0] = lo;
  st[1] = hi;
  st[3] = (float)(s2 / (double)n);  // mean of squares
  st[4] = (float)(s / (double)n);   // mean
  st[5] = 1.0f;                     // the FP64 sums
}

// densityInside - densityOutside from the statistics (pclOpEmit.cpp:714-723,
// uniformGridMath.cpp:582-589).  st: [0] min, [1] max, then either [2] sum and
// [3] sum of squares as floats ([5] = 0), or [3] mean of squares and [4] mean
// from FP64 sums ([5] = 1).
__device__ __forceinline__ float sdf_denominator(const float* __restrict__ st, size_t n, float ambient) {
  float mean, mean2;
  if (st[5] == 1.0f) {
    mean = st[4];
    mean2 = st[3];
  } else {
    mean = __fdiv_rn(st[2], (float)n);
    mean2 = __fdiv_rn(st[3], (float)n);
  }
  const float variance = __fsub_rn(mean2, __fmul_rn(mean, mean));
  const float sd = __fsqrt_rn(variance > 0.0f ? variance : 0.0f);
  const float m_sd = __fadd_rn(mean, sd);
  const float inside = st[1] < m_sd ? st[1] : m_sd;  // Min2(densityMax, mean + stddev)
  return __fsub_rn(inside, ambient);
}

// The candidates a crossing edge (q, q + axis) gives its two end points
// (pclOpEmit.cpp:760-842).  Returns false where the edge does not cross.
__device__ __forceinline__ bool edge_candidates(float dq, float dn, float denom, float cell, float& cq, float& cn) {
  if (dq <= 0.0f && 0.0f < dn) {
    const float t0 = __fdiv_rn(dn, denom);
    const float t = t0 < 1.0f ? t0 : 1.0f;
    cq = __fmul_rn(__fsub_rn(1.0f, t), cell);
    cn = __fmul_rn(-t, cell);
    return true;
  }
  if (dq > 0.0f && 0.0f >= dn) {
    const float t0 = __fdiv_rn(dq, denom);
    const float t = t0 < 1.0f ? t0 : 1.0f;
    cq = __fmul_rn(-t, cell);
    cn = __fmul_rn(__fsub_rn(1.0f, t), cell);
    return true;
  }
  return false;
}

__device__ __forceinline__ void update_sdf(float& here, float cand) {
  if (fabsf(cand) < fabsf(here)) here = cand;
}

// Immediate SDF at point p: the candidates of the crossing edges at p, in the
// order of the reference's cell loop (cells in z, y, x order, each cell's +x,
// +y, +z edges in turn): the +z edge of the cell below in z, the +y edge of
// the cell below in y, the +x edge of the cell below in x, then p's own +x,
// +y, +z edges.  Only cells with every index below the point count on that
// axis minus one are visited.
__global__ void k_sdf_immediate(Geom g, const float* __restrict__ dens, float ambient, const float* __restrict__ st,
                                float* __restrict__ sdf, unsigned char* __restrict__ pinned) {
  pdl_entry();
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t pts = g.points();
  if (k >= pts) return;
  const float denom = sdf_denominator(st, pts, ambient);
  const unsigned nx = g.np[0], ny = g.np[1], nz = g.np[2];
  const unsigned x = (unsigned)(k % nx), y = (unsigned)((k / nx) % ny), z = (unsigned)(k / ((size_t)nx * ny));
  const size_t nxy = (size_t)nx * ny;
  float here = FLT_MAX;
  bool pin = false;
  float cq, cn;
  const float dk = __fsub_rn(dens[k], ambient);
  // as the far end of an edge of a cell behind it
  if (z >= 1 && x + 1 < nx && y + 1 < ny &&
      edge_candidates(__fsub_rn(dens[k - nxy], ambient), dk, denom, g.cell[2], cq, cn)) {
    pin = true;
    update_sdf(here, cn);
  }
  if (y >= 1 && x + 1 < nx && z + 1 < nz &&
      edge_candidates(__fsub_rn(dens[k - nx], ambient), dk, denom, g.cell[1], cq, cn)) {
    pin = true;
    update_sdf(here, cn);
  }
  if (x >= 1 && y + 1 < ny && z + 1 < nz &&
      edge_candidates(__fsub_rn(dens[k - 1], ambient), dk, denom, g.cell[0], cq, cn)) {
    pin = true;
    update_sdf(here, cn);
  }
  // as the near end of its own cell's edges
  if (x + 1 < nx && y + 1 < ny && z + 1 < nz) {
    const size_t nb[3] = {k + 1, k + nx, k + nxy};
#pragma unroll
    for (int a = 0; a < 3; ++a)
      if (edge_candidates(dk, __fsub_rn(dens[nb[a]], ambient), denom, g.cell[a], cq, cn)) {
        pin = true;
        update_sdf(here, cq);
      }
  }
  sdf[k] = here;
  pinned[k] = pin ? 1 : 0;
}

// One sweep of ComputeRemainingSDFFromImmediateSDF_Nearest over the tiles on
// tile diagonal `diag` (forward: inc +1 on every axis; backward: -1).  A CTA
// owns one kSdfTile^3 tile: it stages the tile and its three backward faces
// (tiles of earlier diagonals, final for this sweep) in shared memory, walks
// the tile's local diagonal planes there in order, and writes the tile back.
// The points, their neighbours and the updates are those of the serial sweep,
// in an order that respects every dependence, so the result is its own bit
// for bit.
constexpr int kSdfTile = 16;
constexpr int kSdfThreads = kSdfTile * kSdfTile;  // one thread per (j, k) of a local diagonal plane
__global__ void __launch_bounds__(kSdfThreads) k_sdf_sweep(Geom g, int diag, int backward, unsigned tiles_x,
                                                           float* __restrict__ sdf,
                                                           const unsigned char* __restrict__ pinned) {
  pdl_entry();
  constexpr int T = kSdfTile, E = kSdfTile + 1;  // staged extent: the tile plus one backward layer
  __shared__ float S[E * E * E];                 // S[(w + 1) E^2 + (v + 1) E + (u + 1)], u, v, w in [-1, T)
  __shared__ unsigned char pin[T * T * T];
  const int ty = blockIdx.x, tz = blockIdx.y;
  const int tx = diag - ty - tz;
  if (tx < 0 || tx >= (int)tiles_x) return;
  const int nx = g.np[0], ny = g.np[1], nz = g.np[2];
  const long long sy = nx, sz = (long long)nx * ny;
  // tile origin in sweep coordinates (distance from the sweep's first point)
  const int ox = tx * T, oy = ty * T, oz = tz * T;
  auto gidx = [&](int u, int v, int w) -> long long {
    const int x = backward ? nx - 1 - u : u, y = backward ? ny - 1 - v : v, z = backward ? nz - 1 - w : w;
    return x + sy * y + sz * z;
  };
  // stage: the tile (u, v, w in [0, T)) and the backward faces (one of u, v, w = -1, the others in
  // [0, T)); a neighbour before the grid's first point reads FLT_MAX, as in the serial sweep
  // all of a thread's loads are issued before any is stored, so the staging
  // costs one memory latency rather than one per element
  constexpr int kStage = (E * E * E + kSdfThreads - 1) / kSdfThreads;
  float val[kStage];
  unsigned char pv[kStage];
#pragma unroll
  for (int q = 0; q < kStage; ++q) {
    const int t = threadIdx.x + q * kSdfThreads;
    val[q] = FLT_MAX;
    pv[q] = 0;
    if (t >= E * E * E) continue;
    const int lu = t % E - 1, lv = (t / E) % E - 1, lw = t / (E * E) - 1;
    if ((lu < 0) + (lv < 0) + (lw < 0) > 1) continue;  // edges and corners of the backward layer are never read
    const int u = ox + lu, v = oy + lv, w = oz + lw;
    if (u >= 0 && v >= 0 && w >= 0 && u < nx && v < ny && w < nz) {
      const long long o = gidx(u, v, w);
      val[q] = sdf[o];
      pv[q] = pinned[o];
    }
  }
#pragma unroll
  for (int q = 0; q < kStage; ++q) {
    const int t = threadIdx.x + q * kSdfThreads;
    if (t >= E * E * E) continue;
    S[t] = val[q];
    const int lu = t % E - 1, lv = (t / E) % E - 1, lw = t / (E * E) - 1;
    if (lu >= 0 && lv >= 0 && lw >= 0) pin[lu + T * (lv + T * lw)] = pv[q];
  }
  __syncthreads();
  const int j = threadIdx.x % T, kk = threadIdx.x / T;
  for (int s = 0; s <= 3 * (T - 1); ++s) {
    // points (i, j, k) of the tile with i + j + k = s
    const int i = s - j - kk;
    if (i >= 0 && i < T) {
      const int u = ox + i, v = oy + j, w = oz + kk;
      if (u < nx && v < ny && w < nz && !pin[i + T * (j + T * kk)]) {
        const int c = (kk + 1) * E * E + (j + 1) * E + (i + 1);
        const float sx = S[c - 1], syv = S[c - E], szv = S[c - E * E];
        const float ax = fabsf(sx), ay = fabsf(syv), az = fabsf(szv);
        float nb, sp;
        if (ax <= ay) {
          if (ax <= az) {
            nb = sx;
            sp = g.cell[0];
          } else {
            nb = szv;
            sp = g.cell[2];
          }
        } else if (ay <= az) {
          nb = syv;
          sp = g.cell[1];
        } else {
          nb = szv;
          sp = g.cell[2];
        }
        float here = S[c];
        update_sdf(here, __fadd_rn(nb, copysignf(sp, nb)));
        S[c] = here;
      }
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < T * T * T; t += kSdfThreads) {
    const int li = t % T, lj = (t / T) % T, lk = t / (T * T);
    const int u = ox + li, v = oy + lj, w = oz + lk;
    if (u < nx && v < ny && w < nz && !pin[t]) sdf[gidx(u, v, w)] = S[(lk + 1) * E * E + (lj + 1) * E + (li + 1)];
  }
}

__global__ void k_sdf_unreached(size_t pts, float* __restrict__ sdf) {
  pdl_entry();
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < pts && sdf[k] == FLT_MAX) sdf[k] = __int_as_float(0x7fc00000);
}

// ------------------------------------------------------------ marching cubes

// The cell's triangulation by case (bit c: corner c below the iso level):
// triangle count and up to 5 edge triples.  Generated on the host by
// mc_generate below.
struct MCTable {
  unsigned char cnt[256];
  signed char tri[256][15];
};

// Corner offsets and edges (corner pairs in the order the reference
// interpolates them, Render/Resource/marchingCubes.cpp:590-622, 800-816).
__host__ __device__ __forceinline__ int mc_corner(int c, int k) {
  // corners 0..7: (0,0,0) (1,0,0) (1,1,0) (0,1,0) (0,0,1) (1,0,1) (1,1,1) (0,1,1)
  return k == 0 ? (((c + 1) >> 1) & 1) : (k == 1 ? ((c >> 1) & 1) : ((c >> 2) & 1));
}
__host__ __device__ __forceinline__ int mc_edge_a(int e) { return e < 8 ? e : e - 8; }
__host__ __device__ __forceinline__ int mc_edge_b(int e) { return e < 8 ? ((e & 4) | ((e + 1) & 3)) : e - 4; }

// VertexInterp (marchingCubes.cpp:228-250): an end point within 1e-5
// (compared in double, as the reference's double literal makes it), else
// p1 + mu (p2 - p1).
__device__ __forceinline__ void mc_interp(float iso, const float* p1, const float* p2, float v1, float v2,
                                          float* out) {
  if ((double)fabsf(__fsub_rn(iso, v1)) < 0.00001) {
    out[0] = p1[0], out[1] = p1[1], out[2] = p1[2];
  } else if ((double)fabsf(__fsub_rn(iso, v2)) < 0.00001) {
    out[0] = p2[0], out[1] = p2[1], out[2] = p2[2];
  } else if ((double)fabsf(__fsub_rn(v1, v2)) < 0.00001) {
    out[0] = p1[0], out[1] = p1[1], out[2] = p1[2];
  } else {
    const float mu = __fdiv_rn(__fsub_rn(iso, v1), __fsub_rn(v2, v1));
#pragma unroll
    for (int k = 0; k < 3; ++k) out[k] = __fadd_rn(p1[k], __fmul_rn(mu, __fsub_rn(p2[k], p1[k])));
  }
}

__device__ __forceinline__ int mc_mask(const Geom& g, const float* __restrict__ v, size_t o, float iso,
                                       float* val) {
  const size_t nx = g.np[0], nxy = (size_t)g.np[0] * g.np[1];
  int mask = 0;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    val[c] = v[o + mc_corner(c, 0) + nx * mc_corner(c, 1) + nxy * mc_corner(c, 2)];
    if (val[c] < iso) mask |= 1 << c;
  }
  return mask;
}

__global__ void k_mc_count(Geom g, const float* __restrict__ v, float iso, const __grid_constant__ MCTable T,
                           unsigned* __restrict__ counts) {
  pdl_entry();
  const size_t cx = g.np[0] - 1, cy = g.np[1] - 1, cells = cx * cy * (g.np[2] - 1);
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= cells) return;
  const size_t x = k % cx, y = (k / cx) % cy, z = k / (cx * cy);
  float val[8];
  counts[k] = T.cnt[mc_mask(g, v, x + g.np[0] * (y + (size_t)g.np[1] * z), iso, val)];
}

__global__ void k_mc_emit(Geom g, const float* __restrict__ v, float iso, const __grid_constant__ MCTable T,
                          const unsigned* __restrict__ offsets, float* __restrict__ verts,
                          float* __restrict__ normals) {
  pdl_entry();
  const size_t cx = g.np[0] - 1, cy = g.np[1] - 1, cells = cx * cy * (g.np[2] - 1);
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= cells) return;
  const unsigned x = (unsigned)(k % cx), y = (unsigned)((k / cx) % cy), z = (unsigned)(k / (cx * cy));
  float val[8];
  const int mask = mc_mask(g, v, x + g.np[0] * (y + (size_t)g.np[1] * z), iso, val);
  const int nt = T.cnt[mask];
  if (nt == 0) return;
  // corner positions min + index x spacing (marchingCubes.cpp:806-816)
  const float lo[3] = {__fadd_rn(__fmul_rn((float)x, g.cell[0]), g.mn[0]),
                       __fadd_rn(__fmul_rn((float)y, g.cell[1]), g.mn[1]),
                       __fadd_rn(__fmul_rn((float)z, g.cell[2]), g.mn[2])};
  const float hi[3] = {__fadd_rn(lo[0], g.cell[0]), __fadd_rn(lo[1], g.cell[1]), __fadd_rn(lo[2], g.cell[2])};
  float vl[12][3];
#pragma unroll
  for (int e = 0; e < 12; ++e) {
    const int a = mc_edge_a(e), b = mc_edge_b(e);
    if (((mask >> a) & 1) != ((mask >> b) & 1)) {
      float pa[3], pb[3];
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        pa[q] = mc_corner(a, q) ? hi[q] : lo[q];
        pb[q] = mc_corner(b, q) ? hi[q] : lo[q];
      }
      mc_interp(iso, pa, pb, val[a], val[b], vl[e]);
    }
  }
  size_t out = offsets[k];
  for (int t = 0; t < nt; ++t, ++out) {
    const float* q0 = vl[T.tri[mask][3 * t]];
    const float* q1 = vl[T.tri[mask][3 * t + 1]];
    const float* q2 = vl[T.tri[mask][3 * t + 2]];
    float* d = verts + 9 * out;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      d[q] = q0[q];
      d[3 + q] = q1[q];
      d[6 + q] = q2[q];
    }
    if (normals) {
      // face normal (p1 - p0) x (p2 - p0) scaled by 1 / sqrt(|n|^2 + FLT_MIN) (vec3.h:428)
      const float u[3] = {__fsub_rn(q1[0], q0[0]), __fsub_rn(q1[1], q0[1]), __fsub_rn(q1[2], q0[2])};
      const float w[3] = {__fsub_rn(q2[0], q0[0]), __fsub_rn(q2[1], q0[1]), __fsub_rn(q2[2], q0[2])};
      const float n[3] = {__fsub_rn(__fmul_rn(u[1], w[2]), __fmul_rn(u[2], w[1])),
                          __fsub_rn(__fmul_rn(u[2], w[0]), __fmul_rn(u[0], w[2])),
                          __fsub_rn(__fmul_rn(u[0], w[1]), __fmul_rn(u[1], w[0]))};
      const float m2 = __fadd_rn(__fadd_rn(__fmul_rn(n[0], n[0]), __fmul_rn(n[1], n[1])), __fmul_rn(n[2], n[2]));
      const float r = __fdiv_rn(1.0f, __fsqrt_rn(__fadd_rn(m2, FLT_MIN)));
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        normals[9 * out + 3 * q] = __fmul_rn(n[0], r);
        normals[9 * out + 3 * q + 1] = __fmul_rn(n[1], r);
        normals[9 * out + 3 * q + 2] = __fmul_rn(n[2], r);
      }
    }
  }
}

// The triangulation of every case: on each cube face the crossing edges are
// joined into segments (where a face has four crossings, each segment cuts
// off one corner below the iso level, which keeps neighbouring cells'
// surfaces joined), each segment oriented so that the corners below the iso
// level lie on one fixed side seen from outside the cell; segments chain into
// loops, each fanned from its first edge.  Normals of the triangles point
// away from the corners below the iso level.
MCTable mc_generate() {
  static const int face[6][5] = {{0, 1, 2, 3, -3}, {4, 5, 6, 7, 3}, {0, 1, 5, 4, -2},
                                 {3, 2, 6, 7, 2},  {0, 3, 7, 4, -1}, {1, 2, 6, 5, 1}};  // corners, +-axis
  auto edge_of = [](int a, int b) {
    for (int e = 0; e < 12; ++e)
      if ((mc_edge_a(e) == a && mc_edge_b(e) == b) || (mc_edge_a(e) == b && mc_edge_b(e) == a)) return e;
    return -1;
  };
  // sign of ((B - A) x (P - A)) . n for edge midpoints A, B and corner P (doubled coordinates)
  auto side = [](int a, int b, int pin, int ax) {
    int u[3], w[3];
    for (int k = 0; k < 3; ++k) {
      const int A = mc_corner(mc_edge_a(a), k) + mc_corner(mc_edge_b(a), k);
      const int B = mc_corner(mc_edge_a(b), k) + mc_corner(mc_edge_b(b), k);
      u[k] = B - A;
      w[k] = 2 * mc_corner(pin, k) - A;
    }
    const int cr[3] = {u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2], u[0] * w[1] - u[1] * w[0]};
    const int axis = (ax > 0 ? ax : -ax) - 1;
    return ax > 0 ? cr[axis] : -cr[axis];
  };
  MCTable T;
  for (int m = 0; m < 256; ++m) {
    int next[12];
    for (int e = 0; e < 12; ++e) next[e] = -1;
    for (int f = 0; f < 6; ++f) {
      const int* cc = face[f];
      int ee[4], cr[4], nc = 0;
      for (int k = 0; k < 4; ++k) {
        ee[k] = edge_of(cc[k], cc[(k + 1) % 4]);
        if (((m >> cc[k]) & 1) != ((m >> cc[(k + 1) % 4]) & 1)) cr[nc++] = k;
      }
      int seg[2][3], ns = 0;
      if (nc == 2) {
        int pin = -1;
        for (int k = 0; k < 4 && pin < 0; ++k)
          if ((m >> cc[k]) & 1) pin = cc[k];
        seg[0][0] = ee[cr[0]], seg[0][1] = ee[cr[1]], seg[0][2] = pin;
        ns = 1;
      } else if (nc == 4) {
        for (int k = 0; k < 4; ++k)
          if ((m >> cc[k]) & 1) {
            seg[ns][0] = ee[(k + 3) % 4], seg[ns][1] = ee[k], seg[ns][2] = cc[k];
            ++ns;
          }
      }
      for (int s = 0; s < ns; ++s) {
        if (side(seg[s][0], seg[s][1], seg[s][2], cc[4]) < 0)
          next[seg[s][0]] = seg[s][1];
        else
          next[seg[s][1]] = seg[s][0];
      }
    }
    bool seen[12] = {false};
    int nt = 0;
    for (int e = 0; e < 12; ++e) {
      if (next[e] < 0 || seen[e]) continue;
      int loop[12], n = 0, x = e;
      do {
        loop[n++] = x;
        seen[x] = true;
        x = next[x];
      } while (x != e && n < 12);
      for (int i = 1; i + 1 < n && nt < 5; ++i, ++nt) {
        T.tri[m][3 * nt] = (signed char)loop[0];
        T.tri[m][3 * nt + 1] = (signed char)loop[i];
        T.tri[m][3 * nt + 2] = (signed char)loop[i + 1];
      }
    }
    T.cnt[m] = (unsigned char)nt;
    for (int i = 3 * nt; i < 15; ++i) T.tri[m][i] = -1;
  }
  return T;
}

}  // namespace

vg_status launch_density_grid(Ctx* c, const Geom& g, const float4* ps, const float* density, size_t n,
                              float ambient, float* out) {
  const size_t pts = g.points();
  if (n == 0) {
    pdl_launch(c->stream, blocks_for(pts, 256), 256, 0, k_density_ambient, pts, ambient, out);
    VG_LAUNCHED(c);
    VG_CUDA(c, cudaGetLastError());
    return VG_OK;
  }
  CellLists cl;
  vg_status st = build_cell_lists(c, g, ps, n, &cl);
  if (st != VG_OK) return st;
  pdl_launch(c->stream, blocks_for(pts, 128), 128, 0, k_density<false>, g, ps, density, (const unsigned*)cl.start,
             (const unsigned*)cl.items, ambient, out);
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

vg_status launch_density_deviation(Ctx* c, const Geom& g, const float4* ps, const float* density, size_t n,
                                   float ambient, float* out) {
  const size_t pts = g.points();
  if (n == 0) {
    VG_CUDA(c, cudaMemsetAsync(out, 0, pts * sizeof(float), c->stream));
    return VG_OK;
  }
  CellLists cl;
  vg_status st = build_cell_lists(c, g, ps, n, &cl);
  if (st != VG_OK) return st;
  pdl_launch(c->stream, blocks_for(pts, 128), 128, 0, k_density<true>, g, ps, density, (const unsigned*)cl.start,
             (const unsigned*)cl.items, ambient, out);
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

vg_status launch_gradient(Ctx* c, const Geom& g, const float* v, float* grad3) {
  pdl_launch(c->stream, blocks_for(g.points(), 256), 256, 0, k_gradient, g, v, grad3);
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

vg_status launch_baroclinic(Ctx* c, const Geom& g, const float* grad3, const float4* ps, float4* w, size_t n,
                            const float grav[3], float ambient, float dt) {
  if (n == 0) return VG_OK;
  // gravAccel * (1 / ambient density) (vortonSim.cpp:3327, 3367-3372), host FP32
  const float one_over_density = 1.0f / ambient;
  const float pg[3] = {grav[0] * one_over_density, grav[1] * one_over_density, grav[2] * one_over_density};
  pdl_launch(c->stream, blocks_for(n, 256), 256, 0, k_baroclinic, g, grad3, ps, w, (int)n, pg[0], pg[1], pg[2], dt,
             outside_flag(c));
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

vg_status launch_signed_distance(Ctx* c, const Geom& g, const float* dens, float ambient, bool reference_stats,
                                 float* sdf, unsigned char* pinned, float* stats, double* partials,
                                 int partial_blocks) {
  const size_t pts = g.points();
  if (reference_stats) {
    pdl_launch(c->stream, 1, 1, 0, k_stats_serial, dens, pts, stats);
    VG_LAUNCHED(c);
  } else {
    pdl_launch(c->stream, partial_blocks, kStatThreads, 0, k_stats_blocks, dens, pts, partials);
    pdl_launch(c->stream, 1, 1, 0, k_stats_finish, (const double*)partials, partial_blocks, pts, stats);
    c->launches += 2;
  }
  pdl_launch(c->stream, blocks_for(pts, 256), 256, 0, k_sdf_immediate, g, dens, ambient, (const float*)stats, sdf,
             pinned);
  VG_LAUNCHED(c);
  const unsigned tiles[3] = {(g.np[0] + kSdfTile - 1) / kSdfTile, (g.np[1] + kSdfTile - 1) / kSdfTile,
                             (g.np[2] + kSdfTile - 1) / kSdfTile};
  const int diags = (int)(tiles[0] + tiles[1] + tiles[2]) - 2;
  for (int pass = 0; pass < 2; ++pass)
    for (int d = 0; d < diags; ++d) {
      pdl_launch(c->stream, dim3(tiles[1], tiles[2]), kSdfThreads, 0, k_sdf_sweep, g, d, pass, tiles[0], sdf,
                 (const unsigned char*)pinned);
      VG_LAUNCHED(c);
    }
  pdl_launch(c->stream, blocks_for(pts, 256), 256, 0, k_sdf_unreached, pts, sdf);
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

}  // namespace vg

namespace vg {

vg_status launch_marching_cubes(Ctx* c, const Geom& g, const float* v, float iso, float* verts, float* normals,
                                size_t cap, size_t* triangles) {
  static const MCTable T = mc_generate();
  const size_t cells = (size_t)(g.np[0] - 1) * (g.np[1] - 1) * (g.np[2] - 1);
  vg_status st = VG_OK;
  unsigned* counts = (unsigned*)ws(c, S_MC, (2 * cells + 2) * sizeof(unsigned), &st);
  if (st != VG_OK) return st;
  unsigned* offsets = counts + cells + 1;
  pdl_launch(c->stream, blocks_for(cells, 256), 256, 0, k_mc_count, g, v, iso, T, counts);
  VG_LAUNCHED(c);
  if ((st = exclusive_scan(c, counts, cells, offsets, true)) != VG_OK) return st;
  unsigned total = 0;
  VG_CUDA(c, cudaMemcpyAsync(&total, offsets + cells, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
  VG_CUDA(c, cudaStreamSynchronize(c->stream));
  *triangles = total;
  if (total > cap) return fail(c, VG_TOO_LARGE, "marching cubes: " + std::to_string(total) + " triangles, room for " +
                                                    std::to_string(cap));
  if (total == 0) return VG_OK;
  pdl_launch(c->stream, blocks_for(cells, 128), 128, 0, k_mc_emit, g, v, iso, T, (const unsigned*)offsets, verts,
             normals);
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

}  // namespace vg
