// K6-K9: vector-potential Poisson solve  L a = b  (b = -vorticity) with
// Dirichlet boundary values, to a relative-residual tolerance.
//
// The reference solves the same equation with a fixed-work cascade
// (VortonFluid/vortonSim.cpp:2539-2571) that never targets a residual; this
// is a correction-scheme multigrid in iterative refinement:
//   outer loop (FP64): r = b - L a64 computed in FP64 from the FP64 iterate,
//                      stored as FP32; ||r|| and ||b|| as FP64 sums reduced in
//                      a fixed order (deterministic);
//   inner solve (FP32): one V(pre, post)-cycle on the correction e with
//                      point red-black Gauss-Seidel (colour = (x+y+z) parity),
//                      27-point full-weighting restriction of the residual
//                      (the reference's SLOWER_MORE_ACCURATE weights,
//                      uniformGrid.h:1453-1585) and trilinear prolongation;
//   coarsest grid (FP64): red-black Gauss-Seidel run to convergence in one CTA;
//   a64 += e.
// Grids are float[3] per point (x fastest); the three components are three
// independent scalar problems solved together.
#include <float.h>

#include <algorithm>
#include <cmath>

#include "vg_internal.cuh"

namespace vg {

namespace {

constexpr int kRedThreads = 256;

struct Lev {
  Geom g;
  float r2x, r2y, r2z, H;  // FP32 operator constants
  size_t base;             // offset (points) into level arrays
};

__device__ __forceinline__ void unflat(size_t k, const Geom& g, unsigned& x, unsigned& y, unsigned& z) {
  x = (unsigned)(k % g.np[0]);
  y = (unsigned)((k / g.np[0]) % g.np[1]);
  z = (unsigned)(k / ((size_t)g.np[0] * g.np[1]));
}

__device__ __forceinline__ bool interior(const Geom& g, unsigned x, unsigned y, unsigned z) {
  return x > 0 && y > 0 && z > 0 && x + 1 < g.np[0] && y + 1 < g.np[1] && z + 1 < g.np[2];
}

// FP64 residual of the FP64 iterate; writes FP32 r (0 on the boundary) and
// per-block partial sums of r^2 and b^2.
__global__ void __launch_bounds__(kRedThreads) k_residual64(Geom g, double r2x, double r2y, double r2z,
                                                            const double* __restrict__ a, const float* __restrict__ b,
                                                            float* __restrict__ r, double* __restrict__ part) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  double rr = 0.0, bb = 0.0;
  if (k < g.points()) {
    unsigned x, y, z;
    unflat(k, g, x, y, z);
    if (interior(g, x, y, z)) {
      const size_t nx = g.np[0], nxy = (size_t)g.np[0] * g.np[1];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const double ac = a[3 * k + c];
        const double lap = (a[3 * (k + 1) + c] + a[3 * (k - 1) + c] - 2.0 * ac) * r2x +
                           (a[3 * (k + nx) + c] + a[3 * (k - nx) + c] - 2.0 * ac) * r2y +
                           (a[3 * (k + nxy) + c] + a[3 * (k - nxy) + c] - 2.0 * ac) * r2z;
        const double bv = (double)b[3 * k + c];
        const double rv = bv - lap;
        r[3 * k + c] = (float)rv;
        rr += rv * rv;
        bb += bv * bv;
      }
    } else {
      r[3 * k] = 0.f;
      r[3 * k + 1] = 0.f;
      r[3 * k + 2] = 0.f;
    }
  }
  __shared__ double s_rr[kRedThreads / 32], s_bb[kRedThreads / 32];
  for (int o = 16; o > 0; o >>= 1) {
    rr += __shfl_xor_sync(0xffffffffu, rr, o);
    bb += __shfl_xor_sync(0xffffffffu, bb, o);
  }
  if ((threadIdx.x & 31) == 0) {
    s_rr[threadIdx.x >> 5] = rr;
    s_bb[threadIdx.x >> 5] = bb;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a1 = 0.0, a2 = 0.0;
    for (int w = 0; w < kRedThreads / 32; ++w) {
      a1 += s_rr[w];
      a2 += s_bb[w];
    }
    part[2 * blockIdx.x] = a1;
    part[2 * blockIdx.x + 1] = a2;
  }
}

// Sum the per-block partials in a fixed order (one block).
__global__ void __launch_bounds__(1024) k_sum_partials(const double* __restrict__ part, int nb,
                                                       double* __restrict__ out2) {
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
    out2[1] = s2[0];
  }
}

// Point red-black Gauss-Seidel on L e = r (FP32).  One thread per x-pair:
// updates the point of `color` among (2j, 2j+1).  zero_first: e is zero
// before this sweep (first pre-smoothing sweep), so neighbours read as 0.
__global__ void __launch_bounds__(256) k_rbgs(Geom g, float r2x, float r2y, float r2z, float H,
                                              float* __restrict__ e, const float* __restrict__ r, unsigned color,
                                              int zero_first) {
  const unsigned nx = g.np[0], ny = g.np[1], nz = g.np[2];
  const unsigned half = (nx + 1) / 2;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t rows = (size_t)ny * nz;
  if (t >= rows * half) return;
  const unsigned j = (unsigned)(t % half);
  const size_t row = t / half;
  const unsigned y = (unsigned)(row % ny), z = (unsigned)(row / ny);
  if (y == 0 || z == 0 || y + 1 >= ny || z + 1 >= nz) return;
  unsigned x = 2 * j + ((y + z + color) & 1u);
  if (x == 0 || x + 1 >= nx) return;
  const size_t k = x + (size_t)nx * (y + (size_t)ny * z);
  const size_t sy = nx, sz = (size_t)nx * ny;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    float v;
    if (zero_first) {
      v = -r[3 * k + c] * H;
    } else {
      const float sx = e[3 * (k + 1) + c] + e[3 * (k - 1) + c];
      const float syv = e[3 * (k + sy) + c] + e[3 * (k - sy) + c];
      const float szv = e[3 * (k + sz) + c] + e[3 * (k - sz) + c];
      v = (fmaf(sx, r2x, fmaf(syv, r2y, szv * r2z)) - r[3 * k + c]) * H;
    }
    e[3 * k + c] = v;
  }
}

// FP32 residual res = r - L e on interior points (0 on the boundary).
__global__ void __launch_bounds__(256) k_residual32(Geom g, float r2x, float r2y, float r2z,
                                                    const float* __restrict__ e, const float* __restrict__ r,
                                                    float* __restrict__ res) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= g.points()) return;
  unsigned x, y, z;
  unflat(k, g, x, y, z);
  if (!interior(g, x, y, z)) {
    res[3 * k] = res[3 * k + 1] = res[3 * k + 2] = 0.f;
    return;
  }
  const size_t sy = g.np[0], sz = (size_t)g.np[0] * g.np[1];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float ec = e[3 * k + c];
    const float lap = (e[3 * (k + 1) + c] + e[3 * (k - 1) + c] - 2.f * ec) * r2x +
                      (e[3 * (k + sy) + c] + e[3 * (k - sy) + c] - 2.f * ec) * r2y +
                      (e[3 * (k + sz) + c] + e[3 * (k - sz) + c] - 2.f * ec) * r2z;
    res[3 * k + c] = r[3 * k + c] - lap;
  }
}

// Full-weighting restriction of the fine residual to coarse interior points.
__global__ void __launch_bounds__(256) k_restrict(Geom F, Geom C, const float* __restrict__ res,
                                                  float* __restrict__ rc) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= C.points()) return;
  unsigned x, y, z;
  unflat(k, C, x, y, z);
  if (!interior(C, x, y, z)) {
    rc[3 * k] = rc[3 * k + 1] = rc[3 * k + 2] = 0.f;
    return;
  }
  const size_t fx = 2 * x, fy = 2 * y, fz = 2 * z;
  const size_t sy = F.np[0], sz = (size_t)F.np[0] * F.np[1];
  const size_t f0 = fx + sy * fy + sz * fz;
  float a0 = 0.f, a1 = 0.f, a2 = 0.f;
#pragma unroll
  for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
      for (int dx = -1; dx <= 1; ++dx) {
        const float wt = (float)(8 >> (abs(dx) + abs(dy) + abs(dz)));
        const size_t o = f0 + dx + (ptrdiff_t)sy * dy + (ptrdiff_t)sz * dz;
        a0 = fmaf(wt, res[3 * o], a0);
        a1 = fmaf(wt, res[3 * o + 1], a1);
        a2 = fmaf(wt, res[3 * o + 2], a2);
      }
  const float s = 1.0f / 64.0f;
  rc[3 * k] = a0 * s;
  rc[3 * k + 1] = a1 * s;
  rc[3 * k + 2] = a2 * s;
}

// e_fine += trilinear(e_coarse) on fine interior points.
__global__ void __launch_bounds__(256) k_prolong_add(Geom F, Geom C, const float* __restrict__ ec,
                                                     float* __restrict__ ef) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= F.points()) return;
  unsigned x, y, z;
  unflat(k, F, x, y, z);
  if (!interior(F, x, y, z)) return;
  const unsigned cx = x >> 1, cy = y >> 1, cz = z >> 1;
  const unsigned ox = x & 1, oy = y & 1, oz = z & 1;
  const size_t sy = C.np[0], sz = (size_t)C.np[0] * C.np[1];
  const size_t c0 = cx + sy * cy + sz * cz;
  float a0 = 0.f, a1 = 0.f, a2 = 0.f;
  const float wt = 1.0f / (float)(1u << (ox + oy + oz));
  for (unsigned iz = 0; iz <= oz; ++iz)
    for (unsigned iy = 0; iy <= oy; ++iy)
      for (unsigned ix = 0; ix <= ox; ++ix) {
        const size_t o = c0 + ix + sy * iy + sz * iz;
        a0 += ec[3 * o];
        a1 += ec[3 * o + 1];
        a2 += ec[3 * o + 2];
      }
  ef[3 * k] += a0 * wt;
  ef[3 * k + 1] += a1 * wt;
  ef[3 * k + 2] += a2 * wt;
}

// Coarsest grid: FP64 red-black Gauss-Seidel to convergence, one CTA.
__global__ void __launch_bounds__(1024) k_coarse_solve(Geom g, double r2x, double r2y, double r2z,
                                                       const float* __restrict__ r, float* __restrict__ e,
                                                       double* __restrict__ work, int sweeps) {
  const size_t n = g.points();
  const double H = 0.5 / (r2x + r2y + r2z);
  for (size_t k = threadIdx.x; k < 3 * n; k += blockDim.x) work[k] = 0.0;
  __syncthreads();
  const size_t sy = g.np[0], sz = (size_t)g.np[0] * g.np[1];
  for (int it = 0; it < sweeps; ++it) {
    for (unsigned color = 0; color < 2; ++color) {
      for (size_t k = threadIdx.x; k < n; k += blockDim.x) {
        unsigned x, y, z;
        unflat(k, g, x, y, z);
        if (!interior(g, x, y, z) || ((x + y + z) & 1u) != color) continue;
        for (int c = 0; c < 3; ++c) {
          const double s = (work[3 * (k + 1) + c] + work[3 * (k - 1) + c]) * r2x +
                           (work[3 * (k + sy) + c] + work[3 * (k - sy) + c]) * r2y +
                           (work[3 * (k + sz) + c] + work[3 * (k - sz) + c]) * r2z;
          work[3 * k + c] = (s - (double)r[3 * k + c]) * H;
        }
      }
      __syncthreads();
    }
  }
  for (size_t k = threadIdx.x; k < 3 * n; k += blockDim.x) e[k] = (float)work[k];
}

__global__ void k_to_f64(const float* __restrict__ a, double* __restrict__ b, size_t n) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) b[k] = (double)a[k];
}

__global__ void k_add_f64(double* __restrict__ a, const float* __restrict__ e, size_t n) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) a[k] += (double)e[k];
}

__global__ void k_to_f32(const double* __restrict__ a, float* __restrict__ b, size_t n) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) b[k] = (float)a[k];
}

}  // namespace

struct MgPlan {
  int nlev;
  Lev lev[kMaxLayers];
  size_t total;
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
  P.total = total;
  return P;
}

vg_status run_multigrid(Ctx* c, const Geom& g, float* soln3, const float* rhs3, double tol, int max_cycles,
                        int* cycles_out, double* relres0_out, double* relres_out) {
  const MgPlan P = plan_levels(g);
  const size_t n0 = g.points();
  const int pre = 2, post = 2;
  // workspace: e, r, res for every level (FP32), a64 (FP64), partials, coarse work
  const unsigned nb0 = blocks_for(n0, kRedThreads);
  const size_t coarse_pts = P.lev[P.nlev - 1].g.points();
  const size_t bytes = 3 * P.total * 3 * sizeof(float) + n0 * 3 * sizeof(double) + (size_t)nb0 * 2 * sizeof(double) +
                       4 * sizeof(double) + coarse_pts * 3 * sizeof(double) + 1024;
  vg_status st = VG_OK;
  char* mem = (char*)ws(c, S_MG, bytes, &st);
  if (st != VG_OK) return st;
  float* E = (float*)mem;
  float* R = E + 3 * P.total;
  float* RES = R + 3 * P.total;
  double* a64 = (double*)(((uintptr_t)(RES + 3 * P.total) + 255) & ~(uintptr_t)255);
  double* part = a64 + 3 * n0;
  double* sums = part + 2 * (size_t)nb0;
  double* cwork = sums + 4;
  const double r2x = 1.0 / ((double)g.cell[0] * g.cell[0]);
  const double r2y = 1.0 / ((double)g.cell[1] * g.cell[1]);
  const double r2z = 1.0 / ((double)g.cell[2] * g.cell[2]);
  k_to_f64<<<blocks_for(3 * n0, 256), 256, 0, c->stream>>>(soln3, a64, 3 * n0);
  VG_LAUNCHED(c);
  double relres = 0.0, relres0 = -1.0;
  int cyc = 0;
  for (;;) {
    k_residual64<<<nb0, kRedThreads, 0, c->stream>>>(g, r2x, r2y, r2z, a64, rhs3, R, part);
    k_sum_partials<<<1, 1024, 0, c->stream>>>(part, (int)nb0, sums);
    c->launches += 2;
    double h[2];
    VG_CUDA(c, cudaMemcpyAsync(h, sums, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    VG_CUDA(c, cudaStreamSynchronize(c->stream));
    relres = h[1] > 0.0 ? std::sqrt(h[0] / h[1]) : std::sqrt(h[0]);
    if (relres0 < 0.0) relres0 = relres;
    if (!(relres == relres)) return fail(c, VG_NONFINITE, "multigrid: non-finite residual");
    if (relres <= tol || cyc >= max_cycles) break;
    // one V-cycle on the correction
    for (int l = 0; l < P.nlev; ++l) {
      const Lev& L = P.lev[l];
      float* e = E + 3 * L.base;
      float* r = R + 3 * L.base;
      float* res = RES + 3 * L.base;
      const size_t npts = L.g.points();
      const size_t pairs = (size_t)L.g.np[1] * L.g.np[2] * ((L.g.np[0] + 1) / 2);
      if (l == P.nlev - 1) {
        // Gauss-Seidel on m interior points per axis contracts by about
        // cos^2(pi / (m + 1)) per sweep: 3 (m + 1)^2 sweeps reduce the error
        // by ~1e-13, far below what the V-cycle around it needs.
        unsigned m = std::max(L.g.np[0], std::max(L.g.np[1], L.g.np[2])) - 1;
        int sweeps = (int)std::min(3u * m * m + 2u, 4000u);
        const double cx = 1.0 / ((double)L.g.cell[0] * L.g.cell[0]), cy = 1.0 / ((double)L.g.cell[1] * L.g.cell[1]),
                     cz = 1.0 / ((double)L.g.cell[2] * L.g.cell[2]);
        k_coarse_solve<<<1, 1024, 0, c->stream>>>(L.g, cx, cy, cz, r, e, cwork, sweeps);
        VG_LAUNCHED(c);
        break;
      }
      for (int s = 0; s < pre; ++s)
        for (unsigned col = 0; col < 2; ++col) {
          k_rbgs<<<blocks_for(pairs, 256), 256, 0, c->stream>>>(L.g, L.r2x, L.r2y, L.r2z, L.H, e, r, col,
                                                                (s == 0 && col == 0) ? 1 : 0);
          VG_LAUNCHED(c);
        }
      // zero_first only covers the red points; black points read red values
      // and r, so e needs no clearing as long as the red sweep writes every
      // red interior point and the black sweep every black one.
      k_residual32<<<blocks_for(npts, 256), 256, 0, c->stream>>>(L.g, L.r2x, L.r2y, L.r2z, e, r, res);
      const Lev& Cn = P.lev[l + 1];
      k_restrict<<<blocks_for(Cn.g.points(), 256), 256, 0, c->stream>>>(L.g, Cn.g, res, R + 3 * Cn.base);
      c->launches += 2;
    }
    for (int l = P.nlev - 2; l >= 0; --l) {
      const Lev& L = P.lev[l];
      const Lev& Cn = P.lev[l + 1];
      float* e = E + 3 * L.base;
      float* r = R + 3 * L.base;
      const size_t pairs = (size_t)L.g.np[1] * L.g.np[2] * ((L.g.np[0] + 1) / 2);
      k_prolong_add<<<blocks_for(L.g.points(), 256), 256, 0, c->stream>>>(L.g, Cn.g, E + 3 * Cn.base, e);
      VG_LAUNCHED(c);
      for (int s = 0; s < post; ++s)
        for (unsigned col = 0; col < 2; ++col) {
          k_rbgs<<<blocks_for(pairs, 256), 256, 0, c->stream>>>(L.g, L.r2x, L.r2y, L.r2z, L.H, e, r, col, 0);
          VG_LAUNCHED(c);
        }
    }
    k_add_f64<<<blocks_for(3 * n0, 256), 256, 0, c->stream>>>(a64, E, 3 * n0);
    VG_LAUNCHED(c);
    ++cyc;
  }
  k_to_f32<<<blocks_for(3 * n0, 256), 256, 0, c->stream>>>(a64, soln3, 3 * n0);
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  if (cycles_out) *cycles_out = cyc;
  if (relres0_out) *relres0_out = relres0;
  if (relres_out) *relres_out = relres;
  if (relres > tol) return fail(c, VG_NOT_CONVERGED, "multigrid: cycle limit reached above tolerance");
  return VG_OK;
}

}  // namespace vg
