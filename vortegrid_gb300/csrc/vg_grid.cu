// Grid and particle stages of the VortonSim step (HBM / L2 bound):
//  * k_sor_rows      -- StepTowardVectorPoissonSolution, red then black,
//                       Dirichlet (Core/SpatialPartition/uniformGridMath.cpp:
//                       1116-1339): the reference colours whole x-rows by
//                       (y + z) parity and sweeps each row in +x, so one thread
//                       owns one row and walks it in order (bit-exact);
//  * k_downsample    -- UniformGrid::DownSampleSlice (uniformGrid.h:1453-1585);
//  * k_upsample      -- UniformGrid::UpSampleSlice (uniformGrid.h:1637-1700);
//  * k_jacobian      -- ComputeJacobian (uniformGridMath.cpp:304-451);
//  * k_curl          -- ComputeJacobian + ComputeCurlFromJacobian fused: only
//                       the six off-diagonal derivatives the curl needs;
//  * k_stretch       -- StretchAndTiltVortons (VortonFluid/vortonSim.cpp:
//                       2748-2820);
//  * k_pse           -- DiffuseAndDissipateVorticityPSE (vortonSim.cpp:
//                       3616-3879), order-independent form;
//  * k_gather_advect -- AssignParticleVelocityFromField (gain 1) +
//                       EvolveParticlesSlice (Particles/Operation/
//                       pclOpAdvect.cpp:42-81, pclOpEvolve.cpp:36-58);
//  * k_bbox          -- FindBoundingBox (pclOpFindBoundingBox.cpp:102-140).
// All arithmetic that the reference performs in FP32 is written with
// round-to-nearest intrinsics in the reference's order.
#include <float.h>

#include "vg_internal.cuh"

namespace vg {

namespace {

__global__ void k_sor_rows(Geom g, float* __restrict__ s, const float* __restrict__ lap, unsigned color, float r2x,
                           float r2y, float r2z, float H) {
  pdl_entry();
  // rows (y, z) interior with (z % 2 == color) ? y odd-shifted : ...
  const unsigned ny = g.np[1], nz = g.np[2], nx = g.np[0];
  const unsigned rows_per_z = (ny - 2 + 1) / 2 + 1;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t zi = t / rows_per_z;
  const unsigned z = (unsigned)zi + 1;
  if (z + 1 > nz - 1 + 0 || z >= nz - 1) return;
  const unsigned yshift = (z % 2 == color) ? 1u : 0u;
  const unsigned y = 1 + yshift + 2 * (unsigned)(t % rows_per_z);
  if (y >= ny - 1) return;
  const size_t nxy = (size_t)nx * ny;
  const float relax = 1.72f;
  const float omr = __fsub_rn(1.0f, relax);
  size_t c = 1 + (size_t)nx * y + nxy * z;
  for (unsigned x = 1; x + 1 < nx; ++x, ++c) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const float t1 = __fmul_rn(__fadd_rn(s[3 * (c + 1) + a], s[3 * (c - 1) + a]), r2x);
      const float t2 = __fmul_rn(__fadd_rn(s[3 * (c + nx) + a], s[3 * (c - nx) + a]), r2y);
      const float t3 = __fmul_rn(__fadd_rn(s[3 * (c + nxy) + a], s[3 * (c - nxy) + a]), r2z);
      const float v = __fmul_rn(__fsub_rn(__fadd_rn(__fadd_rn(t1, t2), t3), lap[3 * c + a]), H);
      s[3 * c + a] = __fadd_rn(__fmul_rn(omr, s[3 * c + a]), __fmul_rn(relax, v));
    }
  }
}

__global__ void k_downsample(Geom F, const float* __restrict__ f, Geom C, uint3 cd, int inject,
                             float* __restrict__ out) {
  pdl_entry();
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= C.points()) return;
  const unsigned x = (unsigned)(k % C.np[0]), y = (unsigned)((k / C.np[0]) % C.np[1]),
                 z = (unsigned)(k / ((size_t)C.np[0] * C.np[1]));
  const unsigned mx = x * cd.x, my = y * cd.y, mz = z * cd.z;
  const size_t fnx = F.np[0], fnxy = (size_t)F.np[0] * F.np[1];
  if (inject) {
    const size_t o = mx + my * fnx + mz * fnxy;
    out[3 * k] = f[3 * o];
    out[3 * k + 1] = f[3 * o + 1];
    out[3 * k + 2] = f[3 * o + 2];
    return;
  }
  const float table[4] = {8.0f, 4.0f, 2.0f, 1.0f};
  const unsigned sh[3] = {cd.x / 2, cd.y / 2, cd.z / 2};
  float ax = 0.f, ay = 0.f, az = 0.f;
  for (unsigned iz = 0; iz < cd.z + sh[2]; ++iz) {
    const int s2 = (int)iz - (int)sh[2];
    const unsigned hz = mz + (unsigned)s2;
    if (hz >= F.np[2]) continue;
    for (unsigned iy = 0; iy < cd.y + sh[1]; ++iy) {
      const int s1 = (int)iy - (int)sh[1];
      const unsigned hy = my + (unsigned)s1;
      if (hy >= F.np[1]) continue;
      for (unsigned ix = 0; ix < cd.x + sh[0]; ++ix) {
        const int s0 = (int)ix - (int)sh[0];
        const unsigned hx = mx + (unsigned)s0;
        if (hx >= F.np[0]) continue;
        const float wt = table[abs(s0) + abs(s1) + abs(s2)];
        const size_t o = hx + hy * fnx + hz * fnxy;
        ax = __fadd_rn(ax, __fmul_rn(wt, f[3 * o]));
        ay = __fadd_rn(ay, __fmul_rn(wt, f[3 * o + 1]));
        az = __fadd_rn(az, __fmul_rn(wt, f[3 * o + 2]));
      }
    }
  }
  const float r = 1.0f / 64.0f;
  out[3 * k] = __fmul_rn(ax, r);
  out[3 * k + 1] = __fmul_rn(ay, r);
  out[3 * k + 2] = __fmul_rn(az, r);
}

__global__ void k_upsample(Geom C, const float* __restrict__ cv, Geom F, int interior, float* __restrict__ fv) {
  pdl_entry();
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= F.points()) return;
  const unsigned x = (unsigned)(k % F.np[0]), y = (unsigned)((k / F.np[0]) % F.np[1]),
                 z = (unsigned)(k / ((size_t)F.np[0] * F.np[1]));
  if (interior && (x == 0 || y == 0 || z == 0 || x + 1 >= F.np[0] || y + 1 >= F.np[1] || z + 1 >= F.np[2])) return;
  const float two_eps = 2.0f * FLT_EPSILON;
  const float shrink = 1.0f - 4.0f * FLT_EPSILON;
  float p[3];
  const unsigned id[3] = {x, y, z};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float pmin = __fadd_rn(F.mn[a], __fmul_rn(__fmul_rn(fabsf(F.mn[a]), 2.0f), FLT_EPSILON));
    const float sp = __fmul_rn(F.cell[a], shrink);
    p[a] = __fadd_rn(pmin, __fmul_rn((float)id[a], sp));
  }
  (void)two_eps;
  if (!inside_cells(C, p[0], p[1], p[2])) return;
  interp<3>(C, cv, p[0], p[1], p[2], fv + 3 * k);
}

// Per-axis derivative factor and neighbours (uniformGridMath.cpp:326-344, 348-356).
__device__ __forceinline__ void diff_axis(size_t c, unsigned i, unsigned n, size_t stride, float rs, float hrs,
                                          size_t& hi, size_t& lo, float& f) {
  if (i == 0) {
    hi = c + stride; lo = c; f = rs;
  } else if (i == n - 1) {
    hi = c; lo = c - stride; f = rs;
  } else {
    hi = c + stride; lo = c - stride; f = hrs;
  }
}

__global__ void k_jacobian(Geom g, float rsx, float rsy, float rsz, const float* __restrict__ v,
                           float* __restrict__ jac) {
  pdl_entry();
  const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.points()) return;
  const unsigned nx = g.np[0], ny = g.np[1];
  const unsigned id[3] = {(unsigned)(c % nx), (unsigned)((c / nx) % ny), (unsigned)(c / ((size_t)nx * ny))};
  const size_t stride[3] = {1, nx, (size_t)nx * ny};
  const float rs[3] = {rsx, rsy, rsz};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    size_t hi, lo;
    float f;
    diff_axis(c, id[a], g.np[a], stride[a], rs[a], __fmul_rn(0.5f, rs[a]), hi, lo, f);
#pragma unroll
    for (int b = 0; b < 3; ++b) jac[9 * c + 3 * a + b] = __fmul_rn(__fsub_rn(v[3 * hi + b], v[3 * lo + b]), f);
  }
}

__global__ void k_curl(Geom g, float rsx, float rsy, float rsz, const float* __restrict__ v,
                       float* __restrict__ curl) {
  pdl_entry();
  const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.points()) return;
  const unsigned nx = g.np[0], ny = g.np[1];
  const unsigned id[3] = {(unsigned)(c % nx), (unsigned)((c / nx) % ny), (unsigned)(c / ((size_t)nx * ny))};
  const size_t stride[3] = {1, nx, (size_t)nx * ny};
  const float rs[3] = {rsx, rsy, rsz};
  float J[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    size_t hi, lo;
    float f;
    diff_axis(c, id[a], g.np[a], stride[a], rs[a], __fmul_rn(0.5f, rs[a]), hi, lo, f);
#pragma unroll
    for (int b = 0; b < 3; ++b) J[a][b] = (a == b) ? 0.f : __fmul_rn(__fsub_rn(v[3 * hi + b], v[3 * lo + b]), f);
  }
  curl[3 * c] = __fsub_rn(J[1][2], J[2][1]);
  curl[3 * c + 1] = __fsub_rn(J[2][0], J[0][2]);
  curl[3 * c + 2] = __fsub_rn(J[0][1], J[1][0]);
}

// order (optional): the vortons grouped by cell, so that a warp's vortons
// interpolate from the same few cells' corners (each vorton's update is the
// same whichever thread runs it).
__global__ void k_stretch(Geom g, const float* __restrict__ jac, const float4* __restrict__ ps,
                          float4* __restrict__ w, int n, float dt, const unsigned* __restrict__ order,
                          int* __restrict__ flag) {
  pdl_entry();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = order ? (int)order[t] : t;
  const float4 p = ps[i];
  if (!inside_cells(g, p.x, p.y, p.z)) {
    atomicOr(flag, (int)DF_OUT_OF_GRID);
    return;
  }
  float J[9];
  interp<9>(g, jac, p.x, p.y, p.z, J);
  float4 a = w[i];
  const float s0 = __fadd_rn(__fadd_rn(__fmul_rn(J[0], a.x), __fmul_rn(J[1], a.y)), __fmul_rn(J[2], a.z));
  const float s1 = __fadd_rn(__fadd_rn(__fmul_rn(J[3], a.x), __fmul_rn(J[4], a.y)), __fmul_rn(J[5], a.z));
  const float s2 = __fadd_rn(__fadd_rn(__fmul_rn(J[6], a.x), __fmul_rn(J[7], a.y)), __fmul_rn(J[8], a.z));
  a.x = __fadd_rn(a.x, __fmul_rn(__fmul_rn(0.5f, s0), dt));
  a.y = __fadd_rn(a.y, __fmul_rn(__fmul_rn(0.5f, s1), dt));
  a.z = __fadd_rn(a.z, __fmul_rn(__fmul_rn(0.5f, s2), dt));
  w[i] = a;
}

// k_jacobian and k_stretch fused: the velocity Jacobian is formed at the 8
// corners of each vorton's cell from the velocity grid (the differences of
// k_jacobian at those grid points) and interpolated as interp<9> would from
// the Jacobian grid, so the 9-float-per-point grid is never written.  Same
// float operations on the same values as the two kernels; order as k_stretch.
__global__ void k_stretch_vel(Geom g, float rsx, float rsy, float rsz, const float* __restrict__ v,
                              const float4* __restrict__ ps, float4* __restrict__ w, int n, float dt,
                              const unsigned* __restrict__ order, int* __restrict__ flag) {
  pdl_entry();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = order ? (int)order[t] : t;
  const float4 p = ps[i];
  if (!inside_cells(g, p.x, p.y, p.z)) {
    atomicOr(flag, (int)DF_OUT_OF_GRID);
    return;
  }
  const float pp[3] = {p.x, p.y, p.z};
  unsigned idx[3];
  float tw[3], om[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    idx[a] = bin_axis(pp[a], g.mn[a], g.cpe[a]);
    const float cmin = __fadd_rn(g.mn[a], __fmul_rn((float)idx[a], g.cell[a]));
    tw[a] = __fmul_rn(__fsub_rn(pp[a], cmin), g.cpe[a]);
    om[a] = __fsub_rn(1.0f, tw[a]);
  }
  const unsigned nx = g.np[0], ny = g.np[1];
  const size_t stride[3] = {1, nx, (size_t)nx * ny};
  const float rs[3] = {rsx, rsy, rsz};
  float J[9];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float hrs = __fmul_rn(0.5f, rs[a]);
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      float cv[8];  // corners (dx, dy, dz), x fastest: v000, v100, v010, v110, v001, v101, v011, v111
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const unsigned ci[3] = {idx[0] + (q & 1), idx[1] + ((q >> 1) & 1), idx[2] + (q >> 2)};
        const size_t c = ci[0] + (size_t)nx * (ci[1] + (size_t)ny * ci[2]);
        size_t hi, lo;
        float f;
        diff_axis(c, ci[a], g.np[a], stride[a], rs[a], hrs, hi, lo, f);
        cv[q] = __fmul_rn(__fsub_rn(v[3 * hi + b], v[3 * lo + b]), f);
      }
      const float y0 = __fadd_rn(__fmul_rn(__fadd_rn(__fmul_rn(om[0], cv[0]), __fmul_rn(tw[0], cv[1])), om[1]),
                                 __fmul_rn(__fadd_rn(__fmul_rn(om[0], cv[2]), __fmul_rn(tw[0], cv[3])), tw[1]));
      const float y1 = __fadd_rn(__fmul_rn(__fadd_rn(__fmul_rn(om[0], cv[4]), __fmul_rn(tw[0], cv[5])), om[1]),
                                 __fmul_rn(__fadd_rn(__fmul_rn(om[0], cv[6]), __fmul_rn(tw[0], cv[7])), tw[1]));
      J[3 * a + b] = __fadd_rn(__fmul_rn(y0, om[2]), __fmul_rn(y1, tw[2]));
    }
  }
  float4 wa = w[i];
  const float s0 = __fadd_rn(__fadd_rn(__fmul_rn(J[0], wa.x), __fmul_rn(J[1], wa.y)), __fmul_rn(J[2], wa.z));
  const float s1 = __fadd_rn(__fadd_rn(__fmul_rn(J[3], wa.x), __fmul_rn(J[4], wa.y)), __fmul_rn(J[5], wa.z));
  const float s2 = __fadd_rn(__fadd_rn(__fmul_rn(J[6], wa.x), __fmul_rn(J[7], wa.y)), __fmul_rn(J[8], wa.z));
  wa.x = __fadd_rn(wa.x, __fmul_rn(__fmul_rn(0.5f, s0), dt));
  wa.y = __fadd_rn(wa.y, __fmul_rn(__fmul_rn(0.5f, s1), dt));
  wa.z = __fadd_rn(wa.z, __fmul_rn(__fmul_rn(0.5f, s2), dt));
  w[i] = wa;
}

// Order-independent PSE: vorton i exchanges with every vorton of the pair set
// the reference visits (same cell, or cells offset by {0,1}^3 either way with
// the lower cell strictly inside the point range), using pre-step values.
// Pre-step positions and angular velocities in cell order (pss[t], w0s[t] of
// vorton items[t]), so that each cell's vortons are contiguous for k_pse.
__global__ void k_pse_gather(const float4* __restrict__ ps, const float4* __restrict__ w, int n,
                             const unsigned* __restrict__ items, float4* __restrict__ pss, float4* __restrict__ w0s) {
  pdl_entry();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const unsigned j = items[t];
  pss[t] = ps[j];
  w0s[t] = w[j];
}

__global__ void __launch_bounds__(128) k_pse(Geom g, const float4* __restrict__ pss, const float4* __restrict__ w0s,
                                             float4* __restrict__ w, int n, const unsigned* __restrict__ start,
                                             const unsigned* __restrict__ items, float nu, float dt) {
  pdl_entry();
  // threads take the vortons in cell order, so a warp's vortons share their
  // neighbour cells and read them contiguously (each vorton's sums are the
  // same whichever thread runs them)
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = (int)items[t];
  const float4 p = pss[t];
  const float4 wi = w0s[t];
  const int nx = (int)g.np[0], ny = (int)g.np[1], nz = (int)g.np[2];
  // cell coordinates clamped to [-2, n + 1]: beyond that every neighbour test
  // below fails the same way, and ncx = cx + ox cannot overflow
  const int cx = min(max(__float2int_rz(__fmul_rn(__fsub_rn(p.x, g.mn[0]), g.cpe[0])), -2), nx + 1);
  const int cy = min(max(__float2int_rz(__fmul_rn(__fsub_rn(p.y, g.mn[1]), g.cpe[1])), -2), ny + 1);
  const int cz = min(max(__float2int_rz(__fmul_rn(__fsub_rn(p.z, g.mn[2]), g.cpe[2])), -2), nz + 1);
  if (cx < 0 || cy < 0 || cz < 0 || cx >= nx || cy >= ny || cz >= nz) {
    w[i] = wi;  // outside the grid's points: in no cell list, so no exchange
    return;
  }
  const bool here_ok = cx >= 0 && cy >= 0 && cz >= 0 && cx < nx - 1 && cy < ny - 1 && cz < nz - 1;
  const float twonudt = 2.0f * nu * dt;
  float ax = 0.f, ay = 0.f, az = 0.f;
  for (int s = -1; s <= 1; s += 2) {
    for (int k = 0; k < 8; ++k) {
      if (k == 0 && s == 1) continue;
      const int ox = s * (k & 1), oy = s * ((k >> 1) & 1), oz = s * ((k >> 2) & 1);
      const int ncx = cx + ox, ncy = cy + oy, ncz = cz + oz;
      if (ncx < 0 || ncy < 0 || ncz < 0 || ncx >= nx || ncy >= ny || ncz >= nz) continue;
      const int lx = (s == 1) ? cx : ncx, ly = (s == 1) ? cy : ncy, lz = (s == 1) ? cz : ncz;
      if (!(lx < nx - 1 && ly < ny - 1 && lz < nz - 1)) continue;
      const size_t cell = (size_t)ncx + (size_t)nx * ((size_t)ncy + (size_t)ny * ncz);
      const unsigned b = start[cell], e = start[cell + 1];
      for (unsigned kk = b; kk < e; ++kk) {
        const unsigned j = items[kk];
        if (j == (unsigned)i) continue;
        const float4 pj = pss[kk];
        const unsigned here = (k == 0) ? min((unsigned)i, j) : (s == 1 ? (unsigned)i : j);
        const float range = 4.0f * (here == (unsigned)i ? p.w : pj.w);
        const float dx = p.x - pj.x, dy = p.y - pj.y, dz = p.z - pj.z;
        const float dist2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        const float law = __expf(-dist2 / (range * range));
        const float frac = fminf(fmaxf(twonudt * law, -0.5f), 0.5f);
        const float4 wj = w0s[kk];
        ax = fmaf(frac, wj.x - wi.x, ax);
        ay = fmaf(frac, wj.y - wi.y, ay);
        az = fmaf(frac, wj.z - wi.z, az);
      }
    }
  }
  float vx = wi.x + ax, vy = wi.y + ay, vz = wi.z + az;
  if (here_ok) {
    const float f = nu * dt;
    vx -= f * vx;
    vy -= f * vy;
    vz -= f * vz;
  }
  w[i] = make_float4(vx, vy, vz, wi.w);
}

// DiffuseAndDissipateHeatPSE (vortonSim.cpp:3880-4093) in the order-independent
// form of k_pse: vorton i (threads in cell order, reading cell-sorted copies)
// exchanges density with every vorton of its own cell and of the face
// neighbours along +-x, +-y, +-z that the reference pairs it with (the pair's
// "here" cell strictly inside the point range; the range 4 x the "here"
// vorton's size), using the densities from before the step, then relaxes
// toward the ambient density when its own cell is a "here" cell.
__global__ void k_heat_gather(const float4* __restrict__ ps, const float* __restrict__ d, int n,
                              const unsigned* __restrict__ items, float4* __restrict__ pss, float* __restrict__ d0s) {
  pdl_entry();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const unsigned j = items[t];
  pss[t] = ps[j];
  d0s[t] = d[j];
}

__global__ void __launch_bounds__(128) k_heat_pse(Geom g, const float4* __restrict__ pss, const float* __restrict__ d0s,
                                                  float* __restrict__ d, int n, const unsigned* __restrict__ start,
                                                  const unsigned* __restrict__ items, float kappa, float ambient,
                                                  float dt) {
  pdl_entry();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = (int)items[t];
  const float4 p = pss[t];
  const float di = d0s[t];
  const int nx = (int)g.np[0], ny = (int)g.np[1], nz = (int)g.np[2];
  const int cx = min(max(__float2int_rz(__fmul_rn(__fsub_rn(p.x, g.mn[0]), g.cpe[0])), -2), nx + 1);
  const int cy = min(max(__float2int_rz(__fmul_rn(__fsub_rn(p.y, g.mn[1]), g.cpe[1])), -2), ny + 1);
  const int cz = min(max(__float2int_rz(__fmul_rn(__fsub_rn(p.z, g.mn[2]), g.cpe[2])), -2), nz + 1);
  if (cx < 0 || cy < 0 || cz < 0 || cx >= nx || cy >= ny || cz >= nz) {
    d[i] = di;  // in no cell list: no exchange
    return;
  }
  const bool here_ok = cx < nx - 1 && cy < ny - 1 && cz < nz - 1;
  const float twokdt = 2.0f * kappa * dt;
  float acc = 0.f;
  for (int s = -1; s <= 1; s += 2) {
    for (int k = 0; k < 4; ++k) {
      if (k == 0 && s == 1) continue;
      const int ox = k == 1 ? s : 0, oy = k == 2 ? s : 0, oz = k == 3 ? s : 0;
      const int ncx = cx + ox, ncy = cy + oy, ncz = cz + oz;
      if (ncx < 0 || ncy < 0 || ncz < 0 || ncx >= nx || ncy >= ny || ncz >= nz) continue;
      const int lx = (s == 1) ? cx : ncx, ly = (s == 1) ? cy : ncy, lz = (s == 1) ? cz : ncz;
      if (!(lx < nx - 1 && ly < ny - 1 && lz < nz - 1)) continue;
      const size_t cell = (size_t)ncx + (size_t)nx * ((size_t)ncy + (size_t)ny * ncz);
      const unsigned b = start[cell], e = start[cell + 1];
      for (unsigned kk = b; kk < e; ++kk) {
        const unsigned j = items[kk];
        if (j == (unsigned)i) continue;
        const float4 pj = pss[kk];
        const unsigned here = (k == 0) ? min((unsigned)i, j) : (s == 1 ? (unsigned)i : j);
        const float range = 4.0f * (here == (unsigned)i ? p.w : pj.w);
        const float dx = p.x - pj.x, dy = p.y - pj.y, dz = p.z - pj.z;
        const float dist2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        const float law = __expf(-dist2 / (range * range));
        const float ratio = fminf(fmaxf(twokdt * law, -0.5f), 0.5f);
        acc = fmaf(ratio, d0s[kk] - di, acc);
      }
    }
  }
  float v = di + acc;
  if (here_ok) v += fminf(fmaxf(kappa * dt, -0.5f), 0.5f) * (ambient - v);
  d[i] = v;
}

// order (optional): the particles grouped by cell, as in k_stretch.
__global__ void k_gather_advect(Geom g, const float* __restrict__ vel3, float4* __restrict__ pos,
                                float4* __restrict__ vel, int m, float dt, int evolve,
                                const unsigned* __restrict__ order, int* __restrict__ flag) {
  pdl_entry();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  const int i = order ? (int)order[t] : t;
  float4 p = pos[i];
  if (!inside_cells(g, p.x, p.y, p.z)) {
    atomicOr(flag, (int)DF_OUT_OF_GRID);
    if (vel) vel[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    return;
  }
  float u[3];
  interp<3>(g, vel3, p.x, p.y, p.z, u);
  if (vel) vel[i] = make_float4(u[0], u[1], u[2], 0.f);
  if (evolve) {
    p.x = __fadd_rn(p.x, __fmul_rn(u[0], dt));
    p.y = __fadd_rn(p.y, __fmul_rn(u[1], dt));
    p.z = __fadd_rn(p.z, __fmul_rn(u[2], dt));
    pos[i] = p;
  }
}

// AssignParticleVelocityFromField (gain 1) + EvolveParticlesSlice on staged
// particle records (position at bytes 0-11, velocity at 12-23, pitch bytes
// apart), in place: k_gather_advect without copying positions and velocities
// out of and back into the records.  A record outside the grid's cells keeps
// its position and gets zero velocity, as on the copy path.
__global__ void k_gather_advect_records(Geom g, const float* __restrict__ vel3, unsigned char* __restrict__ rec,
                                        size_t pitch, int m, float dt, int* __restrict__ flag) {
  pdl_entry();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  float* r = (float*)(rec + (size_t)i * pitch);
  const float px = r[0], py = r[1], pz = r[2];
  if (!inside_cells(g, px, py, pz)) {
    atomicOr(flag, (int)DF_OUT_OF_GRID);
    r[3] = 0.f;
    r[4] = 0.f;
    r[5] = 0.f;
    return;
  }
  float u[3];
  interp<3>(g, vel3, px, py, pz, u);
  r[0] = __fadd_rn(px, __fmul_rn(u[0], dt));
  r[1] = __fadd_rn(py, __fmul_rn(u[1], dt));
  r[2] = __fadd_rn(pz, __fmul_rn(u[2], dt));
  r[3] = u[0];
  r[4] = u[1];
  r[5] = u[2];
}

// The velocity grid arranged by cell: the 8 corners of cell (x, y, z) as
// float4 (u, v, w, 0), corners in interp's order (x fastest), so that a
// tracer's gather is one 128-byte line instead of four scattered row pairs.
__global__ void k_vel_cells(Geom g, const float* __restrict__ v3, float4* __restrict__ vc) {
  pdl_entry();
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t cx = g.np[0] - 1, cy = g.np[1] - 1;
  const size_t cells = cx * cy * (size_t)(g.np[2] - 1);
  if (t >= 8 * cells) return;
  const size_t cell = t >> 3;
  const unsigned q = (unsigned)(t & 7);
  const size_t x = cell % cx, y = (cell / cx) % cy, z = cell / (cx * cy);
  const size_t k = (x + (q & 1)) + (size_t)g.np[0] * ((y + ((q >> 1) & 1)) + (size_t)g.np[1] * (z + (q >> 2)));
  vc[t] = make_float4(v3[3 * k], v3[3 * k + 1], v3[3 * k + 2], 0.f);
}

// k_gather_advect reading the by-cell copy: the same cell, weights and
// trilinear sums as interp<3> on the grid (bit-identical).
__global__ void k_gather_advect_cells(Geom g, const float4* __restrict__ vc, float4* __restrict__ pos,
                                      float4* __restrict__ vel, int m, float dt, int evolve,
                                      int* __restrict__ flag) {
  pdl_entry();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  float4 p = pos[i];
  if (!inside_cells(g, p.x, p.y, p.z)) {
    atomicOr(flag, (int)DF_OUT_OF_GRID);
    if (vel) vel[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    return;
  }
  const float pp[3] = {p.x, p.y, p.z};
  unsigned idx[3];
  float tw[3], om[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    idx[a] = bin_axis(pp[a], g.mn[a], g.cpe[a]);
    const float cmin = __fadd_rn(g.mn[a], __fmul_rn((float)idx[a], g.cell[a]));
    tw[a] = __fmul_rn(__fsub_rn(pp[a], cmin), g.cpe[a]);
    om[a] = __fsub_rn(1.0f, tw[a]);
  }
  const size_t cell = idx[0] + (size_t)(g.np[0] - 1) * (idx[1] + (size_t)(g.np[1] - 1) * idx[2]);
  float4 c[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) c[q] = vc[8 * cell + q];
  float u[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    auto comp = [&](const float4& v) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); };
    const float y0 = __fadd_rn(__fmul_rn(__fadd_rn(__fmul_rn(om[0], comp(c[0])), __fmul_rn(tw[0], comp(c[1]))), om[1]),
                               __fmul_rn(__fadd_rn(__fmul_rn(om[0], comp(c[2])), __fmul_rn(tw[0], comp(c[3]))), tw[1]));
    const float y1 = __fadd_rn(__fmul_rn(__fadd_rn(__fmul_rn(om[0], comp(c[4])), __fmul_rn(tw[0], comp(c[5]))), om[1]),
                               __fmul_rn(__fadd_rn(__fmul_rn(om[0], comp(c[6])), __fmul_rn(tw[0], comp(c[7]))), tw[1]));
    u[a] = __fadd_rn(__fmul_rn(y0, om[2]), __fmul_rn(y1, tw[2]));
  }
  if (vel) vel[i] = make_float4(u[0], u[1], u[2], 0.f);
  if (evolve) {
    p.x = __fadd_rn(p.x, __fmul_rn(u[0], dt));
    p.y = __fadd_rn(p.y, __fmul_rn(u[1], dt));
    p.z = __fadd_rn(p.z, __fmul_rn(u[2], dt));
    pos[i] = p;
  }
}

// Order-preserving float <-> uint map for atomic min/max.
__device__ __forceinline__ unsigned f2key(float f) {
  const unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__global__ void k_bbox(const float4* __restrict__ pos, int n, unsigned* __restrict__ keys, int* __restrict__ flag) {
  pdl_entry();
  float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 p = pos[i];
    if (!(isfinite(p.x) && isfinite(p.y) && isfinite(p.z))) atomicOr(flag, (int)DF_NONFINITE);
    mn[0] = fminf(mn[0], p.x); mn[1] = fminf(mn[1], p.y); mn[2] = fminf(mn[2], p.z);
    mx[0] = fmaxf(mx[0], p.x); mx[1] = fmaxf(mx[1], p.y); mx[2] = fmaxf(mx[2], p.z);
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    for (int o = 16; o > 0; o >>= 1) {
      mn[a] = fminf(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
      mx[a] = fmaxf(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
    }
  }
  if ((threadIdx.x & 31) == 0) {
    for (int a = 0; a < 3; ++a) {
      atomicMin(&keys[a], f2key(mn[a]));
      atomicMax(&keys[3 + a], f2key(mx[a]));
    }
  }
}

__global__ void k_bbox_finish(const unsigned* __restrict__ keys, float* __restrict__ out6) {
  pdl_entry();
  const int a = threadIdx.x;
  if (a < 6) {
    const unsigned k = keys[a];
    const unsigned u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    out6[a] = __uint_as_float(u);
  }
}

__global__ void k_bbox_init(unsigned* keys) {
  pdl_entry();
  const int a = threadIdx.x;
  if (a < 3) keys[a] = 0xffffffffu;
  else if (a < 6) keys[a] = 0u;
}

}  // namespace

static void recip_spacing(const Geom& g, float rs[3]) {
  // reciprocalSpacing (uniformGridMath.cpp:1124, 317)
  rs[0] = 1.0f / g.cell[0];
  rs[1] = 1.0f / g.cell[1];
  rs[2] = g.cell[2] > FLT_EPSILON ? 1.0f / g.cell[2] : 0.0f;
}

vg_status launch_sor(Ctx* c, const Geom& g, float* s, const float* lap, int steps) {
  if (g.np[0] < 3 || g.np[1] < 3 || g.np[2] < 3 || steps <= 0) return VG_OK;
  float rs[3];
  recip_spacing(g, rs);
  volatile float r2x = rs[0] * rs[0], r2y = rs[1] * rs[1], r2z = rs[2] * rs[2];
  volatile float sum = r2x + r2y;
  sum = sum + r2z;
  const float H = 0.5f / sum;
  const unsigned rows_per_z = (g.np[1] - 2 + 1) / 2 + 1;
  const size_t threads = (size_t)rows_per_z * (g.np[2] - 2);
  for (int it = 0; it < steps; ++it)
    for (unsigned color = 0; color < 2; ++color) {
      pdl_launch(c->stream, blocks_for(threads, 64), 64, 0, k_sor_rows, g, s, lap, color, r2x, r2y, r2z, H);
      VG_LAUNCHED(c);
    }
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

vg_status launch_downsample(Ctx* c, const Geom& F, const float* f3, const Geom& C, bool inject, float* c3) {
  const uint3 cd = make_uint3((F.np[0] - 1) / (C.np[0] - 1), (F.np[1] - 1) / (C.np[1] - 1), (F.np[2] - 1) / (C.np[2] - 1));
  pdl_launch(c->stream, blocks_for(C.points(), 128), 128, 0, k_downsample, F, f3, C, cd, inject ? 1 : 0, c3);
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

vg_status launch_upsample(Ctx* c, const Geom& C, const float* c3, const Geom& F, bool interior, float* f3) {
  pdl_launch(c->stream, blocks_for(F.points(), 128), 128, 0, k_upsample, C, c3, F, interior ? 1 : 0, f3);
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

vg_status run_cascade(Ctx* c, const Geom& g, float* soln3, const float* rhs3, int steps) {
  Geom L[kMaxLayers];
  unsigned dec[kMaxLayers][3];
  const int depth = nested_shape(g, L, dec);
  size_t total = 0, base[kMaxLayers];
  for (int l = 0; l < depth; ++l) {
    base[l] = total;
    total += L[l].points();
  }
  vg_status st = VG_OK;
  float* mem = (float*)ws(c, S_MG, 2 * total * 3 * sizeof(float), &st);
  if (st != VG_OK) return st;
  float* a[kMaxLayers];
  float* b[kMaxLayers];
  for (int l = 0; l < depth; ++l) {
    a[l] = mem + 3 * base[l];
    b[l] = mem + 3 * (total + base[l]);
  }
  a[0] = soln3;
  b[0] = const_cast<float*>(rhs3);
  if ((st = launch_sor(c, L[0], a[0], b[0], steps)) != VG_OK) return st;
  int max_valid = 0;
  for (int l = 1; l < depth; ++l) {
    unsigned mind = L[l].np[0] < L[l].np[1] ? L[l].np[0] : L[l].np[1];
    if (L[l].np[2] < mind) mind = L[l].np[2];
    if (mind > 2) {
      if ((st = launch_downsample(c, L[l - 1], b[l - 1], L[l], true, b[l])) != VG_OK) return st;
      if ((st = launch_downsample(c, L[l - 1], a[l - 1], L[l], true, a[l])) != VG_OK) return st;
      if ((st = launch_sor(c, L[l], a[l], b[l], steps)) != VG_OK) return st;
    } else {
      max_valid = l - 1;
      break;
    }
  }
  for (int l = max_valid; l >= 1; --l) {
    if ((st = launch_upsample(c, L[l], a[l], L[l - 1], true, a[l - 1])) != VG_OK) return st;
    if ((st = launch_sor(c, L[l - 1], a[l - 1], b[l - 1], steps)) != VG_OK) return st;
  }
  return VG_OK;
}

vg_status launch_jacobian(Ctx* c, const Geom& g, const float* v3, float* jac9) {
  float rs[3];
  recip_spacing(g, rs);
  pdl_launch(c->stream, blocks_for(g.points(), 128), 128, 0, k_jacobian, g, rs[0], rs[1], rs[2], v3, jac9);
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

vg_status launch_curl(Ctx* c, const Geom& g, const float* v3, float* curl3) {
  float rs[3];
  recip_spacing(g, rs);
  pdl_launch(c->stream, blocks_for(g.points(), 128), 128, 0, k_curl, g, rs[0], rs[1], rs[2], v3, curl3);
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

vg_status launch_stretch_vel(Ctx* c, const Geom& g, const float* v3, const float4* ps, float4* w, size_t n, float dt,
                             const unsigned* order) {
  if (0.0f == g.ext[0] || 0.0f == g.ext[1] || 0.0f == g.ext[2]) return VG_OK;  // 2D: no stretching
  if (n == 0) return VG_OK;
  float rs[3];
  recip_spacing(g, rs);
  pdl_launch(c->stream, blocks_for(n, 128), 128, 0, k_stretch_vel, g, rs[0], rs[1], rs[2], v3, ps, w, (int)n, dt, order,
             outside_flag(c));
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

vg_status launch_stretch(Ctx* c, const Geom& g, const float* jac9, const float4* ps, float4* w, size_t n, float dt,
                         const unsigned* order) {
  if (0.0f == g.ext[0] || 0.0f == g.ext[1] || 0.0f == g.ext[2]) return VG_OK;  // 2D: no stretching
  if (n == 0) return VG_OK;
  pdl_launch(c->stream, blocks_for(n, 128), 128, 0, k_stretch, g, jac9, ps, w, (int)n, dt, order, outside_flag(c));
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

vg_status launch_heat_pse(Ctx* c, const Geom& g, const CellLists& cl, const float4* ps, float* density, size_t n,
                          float kappa, float ambient, float dt) {
  vg_status st = VG_OK;
  char* tmp = (char*)ws(c, S_WOLD, n * (sizeof(float4) + sizeof(float)), &st);
  if (st != VG_OK) return st;
  float4* pss = (float4*)tmp;
  float* d0s = (float*)(pss + n);
  pdl_launch(c->stream, blocks_for(n, 256), 256, 0, k_heat_gather, ps, density, (int)n, cl.items, pss, d0s);
  pdl_launch(c->stream, blocks_for(n, 128), 128, 0, k_heat_pse, g, pss, d0s, density, (int)n, cl.start, cl.items, kappa,
                                                        ambient, dt);
  c->launches += 2;
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

vg_status launch_pse(Ctx* c, const Geom& g, const CellLists& cl, const float4* ps, float4* w, size_t n, float nu,
                     float dt) {
  if (n == 0) return VG_OK;
  vg_status st = VG_OK;
  float4* pss = (float4*)ws(c, S_WOLD, 2 * n * sizeof(float4), &st);
  if (st != VG_OK) return st;
  float4* w0s = pss + n;
  pdl_launch(c->stream, blocks_for(n, 256), 256, 0, k_pse_gather, ps, w, (int)n, cl.items, pss, w0s);
  pdl_launch(c->stream, blocks_for(n, 128), 128, 0, k_pse, g, pss, w0s, w, (int)n, cl.start, cl.items, nu, dt);
  c->launches += 2;
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

bool gather_by_cell(const Geom& g, size_t m) {
  if (g.np[0] < 2 || g.np[1] < 2 || g.np[2] < 2) return false;
  const size_t cells = (size_t)(g.np[0] - 1) * (g.np[1] - 1) * (size_t)(g.np[2] - 1);
  return cells >= ((size_t)1 << 17) && m >= 2 * cells;
}

vg_status launch_gather_advect_records(Ctx* c, const Geom& g, const float* vel3, unsigned char* rec, size_t pitch,
                                       size_t m, float dt) {
  if (m == 0) return VG_OK;
  if (m > 0x7fffffff) return fail(c, VG_TOO_LARGE, "advect: more than 2^31 particles");
  pdl_launch(c->stream, blocks_for(m, 256), 256, 0, k_gather_advect_records, g, vel3, rec, pitch, (int)m, dt,
             outside_flag(c));
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

vg_status launch_gather_advect(Ctx* c, const Geom& g, const float* vel3, float4* pos, float4* vel, size_t m, float dt,
                               bool evolve, const unsigned* order, bool by_cell) {
  if (m == 0) return VG_OK;
  if (m > 0x7fffffff) return fail(c, VG_TOO_LARGE, "advect: more than 2^31 particles");
  const size_t cells = g.np[0] >= 2 && g.np[1] >= 2 && g.np[2] >= 2
                           ? (size_t)(g.np[0] - 1) * (g.np[1] - 1) * (size_t)(g.np[2] - 1)
                           : 0;
  // Tracer groups of at least two per cell gather from the grid arranged by
  // cell (made once per step; inside a graph capture always, so that every
  // replay remakes it from that replay's grid) -- on grids of at least 2^17
  // cells: a smaller grid stays in L1/L2 and the copy costs more than it saves
  // (65,536 tracers on 32^3 cells: the step 1.6% slower with it).
  if (by_cell && !order && gather_by_cell(g, m)) {
    vg_status st = VG_OK;
    float4* vc = (float4*)ws(c, S_VELCELL, 8 * cells * sizeof(float4), &st);
    if (st != VG_OK) return st;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    VG_CUDA(c, cudaStreamIsCapturing(c->stream, &cap));
    if (cap != cudaStreamCaptureStatusNone || c->velcell_gen != c->vel_gen) {
      pdl_launch(c->stream, blocks_for(8 * cells, 256), 256, 0, k_vel_cells, g, vel3, vc);
      VG_LAUNCHED(c);
      c->velcell_gen = cap != cudaStreamCaptureStatusNone ? ~0ull : c->vel_gen;
    }
    pdl_launch(c->stream, blocks_for(m, 256), 256, 0, k_gather_advect_cells, g, (const float4*)vc, pos, vel, (int)m,
               dt, evolve ? 1 : 0, outside_flag(c));
    VG_LAUNCHED(c);
    VG_CUDA(c, cudaGetLastError());
    return VG_OK;
  }
  pdl_launch(c->stream, blocks_for(m, 256), 256, 0, k_gather_advect, g, vel3, pos, vel, (int)m, dt, evolve ? 1 : 0, order,
                                                              outside_flag(c));
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

vg_status launch_bbox(Ctx* c, const float4* pos, size_t n, float* out6) {
  vg_status st = VG_OK;
  unsigned* keys = (unsigned*)ws(c, S_BBOX, 64, &st);
  if (st != VG_OK) return st;
  pdl_launch(c->stream, 1, 32, 0, k_bbox_init, keys);
  if (n > 0) {
    unsigned blocks = blocks_for(n, 256);
    if (blocks > 4u * (unsigned)sm_count()) blocks = 4u * (unsigned)sm_count();
    pdl_launch(c->stream, blocks, 256, 0, k_bbox, pos, (int)n, keys, c->dflag);
  }
  pdl_launch(c->stream, 1, 32, 0, k_bbox_finish, keys, out6);
  c->launches += 3;
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

}  // namespace vg
