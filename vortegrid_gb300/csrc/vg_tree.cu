// K3/K4/K5: NestedGrid influence tree, treecode evaluation, boundary vector
// potential and the vorticity splat.
//
//  * k_leaf      -- MakeBaseVortonGrid (VortonFluid/vortonSim.cpp:1192-1321):
//                   one thread per leaf point sums its cell's vortons in index
//                   order (|w|-weighted centroid with the FLT_MIN-seeded weight
//                   of vortonClusterAux.h:71, vorticity sum, last size);
//  * k_aggregate -- AggregateClusters (vortonSim.cpp:1337-1569), one launch
//                   per parent layer, children in the reference's z,y,x order;
//  * k_tree_eval -- ComputeVelocity_Tree / ComputeVectorPotential_Tree
//                   (vortonSim.cpp:1650-1905) as an explicit-stack walk that
//                   keeps one partial sum per open layer and adds it to its
//                   parent exactly where the recursion returns, so REFERENCE
//                   numerics reproduce the recursive sum bit for bit;
//  * boundary    -- ComputeVectorPotentialAtGridpoints_Slice with
//                   boundariesOnly (vortonSim.cpp:2055-2138): one thread per
//                   face point;
//  * k_splat     -- PopulateVorticityGridFromVortons + UniformGrid::Accumulate
//                   (vortonSim.cpp:2372-2436, uniformGrid.h:1278-1342) as a
//                   gather: each grid point merges the index-sorted lists of
//                   its 8 adjacent cells and adds their trilinear shares in
//                   vorton-index order -- the reference's summation order --
//                   with no atomics.
// The tree build and the splat always use the reference's operation order
// (they are a small share of the step); FAST numerics change only the
// per-pair law inside the tree walk.
#include <float.h>

#include "vg_internal.cuh"

namespace vg {

namespace {

struct TreeParams {
  int depth;
  Geom layer[kMaxLayers];
  unsigned decim[kMaxLayers][3];
  unsigned long long base[kMaxLayers];
};

__device__ __forceinline__ float ref_vort_mag(float4 w) {
  const float a = __fmul_rn(w.x, 2.0f), b = __fmul_rn(w.y, 2.0f), c = __fmul_rn(w.z, 2.0f);
  return __fsqrt_rn(ref_dot_self(a, b, c));
}

__global__ void k_leaf(Geom g, const float4* __restrict__ ps, const float4* __restrict__ w,
                       const unsigned* __restrict__ start, const unsigned* __restrict__ items,
                       float4* __restrict__ out_pos, float4* __restrict__ out_w) {
  pdl_entry();
  const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.points()) return;
  float px = 0.f, py = 0.f, pz = 0.f, wx = 0.f, wy = 0.f, wz = 0.f, size = 0.f, aux = FLT_MIN;
  const unsigned b = start[c], e = start[c + 1];
  for (unsigned k = b; k < e; ++k) {
    const unsigned i = items[k];
    const float4 p = ps[i];
    const float4 a = w[i];
    const float mag = ref_vort_mag(a);
    px = __fadd_rn(px, __fmul_rn(p.x, mag));
    py = __fadd_rn(py, __fmul_rn(p.y, mag));
    pz = __fadd_rn(pz, __fmul_rn(p.z, mag));
    wx = __fadd_rn(wx, a.x);
    wy = __fadd_rn(wy, a.y);
    wz = __fadd_rn(wz, a.z);
    size = p.w;
    aux = __fadd_rn(aux, mag);
  }
  if (aux != FLT_MIN) {
    const float r = __fdiv_rn(1.0f, aux);
    px = __fmul_rn(px, r);
    py = __fmul_rn(py, r);
    pz = __fmul_rn(pz, r);
  }
  out_pos[c] = make_float4(px, py, pz, size);
  out_w[c] = make_float4(wx, wy, wz, 0.f);
}

// AggregateClusters for parent point k of layer P from its children in C
// (decimation d): vorticity-weighted centroid, summed angular velocity, the
// last child's nonzero size.
__device__ __forceinline__ void aggregate_point(const Geom& P, const Geom& C, uint3 d, const float4* __restrict__ cpos,
                                                const float4* __restrict__ cw, float4* __restrict__ ppos,
                                                float4* __restrict__ pw, size_t k) {
  const unsigned px = (unsigned)(k % P.np[0]);
  const unsigned py = (unsigned)((k / P.np[0]) % P.np[1]);
  const unsigned pz = (unsigned)(k / ((size_t)P.np[0] * P.np[1]));
  float x = 0.f, y = 0.f, z = 0.f, wx = 0.f, wy = 0.f, wz = 0.f, size = 0.f;
  if (px < P.np[0] - 1 && py < P.np[1] - 1 && pz < P.np[2] - 1) {
    float aux = FLT_MIN;
    for (unsigned iz = 0; iz < d.z; ++iz)
      for (unsigned iy = 0; iy < d.y; ++iy)
        for (unsigned ix = 0; ix < d.x; ++ix) {
          const size_t o = (px * d.x + ix) + (size_t)C.np[0] * ((py * d.y + iy) + (size_t)C.np[1] * (pz * d.z + iz));
          const float4 p = cpos[o];
          const float4 a = cw[o];
          const float mag = ref_vort_mag(a);
          x = __fadd_rn(x, __fmul_rn(p.x, mag));
          y = __fadd_rn(y, __fmul_rn(p.y, mag));
          z = __fadd_rn(z, __fmul_rn(p.z, mag));
          wx = __fadd_rn(wx, a.x);
          wy = __fadd_rn(wy, a.y);
          wz = __fadd_rn(wz, a.z);
          aux = __fadd_rn(aux, mag);
          if (p.w != 0.0f) size = p.w;
        }
    const float r = __fdiv_rn(1.0f, aux);
    x = __fmul_rn(x, r);
    y = __fmul_rn(y, r);
    z = __fmul_rn(z, r);
  }
  ppos[k] = make_float4(x, y, z, size);
  pw[k] = make_float4(wx, wy, wz, 0.f);
}

__global__ void k_aggregate(Geom P, Geom C, uint3 d, const float4* __restrict__ cpos, const float4* __restrict__ cw,
                            float4* __restrict__ ppos, float4* __restrict__ pw) {
  pdl_entry();
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= P.points()) return;
  aggregate_point(P, C, d, cpos, cw, ppos, pw, k);
}

// The small top layers l0 .. depth-1 in one CTA, layer after layer (a barrier
// between them makes each layer's writes visible to the next): the same cells
// as one k_aggregate launch per layer, without a launch per few hundred points.
constexpr size_t kTopLayerPoints = 4096;  // layers of at most this many points go to k_aggregate_top
constexpr int kTopThreads = 1024;
__global__ void __launch_bounds__(kTopThreads) k_aggregate_top(const __grid_constant__ TreeParams T, int l0,
                                                               float4* __restrict__ sv_pos, float4* __restrict__ sv_w) {
  pdl_entry();
  for (int l = l0; l < T.depth; ++l) {
    const Geom& P = T.layer[l];
    const Geom& C = T.layer[l - 1];
    const uint3 d = make_uint3(T.decim[l][0], T.decim[l][1], T.decim[l][2]);
    for (size_t k = threadIdx.x; k < P.points(); k += blockDim.x)
      aggregate_point(P, C, d, sv_pos + T.base[l - 1], sv_w + T.base[l - 1], sv_pos + T.base[l], sv_w + T.base[l], k);
    __syncthreads();
  }
}

template <int KIND, bool REF>
__device__ __forceinline__ void add_pair(float3& acc, float qx, float qy, float qz, float4 p, float4 a, float sr,
                                         float sc) {
  if (REF)
    ref_accum<KIND>(acc, qx, qy, qz, p, a, sr, sc);
  else
    fast_accum<KIND>(acc, qx, qy, qz, p, a, sr, sc);
}

struct Frame {
  unsigned ix, iy, iz;
  int layer;
  unsigned counter;
  float ax, ay, az;
};

// Walk the tree from the root for query q (vortonSim.cpp:1650-1905).
template <int KIND, bool REF>
__device__ float3 tree_walk(const TreeParams& T, const float4* __restrict__ sp, const float4* __restrict__ sw,
                            const float4* __restrict__ ps, const float4* __restrict__ w, int n, float qx, float qy,
                            float qz, float sr, float sc) {
  float3 res = make_float3(0.f, 0.f, 0.f);
  if (T.depth <= 1) {  // no tree: direct sum (vortonSim.cpp:2125-2128)
    for (int i = 0; i < n; ++i) add_pair<KIND, REF>(res, qx, qy, qz, ps[i], w[i], sr, sc);
    return res;
  }
  Frame st[kMaxLayers];
  int top = 0;
  st[0] = Frame{0u, 0u, 0u, T.depth - 1, 0u, 0.f, 0.f, 0.f};
  const float mfac = 0.0001f;
  for (;;) {
    Frame& F = st[top];
    const int L = F.layer;
    const unsigned d0 = T.decim[L][0], d1 = T.decim[L][1], d2 = T.decim[L][2];
    if (F.counter == d0 * d1 * d2) {
      if (top == 0) {
        res = make_float3(F.ax, F.ay, F.az);
        break;
      }
      const float cx = F.ax, cy = F.ay, cz = F.az;
      --top;
      Frame& Pf = st[top];
      if (REF) {
        Pf.ax = __fadd_rn(Pf.ax, cx);
        Pf.ay = __fadd_rn(Pf.ay, cy);
        Pf.az = __fadd_rn(Pf.az, cz);
      } else {
        Pf.ax += cx;
        Pf.ay += cy;
        Pf.az += cz;
      }
      Pf.counter++;
      continue;
    }
    const Geom& C = T.layer[L - 1];
    const unsigned c = F.counter;
    const unsigned ix = c % d0, iy = (c / d0) % d1, iz = c / (d0 * d1);
    const unsigned chx = F.ix * d0 + ix, chy = F.iy * d1 + iy, chz = F.iz * d2 + iz;
    bool open = false;
    if (L > 1) {
      const float mx = __fmul_rn(mfac, C.cell[0]);
      const float my = __fmul_rn(mfac, C.cell[1]);
      const float mz = __fadd_rn(__fmul_rn(mfac, C.cell[2]), (0.0f == C.cell[2]) ? FLT_MIN : 0.0f);
      const float lox = __fadd_rn(C.mn[0], __fmul_rn((float)chx, C.cell[0]));
      const float hix = __fadd_rn(C.mn[0], __fmul_rn((float)(chx + 1), C.cell[0]));
      const float loy = __fadd_rn(C.mn[1], __fmul_rn((float)chy, C.cell[1]));
      const float hiy = __fadd_rn(C.mn[1], __fmul_rn((float)(chy + 1), C.cell[1]));
      const float loz = __fadd_rn(C.mn[2], __fmul_rn((float)chz, C.cell[2]));
      const float hiz = __fadd_rn(C.mn[2], __fmul_rn((float)(chz + 1), C.cell[2]));
      open = (qx >= __fsub_rn(lox, mx)) && (qy >= __fsub_rn(loy, my)) && (qz >= __fsub_rn(loz, mz)) &&
             (qx < __fadd_rn(hix, mx)) && (qy < __fadd_rn(hiy, my)) && (qz < __fadd_rn(hiz, mz));
    }
    if (open) {
      ++top;
      st[top] = Frame{chx, chy, chz, L - 1, 0u, 0.f, 0.f, 0.f};
      continue;
    }
    const size_t o = T.base[L - 1] + chx + (size_t)C.np[0] * (chy + (size_t)C.np[1] * chz);
    float3 acc = make_float3(F.ax, F.ay, F.az);
    add_pair<KIND, REF>(acc, qx, qy, qz, sp[o], sw[o], sr, sc);
    F.ax = acc.x;
    F.ay = acc.y;
    F.az = acc.z;
    F.counter++;
  }
  return res;
}

// FAST walk's per-cell constants for one call's spread factors sr, sc:
// tp = (centroid, 1 / R), tw = (angular velocity x 2/3 R^3 sc, R^2), R =
// size / 2 x sr -- what fast_accum derives from (sp, sw) at every pair.
__global__ void k_tree_prep(const float4* __restrict__ sp, const float4* __restrict__ sw, size_t total, float sr,
                            float sc, float4* __restrict__ tp, float4* __restrict__ tw) {
  pdl_entry();
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= total) return;
  const float4 p = sp[k], a = sw[k];
  const float radius = p.w * 0.5f * sr;
  const float s = VG_TWO_THIRDS * radius * radius * radius * sc;
  tp[k] = make_float4(p.x, p.y, p.z, 1.0f / radius);
  tw[k] = make_float4(a.x * s, a.y * s, a.z * s, radius * radius);
}

// fast_accum's law from prepared constants (the same mathematics, the scale
// folded into the angular velocity).
template <int KIND>
__device__ __forceinline__ void prep_accum(float3& acc, float qx, float qy, float qz, float4 tp, float4 tw) {
  const float d0 = qx - tp.x, d1 = qy - tp.y, d2 = qz - tp.z;
  const float dist2 = fmaf(d0, d0, fmaf(d1, d1, d2 * d2));
  if (KIND == 0) {
    const float inv = fminf(rsqrtf(dist2), tp.w);
    const float law = inv * inv * inv;
    const float b0 = d0 * law, b1 = d1 * law, b2 = d2 * law;
    acc.x = fmaf(tw.y, b2, fmaf(-tw.z, b1, acc.x));
    acc.y = fmaf(tw.z, b0, fmaf(-tw.x, b2, acc.y));
    acc.z = fmaf(tw.x, b1, fmaf(-tw.y, b0, acc.z));
  } else {
    const float law = (dist2 < tw.w) ? dist2 * tp.w * tp.w * tp.w : rsqrtf(dist2);
    acc.x = fmaf(tw.x, law, acc.x);
    acc.y = fmaf(tw.y, law, acc.y);
    acc.z = fmaf(tw.z, law, acc.z);
  }
}

// FAST form of the same walk.  The opening test is geometric and separable
// per axis (the query lies in the child's box widened by 1e-4 cells along x,
// y and z), so the cells opened at a layer always form a box of 1 or 2 cells
// per axis (2 where the query is within the margin of a face -- every grid
// point is).  Walk the layers with that box in registers: the children of the
// open cells that are not themselves opened add their monopoles, the opened
// ones form the next layer's box.  Same cells as tree_walk, summed layer by
// layer instead of depth first (FAST numerics sum in any order).
template <int KIND>
__device__ float3 tree_walk_fast(const TreeParams& T, const float4* __restrict__ tp, const float4* __restrict__ tw,
                                 const float4* __restrict__ ps, const float4* __restrict__ w, int n, float qx,
                                 float qy, float qz, float sr, float sc) {
  float3 acc = make_float3(0.f, 0.f, 0.f);
  if (T.depth <= 1) {  // no tree: direct sum (vortonSim.cpp:2125-2128)
    for (int i = 0; i < n; ++i) fast_accum<KIND>(acc, qx, qy, qz, ps[i], w[i], sr, sc);
    return acc;
  }
  const float mfac = 0.0001f;
  const float q[3] = {qx, qy, qz};
  unsigned f0[3] = {0u, 0u, 0u}, fn[3] = {1u, 1u, 1u};  // open box of layer L: [f0, f0 + fn) per axis
  for (int L = T.depth - 1; L >= 1; --L) {
    const Geom& C = T.layer[L - 1];
    unsigned c0[3], cn[3], o0[3], on[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const unsigned d = T.decim[L][a];
      c0[a] = f0[a] * d;
      cn[a] = fn[a] * d;
      on[a] = 0;
      o0[a] = 0;
      if (L > 1) {  // children open along this axis: a contiguous run of 1 or 2
        const float m = (a == 2) ? __fadd_rn(__fmul_rn(mfac, C.cell[2]), (0.0f == C.cell[2]) ? FLT_MIN : 0.0f)
                                 : __fmul_rn(mfac, C.cell[a]);
        for (unsigned i = 0; i < cn[a]; ++i) {
          const unsigned ch = c0[a] + i;
          const float lo = __fadd_rn(C.mn[a], __fmul_rn((float)ch, C.cell[a]));
          const float hi = __fadd_rn(C.mn[a], __fmul_rn((float)(ch + 1), C.cell[a]));
          if (q[a] >= __fsub_rn(lo, m) && q[a] < __fadd_rn(hi, m)) {
            if (on[a] == 0) o0[a] = ch;
            ++on[a];
          }
        }
      }
    }
    const bool any = on[0] && on[1] && on[2];
    // the layer's cells (fewer than 2^32 in a layer); a row's cells are
    // consecutive, visited up to 4 at a time with their loads issued
    // together; an opened cell's term is computed and dropped (acc kept)
    const float4* __restrict__ lp = tp + T.base[L - 1];
    const float4* __restrict__ lw = tw + T.base[L - 1];
    const unsigned sy = C.np[0], sz = C.np[0] * C.np[1];
    for (unsigned iz = 0; iz < cn[2]; ++iz) {
      const unsigned chz = c0[2] + iz;
      const bool oz = any && chz - o0[2] < on[2];
      for (unsigned iy = 0; iy < cn[1]; ++iy) {
        const unsigned chy = c0[1] + iy;
        const bool oyz = oz && chy - o0[1] < on[1];
        const unsigned row = c0[0] + sy * chy + sz * chz;
        for (unsigned ix0 = 0; ix0 < cn[0]; ix0 += 4) {
          float4 cp[4], cw[4];
#pragma unroll
          for (unsigned u = 0; u < 4; ++u)
            if (ix0 + u < cn[0]) {
              cp[u] = lp[row + ix0 + u];
              cw[u] = lw[row + ix0 + u];
            }
#pragma unroll
          for (unsigned u = 0; u < 4; ++u) {
            const unsigned ix = ix0 + u;
            if (ix >= cn[0]) break;
            float3 next = acc;
            prep_accum<KIND>(next, qx, qy, qz, cp[u], cw[u]);
            if (!(oyz && c0[0] + ix - o0[0] < on[0])) acc = next;
          }
        }
      }
    }
    if (!any) break;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      f0[a] = o0[a];
      fn[a] = on[a];
    }
  }
  return acc;
}

// REFERENCE numerics walk the raw cells (sp, sw); FAST the prepared ones (tp, tw).
template <int KIND, bool REF>
__device__ __forceinline__ float3 walk(const TreeParams& T, const float4* __restrict__ sp,
                                       const float4* __restrict__ sw, const float4* __restrict__ tp,
                                       const float4* __restrict__ tw, const float4* __restrict__ ps,
                                       const float4* __restrict__ w, int n, float qx, float qy, float qz, float sr,
                                       float sc) {
  if (REF) return tree_walk<KIND, true>(T, sp, sw, ps, w, n, qx, qy, qz, sr, sc);
  return tree_walk_fast<KIND>(T, tp, tw, ps, w, n, qx, qy, qz, sr, sc);
}

template <int KIND, bool REF>
__global__ void __launch_bounds__(128) k_tree_eval(const __grid_constant__ TreeParams T, const float4* __restrict__ sp,
                                                    const float4* __restrict__ sw, const float4* __restrict__ tp,
                                                    const float4* __restrict__ tw, const float4* __restrict__ ps,
                                                    const float4* __restrict__ w, int n, const float4* __restrict__ q,
                                                    int m, float sr, float sc, float4* __restrict__ out) {
  pdl_entry();
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  const float4 v = q[j];
  const float3 r = walk<KIND, REF>(T, sp, sw, tp, tw, ps, w, n, v.x, v.y, v.z, sr, sc);
  out[j] = make_float4(r.x, r.y, r.z, 0.f);
}

// Boundary points: z faces (nx*ny each), y faces (nx*(nz-2)), x faces ((ny-2)*(nz-2)).
__device__ __forceinline__ bool face_point(const Geom& g, size_t t, unsigned& x, unsigned& y, unsigned& z) {
  const size_t nx = g.np[0], ny = g.np[1], nz = g.np[2];
  const size_t fz = nx * ny;
  if (t < 2 * fz) {
    z = (t < fz) ? 0 : (unsigned)(nz - 1);
    const size_t r = t % fz;
    x = (unsigned)(r % nx);
    y = (unsigned)(r / nx);
    return nz > 1 || t < fz;
  }
  t -= 2 * fz;
  const size_t iz = nz > 2 ? nz - 2 : 0;
  const size_t fy = nx * iz;
  if (t < 2 * fy) {
    y = (t < fy) ? 0 : (unsigned)(ny - 1);
    const size_t r = t % fy;
    x = (unsigned)(r % nx);
    z = (unsigned)(r / nx) + 1;
    return ny > 1 || t < fy;
  }
  t -= 2 * fy;
  const size_t iy = ny > 2 ? ny - 2 : 0;
  const size_t fx = iy * iz;
  if (t < 2 * fx) {
    x = (t < fx) ? 0 : (unsigned)(nx - 1);
    const size_t r = t % fx;
    y = (unsigned)(r % iy) + 1;
    z = (unsigned)(r / iy) + 1;
    return nx > 1 || t < fx;
  }
  return false;
}

template <bool REF>
__global__ void __launch_bounds__(128) k_boundary_vecpot(const __grid_constant__ TreeParams T, Geom g,
                                                          const float4* __restrict__ sp, const float4* __restrict__ sw,
                                                          const float4* __restrict__ tp, const float4* __restrict__ tw,
                                                          const float4* __restrict__ ps, const float4* __restrict__ w,
                                                          int n, int copy_odd_x, size_t nface,
                                                          float* __restrict__ grid3) {
  pdl_entry();
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nface) return;
  unsigned x, y, z;
  if (!face_point(g, t, x, y, z)) return;
  const bool full_row = (z == 0 || z == g.np[2] - 1 || y == 0 || y == g.np[1] - 1);
  unsigned xq = x;
  bool zero = false;
  if (copy_odd_x && (x & 1u)) {
    // odd x reuses the preceding point's value; on rows that only visit the
    // two x faces, x-1 was not computed and still holds zero
    if (full_row || g.np[0] - 1 == 1)
      xq = x - 1;
    else
      zero = true;
  }
  const float nudge = 1.0f - 2.0f * FLT_EPSILON;  // vortonSim.cpp:2063-2064
  float3 r = make_float3(0.f, 0.f, 0.f);
  if (!zero) {
    const float qx = __fadd_rn(g.mn[0], __fmul_rn((float)xq, __fmul_rn(g.cell[0], nudge)));
    const float qy = __fadd_rn(g.mn[1], __fmul_rn((float)y, __fmul_rn(g.cell[1], nudge)));
    const float qz = __fadd_rn(g.mn[2], __fmul_rn((float)z, __fmul_rn(g.cell[2], nudge)));
    r = walk<1, REF>(T, sp, sw, tp, tw, ps, w, n, qx, qy, qz, 1.0f, 1.0f);
  }
  const size_t o = x + (size_t)g.np[0] * (y + (size_t)g.np[1] * z);
  grid3[3 * o] = r.x;
  grid3[3 * o + 1] = r.y;
  grid3[3 * o + 2] = r.z;
}

// Gather-form splat: point P accumulates from the 8 cells P - {0,1}^3 in
// ascending vorton index (k-way merge of the cells' sorted lists).
__global__ void __launch_bounds__(128) k_splat(Geom g, const float4* __restrict__ ps, const float4* __restrict__ w,
                                               const unsigned* __restrict__ start, const unsigned* __restrict__ items,
                                               float scale, float four_pi_over3, float cell_volume,
                                               float* __restrict__ grid3) {
  pdl_entry();
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= g.points()) return;
  // volumeCorrection = scale * (4 pi / 3 * r^3) / cellVolume, r = first vorton's radius
  const float radius = __fmul_rn(ps[0].w, 0.5f);
  const float vorton_volume = __fmul_rn(four_pi_over3, __fmul_rn(__fmul_rn(radius, radius), radius));
  const float corr = __fdiv_rn(__fmul_rn(scale, vorton_volume), cell_volume);
  const unsigned nx = g.np[0], ny = g.np[1], nz = g.np[2];
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
  (void)nz;
  float ax = 0.f, ay = 0.f, az = 0.f;
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
    const float4 a = w[best];
    // Accumulate (uniformGrid.h:1278-1342): this point is corner `bo` of the vorton's cell.
    const float pp[3] = {p.x, p.y, p.z};
    float tw[3], om[3];
#pragma unroll
    for (int ax3 = 0; ax3 < 3; ++ax3) {
      const unsigned idx = bin_axis(pp[ax3], g.mn[ax3], g.cpe[ax3]);
      const float cmin = __fadd_rn(g.mn[ax3], __fmul_rn((float)idx, g.cell[ax3]));
      const float t = __fmul_rn(__fsub_rn(pp[ax3], cmin), g.cpe[ax3]);
      const float lo = t > 0.0f ? t : 0.0f;  // Clamp0to1 = Min2(Max2(x, 0), 1) (vec3.h:565-571)
      tw[ax3] = lo < 1.0f ? lo : 1.0f;
      om[ax3] = __fsub_rn(1.0f, tw[ax3]);
    }
    const float fx = (bo & 1) ? tw[0] : om[0];
    const float fy = (bo & 2) ? tw[1] : om[1];
    const float fz = (bo & 4) ? tw[2] : om[2];
    const float wt = __fmul_rn(__fmul_rn(fx, fy), fz);
    const float ix = __fmul_rn(__fmul_rn(a.x, 2.0f), corr);
    const float iy = __fmul_rn(__fmul_rn(a.y, 2.0f), corr);
    const float iz = __fmul_rn(__fmul_rn(a.z, 2.0f), corr);
    ax = __fadd_rn(ax, __fmul_rn(wt, ix));
    ay = __fadd_rn(ay, __fmul_rn(wt, iy));
    az = __fadd_rn(az, __fmul_rn(wt, iz));
  }
  grid3[3 * k] = ax;
  grid3[3 * k + 1] = ay;
  grid3[3 * k + 2] = az;
}

TreeParams make_params(const Tree& t) {
  TreeParams T;
  T.depth = t.depth;
  for (int l = 0; l < t.depth; ++l) {
    T.layer[l] = t.layer[l];
    for (int a = 0; a < 3; ++a) T.decim[l][a] = t.decim[l][a];
    T.base[l] = t.base[l];
  }
  return T;
}

}  // namespace

vg_status build_tree(Ctx* c, const Geom& g, const float4* ps, const float4* w, size_t n, const CellLists& cl,
                     Tree* t) {
  t->depth = nested_shape(g, t->layer, t->decim);
  if (t->depth <= 0 || t->depth > kMaxLayers) return fail(c, VG_TOO_LARGE, "influence tree: too many layers");
  size_t total = 0;
  for (int l = 0; l < t->depth; ++l) {
    t->base[l] = total;
    total += t->layer[l].points();
  }
  t->total = total;
  vg_status st = VG_OK;
  float4* mem = (float4*)ws(c, S_TREE, 2 * total * sizeof(float4), &st);
  if (st != VG_OK) return st;
  t->sv_pos = mem;
  t->sv_w = mem + total;
  const Geom& leaf = t->layer[0];
  pdl_launch(c->stream, blocks_for(leaf.points(), 256), 256, 0, k_leaf, leaf, ps, w, cl.start, cl.items, t->sv_pos,
                                                                  t->sv_w);
  VG_LAUNCHED(c);
  // the first layer from which every layer is small: those run in one CTA
  int l0 = t->depth;
  while (l0 > 1 && t->layer[l0 - 1].points() <= kTopLayerPoints) --l0;
  for (int l = 1; l < l0; ++l) {
    const Geom& P = t->layer[l];
    const uint3 d = make_uint3(t->decim[l][0], t->decim[l][1], t->decim[l][2]);
    pdl_launch(c->stream, blocks_for(P.points(), 128), 128, 0, k_aggregate, P, t->layer[l - 1], d, t->sv_pos + t->base[l - 1],
                                                                     t->sv_w + t->base[l - 1], t->sv_pos + t->base[l],
                                                                     t->sv_w + t->base[l]);
    VG_LAUNCHED(c);
  }
  if (l0 < t->depth) {
    pdl_launch(c->stream, 1, kTopThreads, 0, k_aggregate_top, make_params(*t), l0, t->sv_pos, t->sv_w);
    VG_LAUNCHED(c);
  }
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

// The FAST walk's prepared cells (workspace slot S_TREEPREP) for spread
// factors sr, sc; nothing when the tree has no layers (the walk then sums the
// vortons directly).
static vg_status tree_prep(Ctx* c, const Tree& t, float sr, float sc, float4** tp, float4** tw) {
  if (t.depth <= 1 || t.total == 0) return VG_OK;
  vg_status st = VG_OK;
  float4* buf = (float4*)ws(c, S_TREEPREP, 2 * t.total * sizeof(float4), &st);
  if (st != VG_OK) return st;
  *tp = buf;
  *tw = buf + t.total;
  pdl_launch(c->stream, blocks_for(t.total, 256), 256, 0, k_tree_prep, t.sv_pos, t.sv_w, t.total, sr, sc, *tp, *tw);
  VG_LAUNCHED(c);
  return VG_OK;
}

vg_status launch_tree_eval(Ctx* c, int kind, bool ref, const Tree& t, const float4* ps, const float4* w, size_t n,
                           const float4* q, size_t m, float sr, float sc, float4* out) {
  if (m == 0) return VG_OK;
  const TreeParams T = make_params(t);
  const unsigned blocks = blocks_for(m, 128);
  float4 *tp = nullptr, *tw = nullptr;
  if (!ref) {
    vg_status st = tree_prep(c, t, sr, sc, &tp, &tw);
    if (st != VG_OK) return st;
  }
#define VG_TREE_LAUNCH(K, R) \
  pdl_launch(c->stream, blocks, 128, 0, k_tree_eval<K, R>, T, t.sv_pos, t.sv_w, tp, tw, ps, w, (int)n, q, (int)m, sr, sc, out)
  if (kind == 0) {
    if (ref) VG_TREE_LAUNCH(0, true); else VG_TREE_LAUNCH(0, false);
  } else {
    if (ref) VG_TREE_LAUNCH(1, true); else VG_TREE_LAUNCH(1, false);
  }
#undef VG_TREE_LAUNCH
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

vg_status launch_boundary_vecpot(Ctx* c, const Tree& t, const Geom& g, const float4* ps, const float4* w, size_t n,
                                 bool copy_odd_x, bool ref, float* grid3) {
  const TreeParams T = make_params(t);
  const size_t nx = g.np[0], ny = g.np[1], nz = g.np[2];
  const size_t nface = 2 * nx * ny + 2 * nx * (nz > 2 ? nz - 2 : 0) + 2 * (ny > 2 ? ny - 2 : 0) * (nz > 2 ? nz - 2 : 0);
  if (nface == 0) return VG_OK;
  if (ref) {
    pdl_launch(c->stream, blocks_for(nface, 128), 128, 0, k_boundary_vecpot<true>, 
        T, g, t.sv_pos, t.sv_w, nullptr, nullptr, ps, w, (int)n, copy_odd_x ? 1 : 0, nface, grid3);
  } else {
    float4 *tp = nullptr, *tw = nullptr;
    vg_status st = tree_prep(c, t, 1.0f, 1.0f, &tp, &tw);
    if (st != VG_OK) return st;
    pdl_launch(c->stream, blocks_for(nface, 128), 128, 0, k_boundary_vecpot<false>, 
        T, g, t.sv_pos, t.sv_w, tp, tw, ps, w, (int)n, copy_odd_x ? 1 : 0, nface, grid3);
  }
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

vg_status launch_splat(Ctx* c, const Geom& g, const float4* ps, const float4* w, size_t n, const CellLists& cl,
                       float scale, float radius, float* grid3) {
  const size_t pts = g.points();
  if (n == 0) {
    VG_CUDA(c, cudaMemsetAsync(grid3, 0, pts * 3 * sizeof(float), c->stream));
    return VG_OK;
  }
  // volume correction (vortonSim.cpp:2398-2402) from the first vorton's radius,
  // evaluated in the kernel from ps[0].w so no host round trip is needed
  volatile float cell_volume = g.cell[0] * g.cell[1];
  cell_volume = cell_volume * g.cell[2];
  const float four_pi = 4.0f * 3.1415926535897932384626433832795f;
  const float four_pi_over3 = four_pi / 3.0f;
  (void)radius;
  pdl_launch(c->stream, blocks_for(pts, 128), 128, 0, k_splat, g, ps, w, cl.start, cl.items, scale, four_pi_over3,
                                                        cell_volume, grid3);
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

}  // namespace vg
