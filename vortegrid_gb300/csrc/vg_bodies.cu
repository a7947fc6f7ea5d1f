// Fluid-body boundary conditions on device-resident particles: rigid spheres
// and boxes (solid, or hollow containers) in the fluid.
//
//  * vg_collide_vortons_device -- FluidBodySim::CollideVortonsSlice
//    (FluidBodySim/fluidBodySim.cpp:759-1180) for each body in turn, as
//    SolveBoundaryConditions runs it for vortons (fluidBodySim.cpp:1651-1715):
//    a vorton within a boundary layer of 1.5 radii of the body is moved just
//    outside it, bounced (impact coefficient 1.01), given the Brinkman
//    penalty vorticity at the contact point blended with gain 0.1 and the
//    body's spin, and exchanges heat with the body through its density;
//  * vg_collide_tracers_device -- CollideTracersSlice (fluidBodySim.cpp:
//    1300-1455): a tracer in contact is moved outside and bounced;
//  * vg_remove_embedded_device -- RemoveEmbeddedParticles
//    (fluidBodySim.cpp:365-417): particles inside bodies are removed in the
//    order the reference's swap-with-last walk leaves the survivors.
// One thread per particle; every particle's update depends on its own state
// and the body only (a particle that meets a hollow box's wall is processed
// again, up to 5 times, as the reference's loop does), so the particle
// results are the reference's bit for bit.  Each body's impulse, heat and
// temperature sums are reduced per block in a fixed order and then over the
// blocks in order, in FP64: deterministic, and within rounding of the
// reference's serial float sums.
#include <float.h>

#include <string>

#include "vg_internal.cuh"

struct vg_ctx : public vg::Ctx {};

using namespace vg;

namespace {

constexpr int kMaxBodies = 16;
constexpr int kBodyThreads = 256;

struct Body {
  int box;
  float parity, brad;
  float pos[3], vel[3], angvel[3], row[9];
  float pn[6][3], pw[6];
  float temperature, conductivity;
};

// The body of the 32-float layout (include/vortegrid.h): a SphereShape, or a
// ConvexPolytope made by ConvexPolytope_MakeBox (Collision/convexPolytope.cpp:
// 346-376) with its bounding sphere.  Host FP32 arithmetic in the reference's order.
bool load_body(const float* q, Body* b, std::string* err) {
  memset(b, 0, sizeof(*b));
  if (q[0] != 0.0f && q[0] != 1.0f) {
    *err = "body shape must be 0 (sphere) or 1 (box)";
    return false;
  }
  b->box = q[0] != 0.0f;
  b->parity = (b->box && q[1] != 0.0f) ? -1.0f : 1.0f;
  for (int a = 0; a < 3; ++a) {
    b->pos[a] = q[2 + a];
    b->vel[a] = q[5 + a];
    b->angvel[a] = q[8 + a];
  }
  for (int k = 0; k < 9; ++k) b->row[k] = q[11 + k];
  b->temperature = q[23];
  b->conductivity = q[24];
  if (!b->box) {
    if (!(q[20] >= 0.0f)) {
      *err = "sphere radius must not be negative";
      return false;
    }
    b->brad = q[20];
    return true;
  }
  const float half[3] = {q[20] * 0.5f, q[21] * 0.5f, q[22] * 0.5f};
  for (int a = 0; a < 3; ++a) {
    for (int k = 0; k < 3; ++k) b->pn[2 * a][k] = b->pn[2 * a + 1][k] = 0.0f;
    b->pn[2 * a][a] = 1.0f;
    b->pn[2 * a + 1][a] = -1.0f;
    b->pw[2 * a] = b->pw[2 * a + 1] = half[a];
  }
  if (b->parity < 0.0f) {
    const float thin = 1.0f - FLT_EPSILON;
    const float m01 = half[0] < half[1] ? half[0] : half[1];
    b->brad = thin * (m01 < half[2] ? m01 : half[2]);
  } else {
    const float fatten = 1.0f + FLT_EPSILON;
    const float m2 = q[20] * q[20] + q[21] * q[21] + q[22] * q[22];
    b->brad = 0.5f * fatten * sqrtf(m2);
  }
  return true;
}

struct V3 {
  float x, y, z;
};
__device__ __forceinline__ V3 mk(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 add(V3 a, V3 b) { return mk(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)); }
__device__ __forceinline__ V3 sub(V3 a, V3 b) { return mk(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)); }
__device__ __forceinline__ V3 mul(V3 a, float f) { return mk(__fmul_rn(a.x, f), __fmul_rn(a.y, f), __fmul_rn(a.z, f)); }
__device__ __forceinline__ float dot(V3 a, V3 b) {
  return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
  return mk(__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)), __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
            __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}
__device__ __forceinline__ float mag(V3 a) { return __fsqrt_rn(dot(a, a)); }
// Vec3::GetDirFast (vec3.h:429) and GetDir (vec3.h:428)
__device__ __forceinline__ V3 dirfast(V3 a) { return mul(a, ref_finvsqrtf(__fadd_rn(dot(a, a), FLT_MIN))); }
__device__ __forceinline__ V3 dir(V3 a) {
  return mul(mul(a, 1.0f), __fdiv_rn(1.0f, __fsqrt_rn(__fadd_rn(dot(a, a), FLT_MIN))));
}
__device__ __forceinline__ V3 from(const float* p) { return mk(p[0], p[1], p[2]); }

// Mat33::TransformByTranspose (mat33.h:131-134) and Transform (mat33.h:108-113)
__device__ __forceinline__ V3 xform_t(const Body& b, V3 v) {
  return mk(dot(mk(b.row[0], b.row[1], b.row[2]), v), dot(mk(b.row[3], b.row[4], b.row[5]), v),
            dot(mk(b.row[6], b.row[7], b.row[8]), v));
}
__device__ __forceinline__ V3 xform(const Body& b, V3 v) {
  return mk(dot(mk(b.row[0], b.row[3], b.row[6]), v), dot(mk(b.row[1], b.row[4], b.row[7]), v),
            dot(mk(b.row[2], b.row[5], b.row[8]), v));
}

// ConvexPolytope::ContactDistance (convexPolytope.cpp:97-144)
__device__ float contact_distance(const Body& b, V3 q, int* idx) {
  const V3 r = xform_t(b, sub(q, from(b.pos)));
  float largest = -FLT_MAX;
  for (int i = 0; i < 6; ++i) {
    const float d = __fsub_rn(dot(r, from(b.pn[i])), b.pw[i]);
    if (d > largest) {
      largest = d;
      *idx = i;
    }
  }
  return __fmul_rn(largest, b.parity);
}

// ConvexPolytope::CollisionDistance with velocities (convexPolytope.cpp:151-196)
__device__ float collision_distance(const Body& b, V3 q, V3 qv, int* idx) {
  const V3 r = xform_t(b, sub(q, from(b.pos)));
  const V3 rv = xform_t(b, sub(qv, from(b.vel)));
  float largest = -FLT_MAX;
  for (int i = 0; i < 6; ++i) {
    const float d = __fsub_rn(dot(r, from(b.pn[i])), b.pw[i]);
    if (d > largest) {
      const float speed = __fmul_rn(dot(rv, from(b.pn[i])), b.parity);
      if (speed <= 0.0f || d >= 0.0f || b.parity < 0.0f) {
        largest = d;
        *idx = i;
      }
    }
  }
  return __fmul_rn(largest, b.parity);
}

// ConvexPolytope::ContactPoint (convexPolytope.cpp:325-339)
__device__ __forceinline__ V3 contact_point(const Body& b, V3 q, int idx, float dist, V3* n) {
  *n = mul(xform(b, from(b.pn[idx])), b.parity);
  return sub(q, mul(*n, dist));
}

// Block sum of K values in a fixed order: lanes by a tree, then the 8 warps
// in order (threads 0..K-1), in FP32 -- FP64 arithmetic runs at a small
// fraction of FP32's rate on this part, and FP64 sums over every block
// dominated the launch; thread k writes the block's partial sum k.
template <int K>
__device__ void block_sums(float (&v)[K], float* __restrict__ out) {
  __shared__ float sh[kBodyThreads / 32][K];
  // most blocks hold no particle in contact with the body: their sums are zero
  bool any = false;
#pragma unroll
  for (int k = 0; k < K; ++k) any = any || v[k] != 0.0f;
  if (!__syncthreads_or(any)) {
    if (threadIdx.x < K) out[K * blockIdx.x + threadIdx.x] = 0.0f;
    return;
  }
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) sh[warp][k] = v[k];
  __syncthreads();
  if (threadIdx.x < K) {
    float s = 0.0f;
    for (int w = 0; w < kBodyThreads / 32; ++w) s += sh[w][threadIdx.x];
    out[K * blockIdx.x + threadIdx.x] = s;
  }
}

// The blocks' partial sums added in a fixed order by one CTA: thread t sums
// the contiguous run of blocks [t c, (t + 1) c) with compensated (Kahan) FP32
// additions -- or, for a count (the last value when kCount), exactly in
// integers -- then a tree over the threads in FP64 (halving strides):
// deterministic, within a few FP32 rounding units of the exact sum.
constexpr int kSumThreads = 256;
template <int K, bool kCount>
__global__ void __launch_bounds__(kSumThreads) k_sum_blocks(const float* __restrict__ part, int nb,
                                                            double* __restrict__ out) {
  __shared__ double sh[K][kSumThreads];
  const int t = threadIdx.x;
  const int per = (nb + kSumThreads - 1) / kSumThreads;
  const int b0 = min(nb, t * per), b1 = min(nb, b0 + per);
  constexpr int KF = kCount ? K - 1 : K;
  float s[K], comp[K];
  unsigned long long cnt = 0;
#pragma unroll
  for (int k = 0; k < K; ++k) s[k] = comp[k] = 0.0f;
  for (int b = b0; b < b1; ++b) {
#pragma unroll
    for (int k = 0; k < KF; ++k) {
      const float y = __fsub_rn(part[K * (size_t)b + k], comp[k]);
      const float tt = __fadd_rn(s[k], y);
      comp[k] = __fsub_rn(__fsub_rn(tt, s[k]), y);
      s[k] = tt;
    }
    if (kCount) cnt += (unsigned long long)part[K * (size_t)b + K - 1];
  }
#pragma unroll
  for (int k = 0; k < KF; ++k) sh[k][t] = (double)s[k];
  if (kCount) sh[K - 1][t] = (double)cnt;
  __syncthreads();
  for (int h = kSumThreads / 2; h > 0; h >>= 1) {
    if (t < h)
#pragma unroll
      for (int k = 0; k < K; ++k) sh[k][t] += sh[k][t + h];
    __syncthreads();
  }
  if (t < K) out[t] = sh[t][0];
}

// The bodies of one call, in order (a kernel parameter).
struct Bodies {
  Body b[kMaxBodies];
};

// One body's CollideVortonsSlice for one vorton, on the vorton's state in
// registers (position + size, velocity, angular velocity, density); the sums
// of its contacts go to acc: angular impulse (3), heat to body, sum of
// particle temperatures, particles collided.  Returns whether it changed.
__device__ bool collide_vorton(const Body& B, float4& p4s, float4& v4s, float4& a4s, float& dens_s, float ambient,
                               float cp, float (&acc)[6]) {
  bool changed = false;
  {
    const float thin = __fsub_rn(1.0f, FLT_EPSILON), fatten = __fadd_rn(1.0f, FLT_EPSILON);
    const float nudge = __fadd_rn(1.0f, 1.0e-4f), impact = __fadd_rn(1.0f, 0.01f);
    const float one_over_cp = __fdiv_rn(1.0f, cp);
    const V3 bpos = from(B.pos), bvel = from(B.vel), bspin = from(B.angvel);
    int incr = 1, repeat = 0;
    for (int pass = 0; pass < 6; ++pass) {
      repeat = (0 == incr) ? repeat + 1 : 0;
      if (pass > 0 && incr != 0) break;
      incr = 1;
      const float4 p4 = p4s, v4 = v4s, a4 = a4s;
      V3 p = mk(p4.x, p4.y, p4.z), v = mk(v4.x, v4.y, v4.z), w = mk(a4.x, a4.y, a4.z);
      const float size = p4.w, r = __fmul_rn(size, 0.5f), r2 = __fmul_rn(r, r);
      const V3 s2v = sub(p, bpos);
      const float fs2v = mag(s2v);
      const float bnd = __fmul_rn(1.5f, r);
      bool broad;
      if (B.parity < 0.0f) {
        const float d = __fsub_rn(B.brad, bnd);
        broad = fs2v > __fmul_rn(d > 0.0f ? d : 0.0f, thin);
      } else {
        broad = fs2v < __fmul_rn(__fadd_rn(B.brad, bnd), fatten);
      }
      if (!broad) break;
      V3 cw, nrm;
      float cdist;
      if (!B.box) {
        const V3 d = mul(s2v, __fdiv_rn(1.0f, fs2v));
        cw = add(mul(d, B.brad), bpos);
        nrm = d;
        cdist = __fsub_rn(fs2v, B.brad);
      } else {
        int idx = 0;
        cdist = contact_distance(B, p, &idx);
        if (!(cdist < bnd)) break;
        cw = contact_point(B, p, idx, cdist, &nrm);
        if (B.parity < 0.0f && repeat < 5 && cdist < r) incr = 0;
      }
      acc[5] += 1.0f;
      V3 vort_old = mul(w, 2.0f);
      // (the flow relative to the body at the contact point, and the bend
      // direction formed from it, feed only the reference's disabled
      // placement approaches 1 and 2, fluidBodySim.cpp:951-975, so they are
      // not computed)
      const float disp = cdist < r ? r : cdist;
      p = add(cw, mul(mul(nrm, disp), nudge));
      {
        const float speed_n = dot(sub(v, bvel), nrm);
        v = add(v, mul(mul(nrm, -speed_n), impact));
      }
      if (repeat >= 1) {
        v = mk(0.f, 0.f, 0.f);
        w = mk(0.f, 0.f, 0.f);
        vort_old = w;
      } else {
        // Vorton::AssignVorticityByPenalty (vorton.h:275-306)
        const V3 rel = sub(cw, p);
        const V3 vd = sub(v, bvel);
        const float dist = __fsub_rn(mag(rel), __fmul_rn(size, 0.4f));
        const V3 vdir = dir(cross(vd, rel));
        const float vmag = __fdiv_rn(mag(vd), dist);
        w = mul(mul(vdir, vmag), 0.5f);
      }
      w = add(w, sub(mul(bspin, 1.0f), mul(vort_old, 0.5f)));
      {
        const float gain = 0.1f, one_minus = __fsub_rn(1.0f, gain);
        w = mul(add(mul(mul(w, 2.0f), gain), mul(vort_old, one_minus)), 0.5f);
      }
      const V3 angdiff = mul(sub(vort_old, mul(w, 2.0f)), 0.5f);
      float d_new;
      {
        const float d_old = dens_s;
        const float t_old = __fdiv_rn(__fmul_rn(300.0f, ambient), d_old);
        const float t_diff = __fsub_rn(B.temperature, t_old);
        const float g0 = __fmul_rn(__fmul_rn(__fmul_rn(B.conductivity, r), 0.03f), cp);
        const float g1 = g0 > -0.5f ? g0 : -0.5f;
        const float t_gain = g1 < 0.5f ? g1 : 0.5f;
        const float t_change = __fmul_rn(t_diff, t_gain);
        const float heat_ex = __fmul_rn(t_change, one_over_cp);
        const float t_new = __fadd_rn(t_old, t_change);
        d_new = __fdiv_rn(__fmul_rn(ambient, 300.0f), t_new);
        acc[3] -= heat_ex;
        acc[4] += t_old;
      }
      {
        const float pi_over_6 = __fdiv_rn(3.1415926535897932384626433832795f, 6.0f);
        const float volume = __fmul_rn(__fmul_rn(__fmul_rn(pi_over_6, size), size), size);
        const float moi = __fmul_rn(__fmul_rn(0.4f, __fmul_rn(d_new, volume)), r2);
        const V3 ai = mul(angdiff, moi);
        acc[0] += ai.x;
        acc[1] += ai.y;
        acc[2] += ai.z;
      }
      p4s = make_float4(p.x, p.y, p.z, p4.w);
      v4s = make_float4(v.x, v.y, v.z, v4.w);
      a4s = make_float4(w.x, w.y, w.z, a4.w);
      dens_s = d_new;
      changed = true;
    }
  }
  return changed;
}

// CollideVortonsSlice for every body in order, one vorton per thread: its
// state stays in registers from body to body (each body sees the vorton as
// the bodies before left it, as with one launch per body) and is written
// once.  Per body, block partial sums at part + 6 blocks k.
__global__ void __launch_bounds__(kBodyThreads) k_collide_vortons(const __grid_constant__ Bodies BB, int nb,
                                                                  float4* __restrict__ ps, float4* __restrict__ vel,
                                                                  float4* __restrict__ w4, float* __restrict__ dens,
                                                                  int n, float ambient, float cp,
                                                                  float* __restrict__ part) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float4 p4, v4, a4;
  float d = 0.f;
  if (i < n) {
    p4 = ps[i];
    v4 = vel[i];
    a4 = w4[i];
    d = dens[i];
  }
  bool changed = false;
  for (int k = 0; k < nb; ++k) {
    float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (i < n) changed |= collide_vorton(BB.b[k], p4, v4, a4, d, ambient, cp, acc);
    block_sums<6>(acc, part + (size_t)6 * gridDim.x * k);
  }
  if (i < n && changed) {
    ps[i] = p4;
    vel[i] = v4;
    w4[i] = a4;
    dens[i] = d;
  }
}

// One body's CollideTracersSlice for one tracer, on its state in registers;
// the sums of its contacts go to acc: linear impulse (3), angular impulse (3).
// dens: NULL, or the tracers' densities (tracer i's read when it collides).
// Returns whether it changed.
__device__ bool collide_tracer(const Body& B, float4& p4s, float4& v4s, const float* __restrict__ dens, int i,
                               float (&acc)[6]) {
  bool changed = false;
  {
    const float thin = __fsub_rn(1.0f, FLT_EPSILON), fatten = __fadd_rn(1.0f, FLT_EPSILON);
    const float nudge = __fadd_rn(1.0f, 1.0e-4f), impact = __fadd_rn(1.0f, 0.01f);
    const V3 bpos = from(B.pos), bvel = from(B.vel), bspin = from(B.angvel);
    int incr = 1, repeat = 0;
    for (int pass = 0; pass < 6; ++pass) {
      repeat = (0 == incr) ? repeat + 1 : 0;
      if (pass > 0 && incr != 0) break;
      incr = 1;
      const float4 p4 = p4s, v4 = v4s;
      const V3 p = mk(p4.x, p4.y, p4.z), v = mk(v4.x, v4.y, v4.z);
      const float size = p4.w, r = __fmul_rn(size, 0.5f);
      const V3 s2t = sub(p, bpos);
      const float fs2t = mag(s2t);
      bool broad;
      if (B.parity < 0.0f) {
        const float d = __fsub_rn(B.brad, r);
        broad = fs2t > __fmul_rn(d > 0.0f ? d : 0.0f, thin);
      } else {
        broad = fs2t < __fmul_rn(__fadd_rn(B.brad, r), fatten);
      }
      if (!broad) break;
      V3 cpt, nrm, disp_new;
      if (!B.box) {
        const float rescale = __fdiv_rn(__fmul_rn(__fadd_rn(B.brad, r), __fadd_rn(1.0f, FLT_EPSILON)), fs2t);
        disp_new = mul(s2t, rescale);
        cpt = disp_new;
        nrm = dirfast(s2t);
      } else {
        int idx = 0;
        const float cdist = collision_distance(B, p, v, &idx);
        if (!(cdist < r)) break;
        cpt = contact_point(B, p, idx, cdist, &nrm);
        disp_new = sub(add(cpt, mul(mul(nrm, r), nudge)), bpos);
        if (B.parity < 0.0f && repeat < 5) incr = 0;
      }
      const V3 vbody = add(bvel, cross(bspin, disp_new));
      const float speed_n = dot(sub(v, vbody), nrm);
      const V3 vnew = add(v, mul(mul(nrm, -speed_n), impact));
      const float pi_over_6 = __fdiv_rn(3.1415926535897932384626433832795f, 6.0f);
      const float d0 = dens ? dens[i] : 1.0f;
      const float mass = __fmul_rn(d0, __fmul_rn(__fmul_rn(__fmul_rn(pi_over_6, size), size), size));
      const V3 li = mul(sub(v, vnew), mass);
      const V3 ai = cross(sub(cpt, bpos), li);
      acc[0] += li.x;
      acc[1] += li.y;
      acc[2] += li.z;
      acc[3] += ai.x;
      acc[4] += ai.y;
      acc[5] += ai.z;
      const V3 pn = add(bpos, disp_new);
      p4s = make_float4(pn.x, pn.y, pn.z, p4.w);
      v4s = make_float4(vnew.x, vnew.y, vnew.z, v4.w);
      changed = true;
    }
  }
  return changed;
}

// CollideTracersSlice for every body in order, one tracer per thread, its
// state in registers from body to body and written once (as k_collide_vortons).
__global__ void __launch_bounds__(kBodyThreads) k_collide_tracers(const __grid_constant__ Bodies BB, int nb,
                                                                  float4* __restrict__ ps, float4* __restrict__ vel,
                                                                  const float* __restrict__ dens, int n,
                                                                  float* __restrict__ part) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float4 p4, v4;
  if (i < n) {
    p4 = ps[i];
    v4 = vel[i];
  }
  bool changed = false;
  for (int k = 0; k < nb; ++k) {
    float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (i < n) changed |= collide_tracer(BB.b[k], p4, v4, dens, i, acc);
    block_sums<6>(acc, part + (size_t)6 * gridDim.x * k);
  }
  if (i < n && changed) {
    ps[i] = p4;
    vel[i] = v4;
  }
}

// RemoveEmbeddedParticles' test for one body: survives unless inside it.
__global__ void k_embedded_flags(const __grid_constant__ Body B, const float4* __restrict__ ps, size_t n,
                                 unsigned* __restrict__ flag) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p4 = ps[i];
  const V3 p = mk(p4.x, p4.y, p4.z);
  bool kill = false;
  if (mag(sub(p, from(B.pos))) < B.brad) {
    if (!B.box) {
      kill = true;
    } else {
      int idx = 0;
      kill = contact_distance(B, p, &idx) < __fmul_rn(p4.w, 0.5f);
    }
  }
  flag[i] = kill ? 0u : 1u;
}

// As the kill-by-age compaction (vg_pclops.cu): the k-th survivor at or above
// m counted from the end fills the k-th removed slot below m.
__global__ void k_embedded_sources(const unsigned* __restrict__ flag, const unsigned* __restrict__ P, size_t n,
                                   unsigned* __restrict__ src) {
  const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned m = P[n];
  if (p >= n || p < m || !flag[p]) return;
  src[m - P[p] - 1] = (unsigned)p;
}

__global__ void k_embedded_fill(const unsigned* __restrict__ flag, const unsigned* __restrict__ P, size_t n,
                                const unsigned* __restrict__ src, float4* a, float4* b, float4* c, float* d) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned m = P[n];
  if (i >= m || flag[i]) return;
  const unsigned s = src[i - P[i]];
  a[i] = a[s];
  if (b) b[i] = b[s];
  if (c) c[i] = c[s];
  if (d) d[i] = d[s];
}

vg_status load_bodies(Ctx* c, const float* bodies, int nb, Body* out) {
  if (nb < 0 || nb > kMaxBodies) return fail(c, VG_INVALID, "between 0 and 16 bodies");
  if (nb && !bodies) return VG_INVALID;
  std::string err;
  for (int k = 0; k < nb; ++k)
    if (!load_body(bodies + 32 * k, out + k, &err)) return fail(c, VG_INVALID, "body " + std::to_string(k) + ": " + err);
  return VG_OK;
}

}  // namespace

extern "C" {

vg_status vg_collide_vortons_device(vg_ctx* c, const float* bodies, int nb, float* pos_size, float* vel4,
                                    float* angvel4, float* density, size_t n, float ambient_density,
                                    float specific_heat, float* body_out, unsigned long long* collided) {
  if (!c || (n && (!pos_size || !vel4 || !angvel4 || !density)) || (nb && !body_out)) return VG_INVALID;
  if (n > 0x7fffffff) return fail(c, VG_TOO_LARGE, "more than 2^31 vortons");
  if (!(ambient_density > 0.0f) || !(specific_heat > 0.0f))
    return fail(c, VG_INVALID, "ambient density and specific heat must be positive");
  Body B[kMaxBodies];
  vg_status st = load_bodies(c, bodies, nb, B);
  if (st != VG_OK) return st;
  const unsigned blocks = n ? blocks_for(n, kBodyThreads) : 1;
  double* sums = (double*)ws(c, S_BODY, 6 * kMaxBodies * sizeof(double) + (size_t)blocks * 6 * kMaxBodies * sizeof(float),
                             &st);
  if (st != VG_OK) return st;
  float* part = (float*)(sums + 6 * kMaxBodies);
  if (nb) {
    Bodies BB;
    memcpy(BB.b, B, sizeof(BB.b));
    k_collide_vortons<<<blocks, kBodyThreads, 0, c->stream>>>(BB, nb, (float4*)pos_size, (float4*)vel4,
                                                             (float4*)angvel4, density, (int)n, ambient_density,
                                                             specific_heat, part);
    ++c->launches;
  }
  for (int k = 0; k < nb; ++k) {
    k_sum_blocks<6, true><<<1, kSumThreads, 0, c->stream>>>(part + (size_t)6 * blocks * k, (int)blocks, sums + 6 * k);
    ++c->launches;
  }
  VG_CUDA(c, cudaGetLastError());
  double h[6 * kMaxBodies];
  if (nb) VG_CUDA(c, cudaMemcpyAsync(h, sums, 6 * nb * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  VG_CUDA(c, cudaStreamSynchronize(c->stream));
  for (int k = 0; k < nb; ++k) {
    float* o = body_out + 9 * k;
    o[0] = o[1] = o[2] = 0.0f;  // the smoothed-particle form applies no linear impulse (fluidBodySim.cpp:1163-1174)
    o[3] = (float)h[6 * k], o[4] = (float)h[6 * k + 1], o[5] = (float)h[6 * k + 2];
    o[6] = (float)h[6 * k + 3], o[7] = (float)h[6 * k + 4];
    const unsigned long long cnt = (unsigned long long)h[6 * k + 5];
    if (collided) collided[k] = cnt;
    // the body's new temperature (SolveBoundaryConditions, fluidBodySim.cpp:1703-1714), heat capacity
    // taken as one over the body's [25] entry when given, else 1
    const float t_body = bodies[32 * k + 23];
    const float inv_cap = bodies[32 * k + 25] > 0.0f ? bodies[32 * k + 25] : 1.0f;
    if (cnt) {
      const float avg = o[7] / (float)cnt;
      const float half = 0.5f * fabsf(avg - t_body);
      const float proposed = o[6] * inv_cap;
      const float clamped = proposed < -half ? -half : (proposed > half ? half : proposed);
      o[8] = t_body + clamped;
    } else {
      o[8] = t_body;
    }
  }
  return VG_OK;
}

vg_status vg_collide_tracers_device(vg_ctx* c, const float* bodies, int nb, float* pos_size, float* vel4,
                                    const float* density, size_t n, float* body_out) {
  if (!c || (n && (!pos_size || !vel4)) || (nb && !body_out)) return VG_INVALID;
  if (n > 0x7fffffff) return fail(c, VG_TOO_LARGE, "more than 2^31 tracers");
  Body B[kMaxBodies];
  vg_status st = load_bodies(c, bodies, nb, B);
  if (st != VG_OK) return st;
  const unsigned blocks = n ? blocks_for(n, kBodyThreads) : 1;
  double* sums = (double*)ws(c, S_BODY, 6 * kMaxBodies * sizeof(double) + (size_t)blocks * 6 * kMaxBodies * sizeof(float),
                             &st);
  if (st != VG_OK) return st;
  float* part = (float*)(sums + 6 * kMaxBodies);
  if (nb) {
    Bodies BB;
    memcpy(BB.b, B, sizeof(BB.b));
    k_collide_tracers<<<blocks, kBodyThreads, 0, c->stream>>>(BB, nb, (float4*)pos_size, (float4*)vel4, density,
                                                             (int)n, part);
    ++c->launches;
  }
  for (int k = 0; k < nb; ++k) {
    k_sum_blocks<6, false><<<1, kSumThreads, 0, c->stream>>>(part + (size_t)6 * blocks * k, (int)blocks, sums + 6 * k);
    ++c->launches;
  }
  VG_CUDA(c, cudaGetLastError());
  double h[6 * kMaxBodies];
  if (nb) VG_CUDA(c, cudaMemcpyAsync(h, sums, 6 * nb * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  VG_CUDA(c, cudaStreamSynchronize(c->stream));
  for (int k = 0; k < 6 * nb; ++k) body_out[k] = (float)h[k];
  return VG_OK;
}

vg_status vg_remove_embedded_device(vg_ctx* c, const float* bodies, int nb, float* pos_size, float* b4, float* c4,
                                    float* d1, size_t m, size_t* m_out) {
  if (!c || !m_out || (m && !pos_size)) return VG_INVALID;
  *m_out = m;
  if (m > 0x7fffffff) return fail(c, VG_TOO_LARGE, "more than 2^31 particles");
  Body B[kMaxBodies];
  vg_status st = load_bodies(c, bodies, nb, B);
  if (st != VG_OK) return st;
  if (m == 0 || nb == 0) return VG_OK;
  unsigned* flag = (unsigned*)ws(c, S_PCL, (3 * m + 1) * sizeof(unsigned), &st);
  if (st != VG_OK) return st;
  unsigned* P = flag + m;
  unsigned* src = P + m + 1;
  size_t cur = m;
  for (int k = 0; k < nb && cur > 0; ++k) {
    const unsigned blocks = blocks_for(cur, 256);
    k_embedded_flags<<<blocks, 256, 0, c->stream>>>(B[k], (const float4*)pos_size, cur, flag);
    VG_CUDA(c, cudaGetLastError());
    if ((st = exclusive_scan(c, flag, cur, P, true)) != VG_OK) return st;
    k_embedded_sources<<<blocks, 256, 0, c->stream>>>(flag, P, cur, src);
    k_embedded_fill<<<blocks, 256, 0, c->stream>>>(flag, P, cur, src, (float4*)pos_size, (float4*)b4, (float4*)c4, d1);
    c->launches += 3;
    VG_CUDA(c, cudaGetLastError());
    unsigned h = 0;
    VG_CUDA(c, cudaMemcpyAsync(&h, P + cur, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    VG_CUDA(c, cudaStreamSynchronize(c->stream));
    cur = h;
  }
  *m_out = cur;
  return VG_OK;
}

}  // extern "C"
