// Emitters appending particles to device-resident arrays (PclOpEmit,
// Particles/Operation/pclOpEmit.h:16-34):
//   * vg_emit_device -- PclOpEmit::Operate (pclOpEmit.cpp:188-210).  A handful
//     of particles a frame, each the template plus RandomSpread of the spread
//     drawn from the C library's rand(): the records are made on the host in
//     the reference's draw order and appended with one copy and one kernel,
//     so the live particles never leave the device.
//   * vg_emit_grid_device -- PclOpEmit::Emit (pclOpEmit.cpp:77-186), the
//     tracer seeding: one thread per sub-cell computes its particle (sub-cell
//     s = cell * m^3 + sub, both in z, y, x order, is the reference's emission
//     order) from three draws -- the host's rand() stream copied in, or a
//     counter-based hash on the device.  With vortons, their density
//     deviation grid is the gather-form accumulation of the density kernel,
//     its range a min/max reduction, and the kept sub-cells are compacted in
//     order by an exclusive scan of their flags.
// Positions are formed in the reference's FP32 operation order with
// round-to-nearest intrinsics; the scalars the reference computes once
// (particle size with the C library's powf, sub-cell shift, jitter
// magnitude, 1 / RAND_MAX) are computed the same way on the host.
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "vg_internal.cuh"

struct vg_ctx : public vg::Ctx {};

using namespace vg;

namespace {

constexpr int kEmitThreads = 256;

// One Operate record: the 17 values of vg_particle_values and the birth frame.
struct EmitRecord {
  float v[17];
  int birth;
};

// Writes one particle into whichever arrays the group keeps.
__device__ __forceinline__ void put(const vg_particles& P, size_t i, const float p[3], float size, const float v[3],
                                    const float w[3], const float o[3], float dens, const float fire[3], int birth) {
  reinterpret_cast<float4*>(P.pos_size)[i] = make_float4(p[0], p[1], p[2], size);
  if (P.vel4) reinterpret_cast<float4*>(P.vel4)[i] = make_float4(v[0], v[1], v[2], 0.0f);
  if (P.angvel4) reinterpret_cast<float4*>(P.angvel4)[i] = make_float4(w[0], w[1], w[2], 0.0f);
  if (P.orient4) reinterpret_cast<float4*>(P.orient4)[i] = make_float4(o[0], o[1], o[2], 0.0f);
  if (P.density) P.density[i] = dens;
  if (P.fire4) reinterpret_cast<float4*>(P.fire4)[i] = make_float4(fire[0], fire[1], fire[2], 0.0f);
  if (P.birth) P.birth[i] = birth;
}

__global__ void k_emit_append(vg_particles P, const EmitRecord* __restrict__ rec, size_t k) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= k) return;
  const EmitRecord r = rec[i];
  put(P, P.count + i, r.v, r.v[16], r.v + 3, r.v + 9, r.v + 6, r.v[12], r.v + 13, r.birth);
}

// The counter-based jitter stream: MurmurHash3's 32-bit finalizer (fmix32,
// Austin Appleby, public domain) of the draw index's low word keyed by the
// seed and its high word, scaled to [0, RAND_MAX].
__device__ __forceinline__ unsigned fmix32(unsigned h) {
  h ^= h >> 16;
  h *= 0x85ebca6bu;
  h ^= h >> 13;
  h *= 0xc2b2ae35u;
  h ^= h >> 16;
  return h;
}

__device__ __forceinline__ int jitter_hash(unsigned seed, unsigned long long d, unsigned long long range) {
  const unsigned key = fmix32(seed ^ ((unsigned)(d >> 32) * 0x9e3779b9u + 0x7f4a7c15u));
  const unsigned h = fmix32((unsigned)d ^ key);
  return (int)(((unsigned long long)h * range) >> 32);
}

struct EmitGrid {
  Geom g;
  unsigned m, m3, nc[3];
  float shift[3], jm[3], size, one_over_rand_max, scale;
  unsigned seed;
  unsigned long long range;  // RAND_MAX + 1
  const int* draws;          // host rand() stream (3 per sub-cell) or NULL for the hash
  const float* dev;          // density deviation grid (vortons given) or NULL
};

// Position of sub-cell s's particle: min corner + (it / m) spacing + shift +
// RandomSpread(jitter magnitude), the Vec3's z drawn first.
__device__ __forceinline__ void emit_position(const EmitGrid& E, size_t s, float p[3]) {
  const size_t cell = s / E.m3;
  const unsigned sub = (unsigned)(s - cell * E.m3);
  const unsigned idx[3] = {(unsigned)(cell % E.nc[0]), (unsigned)((cell / E.nc[0]) % E.nc[1]),
                           (unsigned)(cell / ((size_t)E.nc[0] * E.nc[1]))};
  const unsigned it[3] = {sub % E.m, (sub / E.m) % E.m, sub / (E.m * E.m)};
  int r[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const unsigned long long d = 3ull * s + (unsigned long long)j;
    r[2 - j] = E.draws ? E.draws[d] : jitter_hash(E.seed, d, E.range);
  }
  const float fm = __uint2float_rn(E.m);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float cmin = __fadd_rn(E.g.mn[a], __fmul_rn(__uint2float_rn(idx[a]), E.g.cell[a]));
    const float disp = __fmul_rn(__fdiv_rn(__uint2float_rn(it[a]), fm), E.g.cell[a]);
    const float j = __fmul_rn(E.jm[a], __fsub_rn(__fmul_rn(__int2float_rn(r[a]), E.one_over_rand_max), 0.5f));
    p[a] = __fadd_rn(__fadd_rn(__fadd_rn(cmin, disp), E.shift[a]), j);
  }
}

// With vortons: whether the particle is kept, and its density.
__device__ __forceinline__ bool emit_mask(const EmitGrid& E, const float p[3], float* dens, int* flag) {
  if (!inside_cells(E.g, p[0], p[1], p[2])) {
    atomicOr(flag, DF_OUT_OF_GRID);
    return false;
  }
  float here;
  interp<1>(E.g, E.dev, p[0], p[1], p[2], &here);
  *dens = __fmul_rn(__fadd_rn(here, E.scale), 1.0f);
  return fabsf(__fdiv_rn(here, E.scale)) >= 0.5f;
}

__device__ __forceinline__ void emit_write(const vg_particles& P, size_t i, const EmitGrid& E, const float p[3],
                                           float dens) {
  const float zero[3] = {0.0f, 0.0f, 0.0f}, fire[3] = {0.0f, 0.0f, 1.0f};
  put(P, P.count + i, p, E.size, zero, zero, zero, dens, fire, 0);
}

// No vortons: every sub-cell's particle, at its own index.
__global__ void __launch_bounds__(kEmitThreads) k_emit_grid_all(EmitGrid E, vg_particles P, size_t total) {
  for (size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x; s < total; s += (size_t)gridDim.x * blockDim.x) {
    float p[3];
    emit_position(E, s, p);
    emit_write(P, s, E, p, 1.0f);
  }
}

__global__ void __launch_bounds__(kEmitThreads) k_emit_grid_flags(EmitGrid E, size_t total, unsigned* __restrict__ keep,
                                                                  int* flag) {
  for (size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x; s < total; s += (size_t)gridDim.x * blockDim.x) {
    float p[3], dens;
    emit_position(E, s, p);
    keep[s] = emit_mask(E, p, &dens, flag) ? 1u : 0u;
  }
}

__global__ void __launch_bounds__(kEmitThreads) k_emit_grid_kept(EmitGrid E, vg_particles P, size_t total,
                                                                 const unsigned* __restrict__ keep,
                                                                 const unsigned* __restrict__ rank, int* flag) {
  for (size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x; s < total; s += (size_t)gridDim.x * blockDim.x) {
    if (!keep[s]) continue;
    float p[3], dens = 0.0f;
    emit_position(E, s, p);
    emit_mask(E, p, &dens, flag);
    emit_write(P, rank[s], E, p, dens);
  }
}

// Order-preserving float -> unsigned map, for min/max by atomics.
__device__ __forceinline__ unsigned ordered(float f) {
  const unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// FindValueRange (Core/SpatialPartition/uniformGridMath.cpp:517-536): lohi[0]
// = ordered min, lohi[1] = ordered max (min and max are exact in any order).
__global__ void __launch_bounds__(kEmitThreads) k_value_range(const float* __restrict__ v, size_t n,
                                                              unsigned* __restrict__ lohi) {
  unsigned lo = 0xffffffffu, hi = 0u;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const unsigned o = ordered(v[i]);
    lo = o < lo ? o : lo;
    hi = o > hi ? o : hi;
  }
#pragma unroll
  for (int d = 16; d; d >>= 1) {
    const unsigned a = __shfl_xor_sync(0xffffffffu, lo, d), b = __shfl_xor_sync(0xffffffffu, hi, d);
    lo = a < lo ? a : lo;
    hi = b > hi ? b : hi;
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(lohi, lo);
    atomicMax(lohi + 1, hi);
  }
}

float unordered(unsigned o) {
  const unsigned u = (o & 0x80000000u) ? (o & 0x7fffffffu) : ~o;
  float f;
  memcpy(&f, &u, sizeof(f));
  return f;
}

// RandomSpread (Core/Math/math.h:183-188) on the host.
float random_spread(float spread, float one_over_rand_max) {
  return spread * ((float)rand() * one_over_rand_max - 0.5f);
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

unsigned grid_blocks(size_t n) {
  const size_t want = (n + kEmitThreads - 1) / kEmitThreads;
  const size_t cap = (size_t)sm_count() * 16;
  return (unsigned)(want < cap ? (want ? want : 1) : cap);
}

}  // namespace

extern "C" {

vg_status vg_emit_device(vg_ctx* c, vg_emitter* em, float time_step, unsigned frame, vg_particles* p) {
  if (!c || !em || !p || !p->pos_size) return VG_INVALID;
  const float f = time_step * em->emit_rate + em->remainder;
  if (!(f < 2147483648.0f && f > -2147483648.0f)) return fail(c, VG_TOO_LARGE, "emit: particle count out of range");
  const int k = (int)f;
  const size_t kk = k > 0 ? (size_t)k : 0;
  if (p->count > p->capacity || kk > p->capacity - p->count)
    return fail(c, VG_TOO_LARGE, "emit: the particle arrays are full");
  em->remainder = f - (float)k;
  if (kk == 0) return VG_OK;
  static_assert(sizeof(vg_particle_values) == 17 * sizeof(float), "vg_particle_values is 17 floats");
  float t[17], s[17];
  memcpy(t, &em->tmpl, sizeof(t));
  memcpy(s, &em->spread, sizeof(s));
  const float one_over_rand_max = 1.0f / (float)RAND_MAX;
  std::vector<EmitRecord> rec(kk);
  for (size_t i = 0; i < kk; ++i) {
    EmitRecord& r = rec[i];
    for (int v = 0; v < 4; ++v)  // Vec3 members: z, y, x drawn in that order
      for (int a = 2; a >= 0; --a) r.v[3 * v + a] = t[3 * v + a] + random_spread(s[3 * v + a], one_over_rand_max);
    for (int v = 12; v < 17; ++v) r.v[v] = t[v] + random_spread(s[v], one_over_rand_max);
    r.birth = (int)frame;
  }
  vg_status st = VG_OK;
  EmitRecord* d = (EmitRecord*)ws(c, S_EMIT, kk * sizeof(EmitRecord), &st);
  if (st != VG_OK) return st;
  VG_CUDA(c, cudaMemcpyAsync(d, rec.data(), kk * sizeof(EmitRecord), cudaMemcpyHostToDevice, c->stream));
  k_emit_append<<<blocks_for(kk, kEmitThreads), kEmitThreads, 0, c->stream>>>(*p, d, kk);
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  VG_CUDA(c, cudaStreamSynchronize(c->stream));
  p->count += kk;
  return VG_OK;
}

vg_status vg_emit_grid_device(vg_ctx* c, const vg_grid_geom* gg, unsigned multiplier, const float* vorton_pos_size,
                              const float* vorton_density, size_t n_vortons, int jitter, unsigned seed,
                              vg_particles* p) {
  if (!c || !gg || !p || !p->pos_size || multiplier == 0) return VG_INVALID;
  if (jitter != VG_JITTER_HOST_RAND && jitter != VG_JITTER_HASH) return VG_INVALID;
  const bool masked = vorton_pos_size != nullptr;
  if (masked && n_vortons && !vorton_density) return VG_INVALID;
  if (n_vortons > 0x7fffffff) return fail(c, VG_TOO_LARGE, "more than 2^31 vortons");
  if (p->count > p->capacity) return VG_INVALID;
  EmitGrid E;
  E.g = to_geom(*gg);
  for (int a = 0; a < 3; ++a) {
    if (E.g.np[a] < 2) return fail(c, VG_INVALID, "emit grid: fewer than 2 points on an axis");
    E.nc[a] = E.g.np[a] - 1;
  }
  if (multiplier > 1290) return fail(c, VG_TOO_LARGE, "emit grid: more than 2^31 particles");
  const unsigned long long m3 = (unsigned long long)multiplier * multiplier * multiplier;
  const unsigned long long total = (unsigned long long)E.nc[0] * E.nc[1] * E.nc[2] * m3;
  if (total > 0x7fffffffull) return fail(c, VG_TOO_LARGE, "emit grid: more than 2^31 particles");
  E.m = multiplier;
  E.m3 = (unsigned)m3;
  const float* sp = E.g.cell;
  E.size = 0.5f * powf(sp[0] * sp[1] * sp[2], 1.0f / 3.0f) / (float)multiplier;
  const float jm_scale = 1.9999f * (1.0f - FLT_EPSILON);
  for (int a = 0; a < 3; ++a) {
    E.shift[a] = (0.5f * sp[a]) * (1.0f / (float)multiplier);
    E.jm[a] = E.shift[a] * jm_scale;
  }
  E.one_over_rand_max = 1.0f / (float)RAND_MAX;
  E.seed = seed;
  E.range = (unsigned long long)RAND_MAX + 1ull;
  E.scale = 0.0f;
  E.draws = nullptr;
  E.dev = nullptr;

  // workspace: [draws | deviation grid | range | keep flags | ranks]
  const size_t pts = E.g.points();
  const size_t b_draws = jitter == VG_JITTER_HOST_RAND ? align256(3 * total * sizeof(int)) : 0;
  const size_t b_dev = masked ? align256(pts * sizeof(float)) : 0;
  const size_t b_range = masked ? 256 : 0;
  const size_t b_keep = masked ? align256(total * sizeof(unsigned)) : 0;
  const size_t b_rank = masked ? align256((total + 1) * sizeof(unsigned)) : 0;
  vg_status st = VG_OK;
  char* w = (char*)ws(c, S_EMIT, b_draws + b_dev + b_range + b_keep + b_rank + 256, &st);
  if (st != VG_OK) return st;
  int* draws = (int*)w;
  float* dev = (float*)(w + b_draws);
  unsigned* lohi = (unsigned*)(w + b_draws + b_dev);
  unsigned* keep = (unsigned*)(w + b_draws + b_dev + b_range);
  unsigned* rank = (unsigned*)(w + b_draws + b_dev + b_range + b_keep);

  if (masked) {
    // PopulateDensityDeviationGridFromParticles and FindValueRange (pclOpEmit.cpp:101-110)
    if ((st = launch_density_deviation(c, E.g, (const float4*)vorton_pos_size, vorton_density, n_vortons, 1.0f,
                                       dev)) != VG_OK)
      return st;
    VG_CUDA(c, cudaMemsetAsync(lohi, 0xff, sizeof(unsigned), c->stream));
    VG_CUDA(c, cudaMemsetAsync(lohi + 1, 0, sizeof(unsigned), c->stream));
    k_value_range<<<grid_blocks(pts), kEmitThreads, 0, c->stream>>>(dev, pts, lohi);
    VG_LAUNCHED(c);
    VG_CUDA(c, cudaGetLastError());
    unsigned h[2];
    VG_CUDA(c, cudaMemcpyAsync(h, lohi, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    VG_CUDA(c, cudaStreamSynchronize(c->stream));
    const float alo = fabsf(unordered(h[0])), ahi = fabsf(unordered(h[1]));
    E.scale = ahi > alo ? ahi : alo;
    if (E.scale == 0.0f) return VG_OK;  // no deviation anywhere: the reference emits nothing
    E.dev = dev;
  } else if (total > p->capacity - p->count) {
    return fail(c, VG_TOO_LARGE, "emit grid: the particle arrays are full");
  }
  if (jitter == VG_JITTER_HOST_RAND) {
    std::vector<int> h(3 * total);
    for (size_t i = 0; i < h.size(); ++i) h[i] = rand();
    VG_CUDA(c, cudaMemcpyAsync(draws, h.data(), h.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    VG_CUDA(c, cudaStreamSynchronize(c->stream));  // h is released on return
    E.draws = draws;
  }
  const unsigned nb = grid_blocks(total);
  if (!masked) {
    k_emit_grid_all<<<nb, kEmitThreads, 0, c->stream>>>(E, *p, (size_t)total);
    VG_LAUNCHED(c);
    VG_CUDA(c, cudaGetLastError());
    VG_CUDA(c, cudaStreamSynchronize(c->stream));
    p->count += total;
    return VG_OK;
  }
  int* flag = outside_flag(c);
  k_emit_grid_flags<<<nb, kEmitThreads, 0, c->stream>>>(E, (size_t)total, keep, flag);
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  if ((st = exclusive_scan(c, keep, (size_t)total, rank, true)) != VG_OK) return st;
  unsigned kept = 0;
  VG_CUDA(c, cudaMemcpyAsync(&kept, rank + total, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
  VG_CUDA(c, cudaStreamSynchronize(c->stream));
  if (kept > p->capacity - p->count) {
    sync_and_check(c, "emit grid");  // clears a pending out-of-grid mark; the size error is the one reported
    return fail(c, VG_TOO_LARGE, "emit grid: the particle arrays are full");
  }
  k_emit_grid_kept<<<nb, kEmitThreads, 0, c->stream>>>(E, *p, (size_t)total, keep, rank, flag);
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  st = sync_and_check(c, "emit grid");
  p->count += kept;
  return st;
}

}  // extern "C"
