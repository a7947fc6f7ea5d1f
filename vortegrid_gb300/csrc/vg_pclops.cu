// Particle operations on device-resident particles, for engines that keep
// vortons and tracers on the GPU across frames instead of copying records in
// and out each step:
//   * PclOpWind::Operate (Particles/Operation/pclOpWind.cpp:18-42):
//     vel = (wind_weight wind) + src_weight vel per component;
//   * PclOpKillAge::Operate (Particles/Operation/pclOpKillAge.cpp:22-47):
//     particles with int(frame - birth) > age_max are removed.  The reference
//     walks the array and fills each removed slot with the last particle
//     (Particles::Kill, Particles/particle.h:490-495), testing the slot again.
//     The survivors' final order follows from that walk: with m survivors,
//     the slots below m keep their survivors, and the k-th removed slot below
//     m (ascending) receives the k-th survivor at or above m counted from the
//     end.  One exclusive scan of the survival flags gives both ranks, so the
//     permutation is two parallel passes, in place (sources lie at or above m,
//     destinations below it).
#include "vg_internal.cuh"

struct vg_ctx : public vg::Ctx {};

using namespace vg;

namespace {

__global__ void k_wind(float4* __restrict__ vel, size_t m, float tx, float ty, float tz, float sw) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  float4 v = vel[i];
  v.x = __fadd_rn(tx, __fmul_rn(sw, v.x));
  v.y = __fadd_rn(ty, __fmul_rn(sw, v.y));
  v.z = __fadd_rn(tz, __fmul_rn(sw, v.z));
  vel[i] = v;
}

__device__ __forceinline__ bool survives(const int* birth, size_t i, unsigned frame, int age_max) {
  return !((int)(frame - (unsigned)birth[i]) > age_max);
}

__global__ void k_survive_flags(const int* __restrict__ birth, size_t n, unsigned frame, int age_max,
                                unsigned* __restrict__ flag) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flag[i] = survives(birth, i, frame, age_max) ? 1u : 0u;
}

// src[k] = the k-th survivor at or above m counted from the end (P: exclusive
// scan of the flags, P[n] = m).
__global__ void k_kill_sources(const unsigned* __restrict__ flag, const unsigned* __restrict__ P, size_t n,
                               unsigned* __restrict__ src) {
  const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned m = P[n];
  if (p >= n || p < m || !flag[p]) return;
  src[m - P[p] - 1] = (unsigned)p;
}

// Removed slot i below m (its rank among removed slots: i - P[i]) takes its source.
__global__ void k_kill_fill(const unsigned* __restrict__ flag, const unsigned* __restrict__ P, size_t n,
                            const unsigned* __restrict__ src, float4* a, float4* b, float4* c, int* birth) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned m = P[n];
  if (i >= m || flag[i]) return;
  const unsigned s = src[i - P[i]];
  if (a) a[i] = a[s];
  if (b) b[i] = b[s];
  if (c) c[i] = c[s];
  birth[i] = birth[s];
}

}  // namespace

extern "C" {

vg_status vg_wind_device(vg_ctx* c, float* vel4, size_t m, const float wind[3], float wind_weight, float src_weight) {
  if (!c || !wind || (m && !vel4)) return VG_INVALID;
  if (wind_weight == 0.0f && src_weight == 1.0f) return VG_OK;  // the reference's do-nothing weights
  if (m == 0) return VG_OK;
  const float t[3] = {wind_weight * wind[0], wind_weight * wind[1], wind_weight * wind[2]};
  k_wind<<<blocks_for(m, 256), 256, 0, c->stream>>>((float4*)vel4, m, t[0], t[1], t[2], src_weight);
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

vg_status vg_kill_age_device(vg_ctx* c, float* a4, float* b4, float* c4, int* birth, size_t m, unsigned frame,
                             int age_max, size_t* m_out) {
  if (!c || !m_out || (m && !birth)) return VG_INVALID;
  *m_out = m;
  if (m == 0) return VG_OK;
  if (m > 0x7fffffff) return fail(c, VG_TOO_LARGE, "more than 2^31 particles");
  vg_status st = VG_OK;
  unsigned* flag = (unsigned*)ws(c, S_PCL, (3 * m + 1) * sizeof(unsigned), &st);
  if (st != VG_OK) return st;
  unsigned* P = flag + m;      // m + 1 entries
  unsigned* src = P + m + 1;   // at most m entries
  const unsigned nb = blocks_for(m, 256);
  k_survive_flags<<<nb, 256, 0, c->stream>>>(birth, m, frame, age_max, flag);
  VG_CUDA(c, cudaGetLastError());
  if ((st = exclusive_scan(c, flag, m, P, true)) != VG_OK) return st;
  k_kill_sources<<<nb, 256, 0, c->stream>>>(flag, P, m, src);
  k_kill_fill<<<nb, 256, 0, c->stream>>>(flag, P, m, src, (float4*)a4, (float4*)b4, (float4*)c4, birth);
  VG_CUDA(c, cudaGetLastError());
  unsigned h = 0;
  VG_CUDA(c, cudaMemcpyAsync(&h, P + m, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
  VG_CUDA(c, cudaStreamSynchronize(c->stream));
  *m_out = h;
  return VG_OK;
}

}  // extern "C"
