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

// Velocity (KIND 0) with packed FP32x2 arithmetic (FADD2 / FMUL2 / FFMA2):
// each thread carries its 8 targets as 4 pairs, and every source is staged in
// shared memory already duplicated into pairs (-p, 1/R, w, -w), so each
// operation below advances two targets in one instruction.  The per-target
// operations and their order are those of k_direct_fast<0> (and the source
// constants those of k_prep_sources<0>, computed here while staging), so the
// results are bit-identical to it; only the instruction count changes (about
// 11 issue slots per interaction instead of 19).
// 8 targets per thread (128 registers) was the fastest of the shapes measured
// on GB300 (4 to 16 targets; scalar accumulation FFMAs or a scalar law mixed in
// were slower): the FFMA2s all run on the heavy half of the FMA pipe, which the
// profile shows ~70% busy.  CTAs of 256 threads, 2 per SM, beat 4 CTAs of 128
// by ~4%: the tile barriers keep a CTA's warps together, whereas independent
// small CTAs on one SM finish far apart (measured 39-100 us for equal work)
// and leave the SM short of warps at the end.
// With more than one source chunk the partial sums go to a scratch buffer and
// k_reduce_pair adds them in chunk order.  (Reducing them inside this kernel,
// by the last CTA of each target block or after a grid-wide barrier, or
// launching the reduction as a programmatic dependent, measured no faster.)
constexpr int kPairTPT = 8;
constexpr int kPairThreads = 256;



__global__ void __launch_bounds__(kPairThreads, 2)
    k_direct_pair(const float4* __restrict__ ps, const float4* __restrict__ w, int n, int chunk, float sr, float sc,
                  const float4* __restrict__ q, int m, float* __restrict__ partial, float4* __restrict__ out) {
  pdl_entry();
  constexpr int kPairs = kPairTPT / 2;
  __shared__ float4 sh[5 * kTile];
  const int base = blockIdx.x * (kPairThreads * kPairTPT) + threadIdx.x;
  float2 qx[kPairs], qy[kPairs], qz[kPairs], ax[kPairs], ay[kPairs], az[kPairs];
#pragma unroll
  for (int pr = 0; pr < kPairs; ++pr) {
    const int j0 = base + 2 * pr * kPairThreads, j1 = j0 + kPairThreads;
    const float4 v0 = (j0 < m) ? q[j0] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 v1 = (j1 < m) ? q[j1] : make_float4(0.f, 0.f, 0.f, 0.f);
    qx[pr] = make_float2(v0.x, v1.x);
    qy[pr] = make_float2(v0.y, v1.y);
    qz[pr] = make_float2(v0.z, v1.z);
    ax[pr] = ay[pr] = az[pr] = make_float2(0.f, 0.f);
  }
  const int k0 = blockIdx.y * chunk;
  const int k1 = min(n, k0 + chunk);
  for (int tile = k0; tile < k1; tile += kTile) {
    const int cnt = min(kTile, k1 - tile);
    __syncthreads();
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
    __syncthreads();
#pragma unroll 2
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
  if (gridDim.y == 1) {  // one chunk: the sums are final (0 + sum, as the reduction would give)
#pragma unroll
    for (int pr = 0; pr < kPairs; ++pr) {
      const int j0 = base + 2 * pr * kPairThreads, j1 = j0 + kPairThreads;
      if (j0 < m) out[j0] = make_float4(0.f + ax[pr].x, 0.f + ay[pr].x, 0.f + az[pr].x, 0.f);
      if (j1 < m) out[j1] = make_float4(0.f + ax[pr].y, 0.f + ay[pr].y, 0.f + az[pr].y, 0.f);
    }
    return;
  }
  float* mine = partial + (size_t)blockIdx.y * (size_t)m * 3;
#pragma unroll
  for (int pr = 0; pr < kPairs; ++pr) {
    const int j0 = base + 2 * pr * kPairThreads, j1 = j0 + kPairThreads;
    if (j0 < m) {
      mine[3 * j0] = ax[pr].x;
      mine[3 * j0 + 1] = ay[pr].x;
      mine[3 * j0 + 2] = az[pr].x;
    }
    if (j1 < m) {
      mine[3 * j1] = ax[pr].y;
      mine[3 * j1 + 1] = ay[pr].y;
      mine[3 * j1 + 2] = az[pr].y;
    }
  }
}

// Sums the chunks' partial sums in chunk order (as k_reduce_partials), with
// up to 16 chunks' loads issued before the first add: the sum is bound by the
// latency of these loads, not by their bytes.
__global__ void __launch_bounds__(256) k_reduce_pair(const float* __restrict__ partial, int ks, int m,
                                                     float4* __restrict__ out, float* __restrict__ grid3, int pts,
                                                     float4* __restrict__ vel) {
  pdl_entry();
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  constexpr int kBatch = 16;
  float x = 0.f, y = 0.f, z = 0.f;
  for (int k0 = 0; k0 < ks; k0 += kBatch) {
    float v[kBatch][3];
#pragma unroll
    for (int k = 0; k < kBatch; ++k)
      if (k0 + k < ks) {
        const float* p = partial + ((size_t)(k0 + k) * m + j) * 3;
        v[k][0] = p[0];
        v[k][1] = p[1];
        v[k][2] = p[2];
      }
#pragma unroll
    for (int k = 0; k < kBatch; ++k)
      if (k0 + k < ks) {
        x += v[k][0];
        y += v[k][1];
        z += v[k][2];
      }
  }
  if (!grid3) {
    out[j] = make_float4(x, y, z, 0.f);
  } else if (j < pts) {  // the velocity step's split: gridpoints as float[3], vortons as records
    grid3[3 * j] = x;
    grid3[3 * j + 1] = y;
    grid3[3 * j + 2] = z;
  } else {
    vel[j - pts] = make_float4(x, y, z, 0.f);
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
  unsigned tblocks = 0, ksplit = 0;
  const int chunk = direct_split(kind, n, m, &tblocks, &ksplit);
  vg_status st = VG_OK;
  if (kind == 0) {
    float* partial = nullptr;
    if (ksplit > 1) {
      partial = (float*)ws(c, S_DIRECT, (size_t)ksplit * m * 3 * sizeof(float), &st);
      if (st != VG_OK) return st;
    }
    dim3 grid(tblocks, ksplit);
    pdl_launch(c->stream, grid, dim3(kPairThreads), 0, k_direct_pair, ps, w, (int)n, chunk, sr, sc, q, (int)m, partial,
               out);
    VG_LAUNCHED(c);
    if (ksplit > 1) {
      const bool to_split = split != nullptr;
      pdl_launch(c->stream, blocks_for(m, 256), 256, 0, k_reduce_pair, (const float*)partial, (int)ksplit, (int)m, out,
                 to_split ? split->grid3 : (float*)nullptr, to_split ? (int)split->pts : 0,
                 to_split ? split->vel : (float4*)nullptr);
      if (split_done) *split_done = to_split;
      VG_LAUNCHED(c);
    }
    VG_CUDA(c, cudaGetLastError());
    return VG_OK;
  }
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
  int chunk = direct_split(kind, n, m, &tblocks, &ksplit);
  while (ksplit > 1 && (size_t)ksplit * m * 3 * sizeof(float) > room) {
    const unsigned k = ksplit - 1;
    chunk = (int)((n + k - 1) / k);
    ksplit = (unsigned)((n + chunk - 1) / chunk);
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
    e = launch_plain(st, dim3(tblocks, ksplit), dim3(kPairThreads), k_direct_pair, ps, w, (int)n, chunk, spread_range,
                     spread_circ, q, (int)m, ksplit > 1 ? partial : (float*)nullptr, out);
    if (e != cudaSuccess) return noalloc_fail(e, "k_direct_pair launch");
    if (ksplit > 1) {
      e = launch_plain(st, dim3(blocks_for(m, 256)), dim3(256), k_reduce_pair, (const float*)partial, (int)ksplit,
                       (int)m, out, (float*)nullptr, 0, (float4*)nullptr);
      if (e != cudaSuccess) return noalloc_fail(e, "k_reduce_pair launch");
    }
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
