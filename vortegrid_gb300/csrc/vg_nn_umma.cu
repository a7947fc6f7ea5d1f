// 3x3x3 convolution on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// Implicit GEMM: M = 128 output voxels (a tile of 8 x 16 voxels in x, y at one
// z), N = CO_T output channels, K = 27 taps x 16-channel slices.  The tile's
// zero-padded halo (10 x 18 x 3 voxels) is stored "chunk-planar": channels
// 0..7 of every halo voxel, 16 bytes each, then channels 8..15.  In that layout
// the A operand of any tap is a K-major, no-swizzle shared-memory matrix:
// 8 consecutive voxels of one x row form a core matrix (8 rows x 16 bytes,
// contiguous), successive y rows are 10 voxels (160 bytes) apart (the stride
// between 8-row groups) and the second 8 channels are one plane further (the
// stride between K-adjacent core matrices).  So each tap is one
// tcgen05.mma.kind::f16 (BF16 x BF16 -> FP32, M = 128, N = CO_T, K = 16)
// reading the halo in place, accumulating in tensor memory.
//
// A CTA (4 warps) is persistent: it keeps the weights of its output-channel
// group for every input slice in shared memory (same planar layout: the B
// operand of tap t starts at row t * CO_T), walks its tiles slice by slice,
// and copies the next slice's halo with cp.async (two buffers) while the
// tensor cores work.
// Thread 0 issues the MMAs and commits them to the mbarrier of the halo buffer
// they read; that barrier gates both the buffer's reuse and, at the end of a
// tile, the epilogue, where each warp reads its 32 accumulator rows with
// tcgen05.ld (one voxel per thread), adds the bias, applies the activation and
// mask, and stores the voxel's channels.  Every mbarrier wait is bounded: on
// timeout the kernel raises a device error bit, stops issuing work, waits for
// its copies and frees its tensor memory.
#include <algorithm>

#include "vg_nn.cuh"

namespace vg {
namespace nn {

namespace {

constexpr int kTX = 8, kTY = 16;                  // tile: 8 x 16 x 1 voxels = M 128
constexpr int kHX = kTX + 2, kHY = kTY + 2;        // halo 10 x 18 x 3
constexpr int kNH = kHX * kHY * 3;                 // 540 halo voxels
constexpr int kPlane = kNH * 16;                   // bytes of one 8-channel plane of a halo slice
constexpr int kHaloBytes = 2 * kPlane;             // one 16-channel slice
constexpr size_t kUmmaWeightBytes = 100 * 1024;
constexpr long long kWaitLimit = 1LL << 24;
constexpr int kBufs = 2;                           // halo buffers in flight (3 costs a CTA per SM, measured slower)

__device__ __forceinline__ unsigned su32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void cp_async16(unsigned dst, const void* src, int src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(src_bytes));
}

__device__ __forceinline__ uint64_t smem_desc(unsigned addr, unsigned lbo, unsigned sbo) {
  return (uint64_t)((addr >> 4) & 0x3fff) | ((uint64_t)((lbo >> 4) & 0x3fff) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3fff) << 32) | ((uint64_t)1 << 46);  // no swizzle, version 1
}

// kind::f16 instruction descriptor: FP32 accumulate, BF16 A and B, both K-major.
__host__ __device__ constexpr unsigned idesc_bf16(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(n >> 3) << 17) | ((128u >> 4) << 24);
}

__device__ __forceinline__ bool mbar_wait(unsigned mbar, unsigned parity) {
  for (long long it = 0; it < kWaitLimit; ++it) {
    unsigned done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(mbar), "r"(parity));
    if (done) return true;
  }
  return false;
}

// Copies one 16-channel slice of the halo of the tile at (x0, y0, z0) into the
// planar buffer at byte address dst (zero-filled outside the volume).
__device__ __forceinline__ void issue_halo_planar(unsigned dst, const ConvIn& in, int x0, int y0, int z0, int ci0) {
  for (int s = threadIdx.x; s < kNH; s += blockDim.x) {
    const int ix = s % kHX, iy = (s / kHX) % kHY, iz = s / (kHX * kHY);
    const int z = z0 + iz - 1, y = y0 + iy - 1, x = x0 + ix - 1;
    const bool inside = z >= 0 && y >= 0 && x >= 0 && z < in.D && y < in.H && x < in.W;
    const __nv_bfloat16* p = in.x1;  // a valid address when nothing is read
    if (inside) {
      if (ci0 < in.C1) {
        if (in.up1) {
          const int H1 = in.H >> 1, W1 = in.W >> 1;
          p = in.x1 + (((size_t)(z >> 1) * H1 + (y >> 1)) * W1 + (x >> 1)) * in.C1 + ci0;
        } else {
          p = in.x1 + (((size_t)z * in.H + y) * in.W + x) * in.C1 + ci0;
        }
      } else {
        p = in.x2 + (((size_t)z * in.H + y) * in.W + x) * in.C2 + (ci0 - in.C1);
      }
    }
    const int nb = inside ? 16 : 0;
    cp_async16(dst + s * 16, p, nb);
    cp_async16(dst + kPlane + s * 16, p + 8, nb);
  }
}

// 16 consecutive FP32 accumulator columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(unsigned taddr, unsigned* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

// Epilogue of one tile: thread (warp w, lane l) owns accumulator row 32 w + l,
// i.e. voxel (x0 + row % 8, y0 + row / 8, z0), and its CO_T channels.
template <int CO_T>
__device__ __forceinline__ void umma_epilogue(unsigned tmem, const ConvIn& in, const ConvOut& out, int x0, int y0,
                                              int z0, int co0) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, m = warp * 32 + lane;
  unsigned r[CO_T];
#pragma unroll
  for (int j = 0; j < CO_T / 16; ++j) tmem_ld16(tmem + ((unsigned)(warp * 32) << 16) + 16 * j, r + 16 * j);
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int q = 0; q < CO_T; ++q) asm volatile("" : "+r"(r[q]));  // uses stay after the wait
  const size_t vox = ((size_t)z0 * in.H + (y0 + (m >> 3))) * in.W + (x0 + (m & 7));
  const int Co = out.Co;
#pragma unroll
  for (int c8 = 0; c8 < CO_T / 8; ++c8) {
    float v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      float t = __uint_as_float(r[c8 * 8 + q]);
      if (out.bias) t += out.bias[co0 + c8 * 8 + q];
      if (out.relu) t = t > 0.f ? t : out.slope * t;
      v[q] = t;
    }
    const size_t at = vox * Co + co0 + c8 * 8;
    if (out.mask) {
      const uint4 mk = *reinterpret_cast<const uint4*>(out.mask + at);
      const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&mk);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        if (!(__low2float(h[q]) > 0.f)) v[2 * q] *= out.mask_slope;
        if (!(__high2float(h[q]) > 0.f)) v[2 * q + 1] *= out.mask_slope;
      }
    }
    if (out.yf) {
      float4* d = reinterpret_cast<float4*>(out.yf + at);
      d[0] = make_float4(v[0], v[1], v[2], v[3]);
      d[1] = make_float4(v[4], v[5], v[6], v[7]);
    } else {
      __align__(16) __nv_bfloat162 h[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) h[q] = __floats2bfloat162_rn(v[2 * q], v[2 * q + 1]);
      *reinterpret_cast<uint4*>(out.y + at) = *reinterpret_cast<const uint4*>(h);
    }
  }
}

template <int CO_T>
__global__ void __launch_bounds__(128) k_conv3_umma(const ConvIn in, const __nv_bfloat16* __restrict__ wt,
                                                    const ConvOut out, int ncog, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  constexpr int kPB = 27 * CO_T * 16;  // bytes of one 8-channel plane of one slice's weights
  constexpr int kCols = CO_T <= 32 ? 32 : 64;
  const int Ci = in.C1 + in.C2, nsl = Ci / 16, Co = out.Co;
  const unsigned s_w = su32(smem);
  const unsigned s_x = s_w + nsl * 2 * kPB;  // kBufs halo buffers
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + nsl * 2 * kPB + kBufs * kHaloBytes);
  unsigned* tslot = reinterpret_cast<unsigned*>(bars + kBufs);
  const int nxt = in.W / kTX, nyt = in.H / kTY, ntiles = nxt * nyt * in.D;
  const int co0 = (blockIdx.x % ncog) * CO_T;
  const int t0 = blockIdx.x / ncog, tstride = gridDim.x / ncog;
  if (t0 >= ntiles) return;  // whole CTA, before any barrier
  const int nst = ((ntiles - t0 + tstride - 1) / tstride) * nsl;
  const int tid = threadIdx.x, warp = tid >> 5;
  auto origin = [&](int st, int& x0, int& y0, int& z0) {
    int t = t0 + (st / nsl) * tstride;
    x0 = (t % nxt) * kTX;
    t /= nxt;
    y0 = (t % nyt) * kTY;
    z0 = t / nyt;
  };
  // weights of this channel group: slice sl, plane c, row tap * CO_T + co
  for (int i = tid; i < 27 * CO_T * nsl; i += blockDim.x) {
    const int sl = i / (27 * CO_T), r = i % (27 * CO_T), tap = r / CO_T, co = r % CO_T;
    const __nv_bfloat16* src = wt + ((size_t)tap * Co + co0 + co) * Ci + sl * 16;
    const unsigned dst = s_w + sl * 2 * kPB + r * 16;
    cp_async16(dst, src, 16);
    cp_async16(dst + kPB, src + 8, 16);
  }
  {
    int x0, y0, z0;
    origin(0, x0, y0, z0);
    issue_halo_planar(s_x, in, x0, y0, z0, 0);
  }
  asm volatile("cp.async.commit_group;\n" ::);
  if (tid == 0) {
    for (int b = 0; b < kBufs; ++b) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&bars[b])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::);
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tslot)), "n"(kCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::);
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::);
  const unsigned tmem = *tslot;
  bool failed = false;
  for (int st = 0; st < nst; ++st) {
    // stage s uses buffer s % kBufs and commits its MMAs to that buffer's
    // barrier (phase s / kBufs); the buffer refilled below was last read by
    // stage st + 1 - kBufs, whose MMAs have had a whole stage to finish
    if (st + 1 >= kBufs && st + 1 < nst) {
      const int old = st + 1 - kBufs;
      const bool got = mbar_wait(su32(&bars[old % kBufs]), (old / kBufs) & 1);
      if (!__syncthreads_and(got)) {
        failed = true;
        break;
      }
    }
    if (st + 1 < nst) {
      int x0, y0, z0;
      origin(st + 1, x0, y0, z0);
      issue_halo_planar(s_x + ((st + 1) % kBufs) * kHaloBytes, in, x0, y0, z0, ((st + 1) % nsl) * 16);
    }
    asm volatile("cp.async.commit_group;\n" ::);
    asm volatile("cp.async.wait_group 1;\n" ::);
    asm volatile("fence.proxy.async.shared::cta;" ::);
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::);
    const int sl = st % nsl;
    if (tid == 0) {
      const unsigned xb = s_x + (st % kBufs) * kHaloBytes, wb = s_w + sl * 2 * kPB;
      for (int tap = 0; tap < 27; ++tap) {
        const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;
        const uint64_t ad = smem_desc(xb + ((dz * kHY + dy) * kHX + dx) * 16, kPlane, kHX * 16);
        const uint64_t bd = smem_desc(wb + tap * CO_T * 16, kPB, 128);
        const unsigned accumulate = (sl > 0 || tap > 0) ? 1u : 0u;
        asm volatile(
            "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc_bf16(CO_T)), "r"(accumulate));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          su32(&bars[st % kBufs])));
    }
    if (sl == nsl - 1) {
      const bool got = mbar_wait(su32(&bars[st % kBufs]), (st / kBufs) & 1);
      if (!__syncthreads_and(got)) {
        failed = true;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::);
      int x0, y0, z0;
      origin(st, x0, y0, z0);
      umma_epilogue<CO_T>(tmem, in, out, x0, y0, z0, co0);
      asm volatile("tcgen05.fence::before_thread_sync;" ::);
    }
    __syncthreads();
  }
  asm volatile("cp.async.wait_all;\n" ::);
  if (failed && tid == 0) atomicOr(err, DF_TIMEOUT);
  asm volatile("tcgen05.fence::before_thread_sync;" ::);
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(kCols));
}

template <int CO_T>
vg_status launch_umma(Ctx* c, const ConvIn& in, const __nv_bfloat16* wt, const ConvOut& out) {
  const int Ci = in.C1 + in.C2, ncog = out.Co / CO_T;
  const size_t smem = (size_t)(Ci / 16) * 2 * 27 * CO_T * 16 + kBufs * kHaloBytes + 64;
  VG_CUDA(c, cudaFuncSetAttribute(k_conv3_umma<CO_T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  VG_CUDA(c, cudaFuncSetAttribute(k_conv3_umma<CO_T>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  // CTAs per SM: shared memory (228 KB per SM, 1 KB reserved per CTA) and the
  // 512 tensor-memory columns bound it; extra CTAs would only queue
  constexpr int kCols = CO_T <= 32 ? 32 : 64;
  const int per_sm = std::max(1, std::min<int>(std::min<int>((228 * 1024) / (int)(smem + 1024), 512 / kCols), 8));
  const long items = (long)(in.W / kTX) * (in.H / kTY) * in.D * ncog;
  long grid = std::min<long>(items, (long)std::max(per_sm, 1) * sm_count());
  grid = std::max<long>(ncog, grid / ncog * ncog);
  k_conv3_umma<CO_T><<<(unsigned)grid, 128, smem, c->stream>>>(in, wt, out, ncog, c->dflag);
  VG_LAUNCHED(c);
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

}  // namespace

bool conv3_umma_fits(const ConvIn& in, int Co) {
  return in.W % kTX == 0 && in.H % kTY == 0 && Co % 16 == 0 && (in.C1 + in.C2) % 16 == 0;
}

vg_status conv3_fwd_umma(Ctx* c, const ConvIn& in, const __nv_bfloat16* wt, const ConvOut& out, bool* handled) {
  *handled = false;
  if (!conv3_umma_fits(in, out.Co) || !c->dflag) return VG_OK;
  const size_t Ci = (size_t)(in.C1 + in.C2);
  const int cands[4] = {out.Co == 48 ? 48 : 64, 32, 16, 0};
  for (int k = 0; cands[k]; ++k) {
    const int co_t = cands[k];
    if (out.Co % co_t || 27 * (size_t)co_t * Ci * 2 > kUmmaWeightBytes) continue;
    *handled = true;
    switch (co_t) {
      case 64: return launch_umma<64>(c, in, wt, out);
      case 48: return launch_umma<48>(c, in, wt, out);
      case 32: return launch_umma<32>(c, in, wt, out);
      default: return launch_umma<16>(c, in, wt, out);
    }
  }
  return VG_OK;
}

}  // namespace nn
}  // namespace vg
