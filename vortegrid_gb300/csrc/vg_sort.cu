// K2: leaf binning and the stable cell sort behind the influence tree, the
// splat and PSE neighbour lists.
//
// Replaces Particles::PartitionParticles (Particles/particle.cpp:398-437),
// which appends each vorton index to the list of the cell
// UniformGridGeometry::OffsetOfPosition names (uniformGrid.h:536-574,
// 645-651), in vorton-index order.  Here:
//   1. k_bin: one thread per vorton computes the leaf offset with the
//      reference's FP32 binning (bit-exact) and counts vortons per cell;
//   2. an exclusive scan of the counts gives each cell's first slot;
//   3. a stable LSD radix sort of (offset, index) pairs by offset (digits
//      of up to 11 bits, as few passes as the cell count needs) produces each cell's
//      vorton indices in ascending order -- the order in which the
//      reference accumulates them -- independent of thread timing.
#include "vg_internal.cuh"

namespace vg {

namespace {

constexpr int kScanBlock = 1024;

__global__ void k_bin(Geom g, const float4* __restrict__ pos, int n, unsigned* __restrict__ key,
                      unsigned* __restrict__ val, unsigned* __restrict__ count, unsigned ncells) {
  pdl_entry();
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p = pos[i];
  const unsigned ix = bin_axis(p.x, g.mn[0], g.cpe[0]);
  const unsigned iy = bin_axis(p.y, g.mn[1], g.cpe[1]);
  const unsigned iz = bin_axis(p.z, g.mn[2], g.cpe[2]);
  unsigned off = ix + g.np[0] * (iy + g.np[1] * iz);
  // Vortons outside the grid's points (undefined behaviour in the reference;
  // negative cells wrap to large values), and non-finite ones, go to an extra
  // slot, ncells, that no consumer of the lists reads: they drop out of the
  // splat, the tree and PSE.
  if (ix >= g.np[0] || iy >= g.np[1] || iz >= g.np[2] || off >= ncells || !(p.x == p.x && p.y == p.y && p.z == p.z))
    off = ncells;
  key[i] = off;
  val[i] = (unsigned)i;
  atomicAdd(&count[off], 1u);
}

// Block-wide exclusive scan of kScanBlock values (one per thread).
__device__ unsigned block_exclusive_scan(unsigned v, unsigned* total) {
  __shared__ unsigned warp_sums[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[wid] = x;
  __syncthreads();
  if (wid == 0) {
    unsigned s = (lane < (int)(blockDim.x >> 5)) ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      unsigned y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    warp_sums[lane] = s;
  }
  __syncthreads();
  const unsigned before = (wid > 0 ? warp_sums[wid - 1] : 0) + x - v;
  if (total) *total = warp_sums[(blockDim.x >> 5) - 1];
  __syncthreads();
  return before;
}

__global__ void __launch_bounds__(kScanBlock) k_scan_blocks(const unsigned* __restrict__ in, size_t n,
                                                            unsigned* __restrict__ out,
                                                            unsigned* __restrict__ block_sums) {
  pdl_entry();
  const size_t i = (size_t)blockIdx.x * kScanBlock + threadIdx.x;
  const unsigned v = i < n ? in[i] : 0;
  unsigned total;
  const unsigned e = block_exclusive_scan(v, &total);
  if (i < n) out[i] = e;
  if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

// Single-block scan of the block sums (any count), in place.
__global__ void __launch_bounds__(kScanBlock) k_scan_sums(unsigned* __restrict__ sums, size_t nb,
                                                          unsigned* __restrict__ grand_total) {
  pdl_entry();
  __shared__ unsigned carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (size_t base = 0; base < nb; base += kScanBlock) {
    const size_t i = base + threadIdx.x;
    const unsigned v = i < nb ? sums[i] : 0;
    unsigned total;
    const unsigned e = block_exclusive_scan(v, &total);
    if (i < nb) sums[i] = e + carry;
    __syncthreads();
    if (threadIdx.x == 0) carry += total;
    __syncthreads();
  }
  if (threadIdx.x == 0 && grand_total) *grand_total = carry;
}

__global__ void k_scan_add(unsigned* __restrict__ out, size_t n, const unsigned* __restrict__ sums) {
  pdl_entry();
  const size_t i = (size_t)blockIdx.x * kScanBlock + threadIdx.x;
  if (i < n) out[i] += sums[blockIdx.x];
}

// ---- stable LSD radix sort, digits of up to 11 bits ----------------------------
constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;  // keys per thread per tile
constexpr int kTileKeys = kSortThreads * kSortItems;
constexpr int kMaxDigitBits = 11;  // as few passes as the cell count needs (2 up to 2^22 cells)

__global__ void __launch_bounds__(kSortThreads) k_digit_hist(const unsigned* __restrict__ key, int n, int shift,
                                                             unsigned mask, int ntiles, unsigned* __restrict__ hist) {
  pdl_entry();
  __shared__ unsigned h[1u << kMaxDigitBits];
  for (unsigned d = threadIdx.x; d <= mask; d += kSortThreads) h[d] = 0;
  __syncthreads();
  const int base = blockIdx.x * kTileKeys;
  for (int k = 0; k < kSortItems; ++k) {
    const int i = base + k * kSortThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(key[i] >> shift) & mask], 1u);
  }
  __syncthreads();
  for (unsigned d = threadIdx.x; d <= mask; d += kSortThreads) hist[(size_t)d * ntiles + blockIdx.x] = h[d];  // digit-major
}

// Scatter one tile: keys are taken in rounds of kSortThreads consecutive
// elements; within a round, a key's rank among equal digits comes from warp
// match masks and per-warp digit counts, so the output is stable.  Only the
// digits present in a round are touched: each (warp, digit) leader posts its
// count, and after the round adds it to the digit's running slot and clears
// its post.  Dynamic shared memory: (1 + warps) x (mask + 1) counters.
__global__ void __launch_bounds__(kSortThreads) k_digit_scatter(const unsigned* __restrict__ key_in,
                                                                const unsigned* __restrict__ val_in, int n, int shift,
                                                                unsigned mask, int ntiles,
                                                                const unsigned* __restrict__ offsets,
                                                                unsigned* __restrict__ key_out,
                                                                unsigned* __restrict__ val_out) {
  pdl_entry();
  constexpr int kWarps = kSortThreads / 32;
  extern __shared__ unsigned sort_smem[];
  const unsigned nd = mask + 1;
  unsigned* running = sort_smem;     // [digit]
  unsigned* warp_cnt = running + nd;  // [warp][digit]
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (unsigned d = threadIdx.x; d < nd; d += kSortThreads) running[d] = offsets[(size_t)d * ntiles + blockIdx.x];
  for (unsigned d = threadIdx.x; d < kWarps * nd; d += kSortThreads) warp_cnt[d] = 0;
  __syncthreads();
  const int base = blockIdx.x * kTileKeys;
  for (int k = 0; k < kSortItems; ++k) {
    const int i = base + k * kSortThreads + threadIdx.x;
    const bool valid = i < n;
    const unsigned kv = valid ? key_in[i] : 0u;
    const unsigned digit = valid ? ((kv >> shift) & mask) : nd;
    const unsigned peers = __match_any_sync(0xffffffffu, digit);
    const unsigned lower = __popc(peers & ((1u << lane) - 1u));
    const bool leader = valid && lower == 0;
    if (leader) warp_cnt[wid * nd + digit] = __popc(peers);
    __syncthreads();
    if (valid) {
      unsigned before = 0;
      for (int ww = 0; ww < wid; ++ww) before += warp_cnt[ww * nd + digit];
      const unsigned dst = running[digit] + before + lower;
      key_out[dst] = kv;
      val_out[dst] = val_in[i];
    }
    __syncthreads();
    if (leader) {
      atomicAdd(&running[digit], (unsigned)__popc(peers));
      warp_cnt[wid * nd + digit] = 0;
    }
    __syncthreads();
  }
}

}  // namespace

// Exclusive scan of n values; out[n] receives the total when out has n+1 slots.
vg_status exclusive_scan(Ctx* c, const unsigned* in, size_t n, unsigned* out, bool write_total) {
  const size_t nb = (n + kScanBlock - 1) / kScanBlock;
  vg_status st = VG_OK;
  unsigned* sums = (unsigned*)ws(c, S_SCAN, (nb + 1) * sizeof(unsigned), &st);
  if (st != VG_OK) return st;
  pdl_launch(c->stream, (unsigned)nb, kScanBlock, 0, k_scan_blocks, in, n, out, sums);
  pdl_launch(c->stream, 1, kScanBlock, 0, k_scan_sums, sums, nb, write_total ? out + n : nullptr);
  pdl_launch(c->stream, (unsigned)nb, kScanBlock, 0, k_scan_add, out, n, sums);
  c->launches += 3;
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

vg_status build_cell_lists(Ctx* c, const Geom& g, const float4* ps, size_t n, CellLists* out) {
  const size_t ncells = g.points();
  if (n > 0x7fffffff || ncells >= 0xffffffffu) return fail(c, VG_TOO_LARGE, "cell lists: too many vortons or cells");
  vg_status st = VG_OK;
  // one slot per grid point and one for vortons outside the grid
  const size_t slots = ncells + 1;
  // S_CELL: key, val, key2, val2 (4 n); S_COUNT: count (slots); S_START: start (slots+1)
  unsigned* kv = (unsigned*)ws(c, S_CELL, 4 * (n + 1) * sizeof(unsigned), &st);
  if (st != VG_OK) return st;
  unsigned* count = (unsigned*)ws(c, S_COUNT, slots * sizeof(unsigned), &st);
  if (st != VG_OK) return st;
  unsigned* start = (unsigned*)ws(c, S_START, (slots + 1) * sizeof(unsigned), &st);
  if (st != VG_OK) return st;
  unsigned *key = kv, *val = kv + (n + 1), *key2 = kv + 2 * (n + 1), *val2 = kv + 3 * (n + 1);
  VG_CUDA(c, cudaMemsetAsync(count, 0, slots * sizeof(unsigned), c->stream));
  if (n > 0) {
    pdl_launch(c->stream, blocks_for(n, 256), 256, 0, k_bin, g, ps, (int)n, key, val, count, (unsigned)ncells);
    VG_LAUNCHED(c);
  }
  st = exclusive_scan(c, count, slots, start, true);
  if (st != VG_OK) return st;
  // Stable radix sort by key: as few passes of at most kMaxDigitBits-bit
  // digits as the largest key (ncells) needs, the bits split evenly.
  int bits = 0;
  while (bits < 32 && ncells >> bits) ++bits;
  const int passes = (bits + kMaxDigitBits - 1) / kMaxDigitBits;
  const int dbits = passes > 0 ? (bits + passes - 1) / passes : 0;
  const unsigned mask = (1u << dbits) - 1u, nd = mask + 1;
  const int ntiles = (int)((n + kTileKeys - 1) / kTileKeys);
  if (n > 0 && passes > 0) {
    unsigned* hist = (unsigned*)ws(c, S_FILL, (size_t)nd * ntiles * sizeof(unsigned) * 2 + 16, &st);
    if (st != VG_OK) return st;
    unsigned* offs = hist + (size_t)nd * ntiles;
    const size_t scatter_smem = (size_t)(1 + kSortThreads / 32) * nd * sizeof(unsigned);
    // kernel attributes are per device: set once for each device used
    static unsigned long long smem_set = 0;
    const unsigned long long dev_bit = 1ull << (c->cfg.device & 63);
    if (!(smem_set & dev_bit)) {
      cudaFuncSetAttribute(k_digit_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)((1 + kSortThreads / 32) * (1u << kMaxDigitBits) * sizeof(unsigned)));
      smem_set |= dev_bit;
    }
    for (int p = 0; p < passes; ++p) {
      pdl_launch(c->stream, ntiles, kSortThreads, 0, k_digit_hist, key, (int)n, dbits * p, mask, ntiles, hist);
      VG_LAUNCHED(c);
      st = exclusive_scan(c, hist, (size_t)nd * ntiles, offs, false);
      if (st != VG_OK) return st;
      pdl_launch(c->stream, ntiles, kSortThreads, scatter_smem, k_digit_scatter, key, val, (int)n, dbits * p, mask,
                 ntiles, offs, key2, val2);
      VG_LAUNCHED(c);
      unsigned* t = key; key = key2; key2 = t;
      t = val; val = val2; val2 = t;
    }
  }
  VG_CUDA(c, cudaGetLastError());
  out->cell = nullptr;
  out->start = start;
  out->items = val;
  // per-vorton cell keys in vorton order are not kept after sorting; the
  // sorted keys are: `key` (same order as items).
  out->cell = key;
  return VG_OK;
}

}  // namespace vg
