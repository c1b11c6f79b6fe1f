// si_sort.cu — the block sort of mpm.js:563-577/614-621 for one tick of many scenes.
//
// The reference counts keys with global atomics, so the order inside a block depends on atomic
// timing. Here the particles of every sorting scene are concatenated with key = bin_base + block key
// and sorted by a stable LSD radix sort (8-bit digits; per pass: tile histograms, a scan per digit,
// a stable scatter ranked with warp match + shared-memory prefixes). It is deterministic, has no
// waits between CTAs, and yields the reference's counts and starts exactly; each scene's particles
// stay inside its own segment because the bin ranges are ordered like the segments.
#include <algorithm>

#include "si_device.h"

namespace si {

// CTA barrier that lanes of one warp may reach along different paths (after an `if` on the lane's
// own particle or a tail loop). __syncthreads() is the warp-aligned barrier (barrier.sync.aligned),
// undefined when a warp's lanes arrive at different instructions; the non-aligned form counts each
// arriving thread, so every thread of the CTA has passed the preceding phase when it completes.
__device__ __forceinline__ void cta_sync() { asm volatile("barrier.sync 0;" ::: "memory"); }

__device__ __forceinline__ int find_scene_p2(const TickScene* ts, int n, uint32_t chunk) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (ts[mid].pchunk_begin <= chunk) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// concatenated (key, local index) of the sorting scenes
__global__ void __launch_bounds__(kCtaThreads) k_sort_init(TickInfo t, uint32_t* keys, uint32_t* vals) {
  for (uint32_t chunk = blockIdx.x; chunk < t.pchunks; chunk += gridDim.x) {
    const TickScene& ts = t.ts[find_scene_p2(t.ts, t.nscenes, chunk)];
    if (!(ts.flags & F_GATHER)) continue;
    const int first = (int)(chunk - ts.pchunk_begin) * t.chunk;
    const int last = min(first + t.chunk, ts.n);
    for (int i = first + threadIdx.x; i < last; i += blockDim.x) {
      keys[ts.seg_base + i] = ts.bin_base + ts.keys[i];
      vals[ts.seg_base + i] = (uint32_t)i;
    }
  }
}

constexpr int kItems = kSortTile / kCtaThreads;   // 16
constexpr int kWarps = kCtaThreads / 32;          // 8

__global__ void __launch_bounds__(kCtaThreads) k_radix_hist(const uint32_t* __restrict__ keys, uint32_t n, int shift,
                                                           uint32_t* hist, uint32_t tiles) {
  __shared__ uint32_t h[256];
  for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    h[threadIdx.x] = 0;
    cta_sync();
    const uint32_t base = tile * kSortTile;
#pragma unroll
    for (int r = 0; r < kItems; r++) {
      uint32_t e = base + r * kCtaThreads + threadIdx.x;
      if (e < n) atomicAdd(&h[(__ldg(&keys[e]) >> shift) & 255u], 1u);
    }
    cta_sync();
    hist[threadIdx.x * tiles + tile] = h[threadIdx.x];
    cta_sync();
  }
}

// one CTA per digit: exclusive scan over the tiles in place, digit total out
__global__ void __launch_bounds__(kCtaThreads) k_radix_scan(uint32_t* hist, uint32_t tiles, uint32_t* digit_total) {
  __shared__ uint32_t warp_sum[kWarps];
  __shared__ uint32_t carry;
  uint32_t* row = hist + (size_t)blockIdx.x * tiles;
  if (threadIdx.x == 0) carry = 0;
  cta_sync();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (uint32_t b = 0; b < tiles; b += kCtaThreads) {
    uint32_t i = b + threadIdx.x;
    uint32_t v = i < tiles ? row[i] : 0u;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_sum[warp] = x;
    cta_sync();
    uint32_t wpre = 0, total = 0;
    for (int w = 0; w < kWarps; w++) { uint32_t s = warp_sum[w]; if (w < warp) wpre += s; total += s; }
    uint32_t c = carry;
    if (i < tiles) row[i] = c + wpre + x - v;
    cta_sync();
    if (threadIdx.x == 0) carry = c + total;
    cta_sync();
  }
  if (threadIdx.x == 0) digit_total[blockIdx.x] = carry;
}

__global__ void __launch_bounds__(kCtaThreads) k_radix_scatter(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                                                              uint32_t* kout, uint32_t* vout, uint32_t n, int shift,
                                                              const uint32_t* __restrict__ hist, const uint32_t* __restrict__ digit_total,
                                                              uint32_t tiles) {
  __shared__ uint32_t dbase[256];
  __shared__ uint32_t wcount[kWarps][256];
  __shared__ uint32_t wpre[kWarps][256];
  __shared__ uint32_t run[256];
  __shared__ uint32_t wsum[kWarps];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // exclusive scan of the digit totals (same in every CTA)
  {
    uint32_t v = digit_total[tid], x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    cta_sync();
    uint32_t pre = 0;
    for (int w = 0; w < warp; w++) pre += wsum[w];
    dbase[tid] = pre + x - v;
  }
  for (int w = 0; w < kWarps; w++) wcount[w][tid] = 0;
  cta_sync();
  const unsigned lt_mask = (1u << lane) - 1u;
  for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    run[tid] = dbase[tid] + hist[tid * tiles + tile];
    cta_sync();
    const uint32_t base = tile * kSortTile;
    for (int r = 0; r < kItems; r++) {
      const uint32_t e = base + r * kCtaThreads + tid;
      const bool ok = e < n;
      uint32_t key = 0, val = 0, d = 256;
      if (ok) { key = kin[e]; val = vin[e]; d = (key >> shift) & 255u; }
      const unsigned peers = __match_any_sync(0xffffffffu, d);
      const unsigned rank = __popc(peers & lt_mask);
      if (ok && rank == 0) wcount[warp][d] = __popc(peers);
      cta_sync();
      {
        uint32_t acc = run[tid];
#pragma unroll
        for (int w = 0; w < kWarps; w++) {
          uint32_t c = wcount[w][tid];
          wpre[w][tid] = acc;
          acc += c;
          wcount[w][tid] = 0;
        }
        run[tid] = acc;
      }
      cta_sync();
      if (ok) {
        const uint32_t pos = wpre[warp][d] + rank;
        kout[pos] = key;
        vout[pos] = val;
      }
      cta_sync();
    }
  }
}

// starts of every bin of every sorting scene: lower_bound in the sorted keys of its segment
__global__ void k_scene_starts(TickInfo t, const uint32_t* __restrict__ skeys) {
  const TickScene& ts = t.ts[blockIdx.y];
  if (!(ts.flags & F_GATHER)) return;
  uint32_t* starts = ts.starts;
  const uint32_t nb = ts.prm->num_blocks;
  const uint32_t* seg = skeys + ts.seg_base;
  const uint32_t n = (uint32_t)ts.n;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k <= nb; k += gridDim.x * blockDim.x) {
    const uint32_t target = ts.bin_base + k;
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
      uint32_t mid = (lo + hi) >> 1;
      if (__ldg(&seg[mid]) < target) lo = mid + 1; else hi = mid;
    }
    starts[k] = lo;
  }
}

void launch_sort(const TickInfo& t, const SortInfo& s, const uint32_t** perm_out, const uint32_t** keys_out,
                 int grid_ctas, cudaStream_t st) {
  *perm_out = s.vals_a;
  *keys_out = s.keys_a;
  if (s.n == 0) return;
  {
    int ctas = (int)std::min<uint32_t>(t.pchunks, (uint32_t)grid_ctas);
    k_sort_init<<<ctas, kCtaThreads, 0, st>>>(t, s.keys_a, s.vals_a);
  }
  const uint32_t tiles = (s.n + kSortTile - 1) / kSortTile;
  uint32_t *ka = s.keys_a, *va = s.vals_a, *kb = s.keys_b, *vb = s.vals_b;
  for (int p = 0; p < s.passes; p++) {
    const int shift = p * kRadixBits;
    int ctas = (int)std::min<uint32_t>(tiles, (uint32_t)grid_ctas);
    k_radix_hist<<<ctas, kCtaThreads, 0, st>>>(ka, s.n, shift, s.hist, tiles);
    k_radix_scan<<<256, kCtaThreads, 0, st>>>(s.hist, tiles, s.digit_total);
    k_radix_scatter<<<ctas, kCtaThreads, 0, st>>>(ka, va, kb, vb, s.n, shift, s.hist, s.digit_total, tiles);
    uint32_t* tk = ka; ka = kb; kb = tk;
    uint32_t* tv = va; va = vb; vb = tv;
  }
  *perm_out = va;
  *keys_out = ka;
}

void launch_scene_starts_all(const TickInfo& t, const uint32_t* sorted_keys, uint32_t max_blocks, cudaStream_t st) {
  if (t.nscenes == 0) return;
  dim3 grid((unsigned)std::min<uint32_t>((max_blocks + 1 + 255) / 256, 1024u), (unsigned)t.nscenes);
  k_scene_starts<<<grid, 256, 0, st>>>(t, sorted_keys);
}

}  // namespace si
