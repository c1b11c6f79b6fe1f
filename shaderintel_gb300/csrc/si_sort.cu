// si_sort.cu — the block sort of mpm.js:563-577/614-621 for one tick of many scenes.
//
// The reference counts keys with global atomics, so the order inside a block depends on atomic
// timing. Here the particles are sorted by a stable LSD radix sort (8-bit digits; per pass: tile
// histograms, a scan per digit, a stable scatter in which each warp ranks a contiguous segment of its
// tile with warp match and per-warp digit counters). One sorting scene is sorted from its own keys;
// the sorting scenes of a tick of several are concatenated into tile-aligned segments, each padded
// with a sentinel key and sorted within its own tiles (a segmented scan of the tile histograms), so
// the passes cover the largest scene's keys. It is deterministic, has no waits between CTAs, and
// yields the reference's counts and starts exactly.
#include <algorithm>
#include <mutex>

#include "si_cuda.h"
#include "si_device.h"
#include "si_math.cuh"
#include "si_region.cuh"


namespace si {

// CTA barrier that lanes of one warp may reach along different paths (after an `if` on the lane's
// own particle or a tail loop). __syncthreads() is the warp-aligned barrier (barrier.sync.aligned),
// undefined when a warp's lanes arrive at different instructions; the non-aligned form counts each
// arriving thread, so every thread of the CTA has passed the preceding phase when it completes.
__device__ __forceinline__ void cta_sync() { asm volatile("barrier.sync 0;" ::: "memory"); }

constexpr int kItems = kSortTile / kCtaThreads;   // 16
constexpr int kWarps = kCtaThreads / 32;          // 8

// Concatenated (key, local index) of the sorting scenes, each scene's segment starting on a tile
// boundary (seg_base) and padded to whole tiles with the sentinel key; tile_scene[tile] names the
// scene of every tile. A CTA fills whole tiles: the tile's scene is the last scene whose seg_base is
// at most the tile's first slot (scenes that do not sort sit at the running end with no slots), found
// in shared memory, so the tick table is read once per 4096 slots. A scene without key buffers
// (F_KEYS_FROM_X) has its block keys computed here from its current positions, as k_keys would. The
// tile histogram of the first pass (digit 0, as k_radix_hist counts it) is taken on the way, so that
// pass does not read the keys back.
__global__ void __launch_bounds__(kCtaThreads) k_sort_init(TickInfo t, uint32_t* keys, uint32_t* vals,
                                                           uint32_t* tile_scene, uint32_t sentinel, uint32_t tiles,
                                                           uint32_t* hist) {
  __shared__ uint32_t scene_tab[kSceneTable];
  __shared__ uint32_t h[256];
  scene_table_load<kSceneSeg>(t, scene_tab);
  const unsigned lane = threadIdx.x & 31u;
  for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    h[threadIdx.x] = 0;
    cta_sync();
    const uint32_t slot0 = tile * kSortTile;
    const int scene = scene_of<kSceneSeg>(t, scene_tab, slot0);
    const TickScene& ts = t.ts[scene];
    if (threadIdx.x == 0) tile_scene[tile] = (uint32_t)scene;
    const int n = ts.n;
    const int first = (int)(slot0 - ts.seg_base);
    const bool from_x = (ts.flags & F_KEYS_FROM_X) != 0;
    const uint32_t nb = from_x ? ts.prm->num_blocks : 0u;
    // stored keys: all sixteen loaded before the counting (positions are read round by round)
    uint32_t kk[kItems];
    if (!from_x) {
#pragma unroll
      for (int r = 0; r < kItems; r++) {
        const int i = first + r * kCtaThreads + (int)threadIdx.x;
        kk[r] = i < n ? __ldg(&ts.keys[i]) : sentinel;
      }
    }
#pragma unroll
    for (int r = 0; r < kItems; r++) {
      const int i = first + r * kCtaThreads + (int)threadIdx.x;
      uint32_t k = from_x ? sentinel : kk[r];
      if (from_x) {
        if (i < n) {
          const float4 x = ts.P[i];
          k = block_key(x.x, x.y, x.z, nb);
        }
      }
      keys[ts.seg_base + i] = k;
      vals[ts.seg_base + i] = (uint32_t)i;
      // one add per distinct digit of the warp, as in k_radix_hist
      const uint32_t d = k & 255u;
      const unsigned peers = __match_any_sync(0xffffffffu, d);
      if (lane == (unsigned)(__ffs(peers) - 1)) atomicAdd(&h[d], (uint32_t)__popc(peers));
    }
    cta_sync();
    hist[threadIdx.x * tiles + tile] = h[threadIdx.x];
    cta_sync();
  }
}


__global__ void __launch_bounds__(kCtaThreads) k_radix_hist(const uint32_t* __restrict__ keys, uint32_t n, int shift,
                                                           uint32_t* hist, uint32_t tiles) {
  __shared__ uint32_t h[256];
  const unsigned lane = threadIdx.x & 31u;
  // a thread's digits of one tile (256: past the end); the next tile's are loaded while this one's
  // are counted
  auto digits = [&](uint32_t tile, uint32_t (&d)[kItems]) {
#pragma unroll
    for (int r = 0; r < kItems; r++) {
      const uint32_t e = tile * kSortTile + r * kCtaThreads + threadIdx.x;
      d[r] = tile < tiles && e < n ? (__ldg(&keys[e]) >> shift) & 255u : 256u;
    }
  };
  uint32_t d[kItems];
  digits(blockIdx.x, d);
  for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    h[threadIdx.x] = 0;
    cta_sync();
    uint32_t dn[kItems];
    digits(tile + gridDim.x, dn);
    // the keys arrive nearly sorted, so most lanes of a warp share a digit: one add per distinct
    // digit of the warp (its lowest lane adds the group's size) instead of one per lane
#pragma unroll
    for (int r = 0; r < kItems; r++) {
      const unsigned peers = __match_any_sync(0xffffffffu, d[r]);
      if (d[r] < 256u && lane == (unsigned)(__ffs(peers) - 1)) atomicAdd(&h[d[r]], (uint32_t)__popc(peers));
    }
    cta_sync();
    hist[threadIdx.x * tiles + tile] = h[threadIdx.x];
    cta_sync();
#pragma unroll
    for (int r = 0; r < kItems; r++) d[r] = dn[r];
  }
}

// one CTA per digit: exclusive scan over the tiles in place, digit total out. A round covers
// kScanItems contiguous tiles a thread, summed in registers, and one block scan of the threads' sums.
constexpr int kScanItems = 8;
__global__ void __launch_bounds__(kCtaThreads) k_radix_scan(uint32_t* hist, uint32_t tiles, uint32_t* digit_total) {
  __shared__ uint32_t warp_sum[kWarps];
  __shared__ uint32_t carry;
  uint32_t* row = hist + (size_t)blockIdx.x * tiles;
  if (threadIdx.x == 0) carry = 0;
  cta_sync();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr uint32_t kRound = (uint32_t)kCtaThreads * kScanItems;
  for (uint32_t b = 0; b < tiles; b += kRound) {
    const uint32_t i0 = b + (uint32_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems], sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
      v[k] = i0 + k < tiles ? row[i0 + k] : 0u;
      sum += v[k];
    }
    uint32_t x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_sum[warp] = x;
    cta_sync();
    uint32_t wpre = 0, total = 0;
    for (int w = 0; w < kWarps; w++) { uint32_t s = warp_sum[w]; if (w < warp) wpre += s; total += s; }
    const uint32_t c = carry;
    uint32_t run = c + wpre + x - sum;   // the tiles before this thread's first
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
      if (i0 + k < tiles) row[i0 + k] = run;
      run += v[k];
    }
    cta_sync();
    if (threadIdx.x == 0) carry = c + total;
    cta_sync();
  }
  if (threadIdx.x == 0) digit_total[blockIdx.x] = carry;
}

// The segmented form of k_radix_scan: per digit, the exclusive prefix over the tiles of each scene
// (restarting where tile_scene changes), and each scene's digit total into seg_total[scene][digit].
// A round covers kScanItems tiles a thread, contiguous: each thread scans its own tiles in registers
// (all its loads in flight together), one segmented block scan combines the threads' last segments,
// and a carry takes the running segment into the next round.
__global__ void __launch_bounds__(kCtaThreads) k_radix_scan_seg(uint32_t* hist, uint32_t tiles,
                                                               const uint32_t* __restrict__ tile_scene,
                                                               uint32_t* seg_total) {
  __shared__ uint32_t warp_sum[kWarps];
  __shared__ uint32_t warp_head[kWarps];
  __shared__ uint32_t carry;
  const uint32_t d = blockIdx.x;
  uint32_t* row = hist + (size_t)d * tiles;
  if (threadIdx.x == 0) carry = 0;
  cta_sync();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr uint32_t kRound = (uint32_t)kCtaThreads * kScanItems;
  for (uint32_t b = 0; b < tiles; b += kRound) {
    const uint32_t i0 = b + (uint32_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems], sc[kScanItems];
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
      const uint32_t i = i0 + k;
      v[k] = i < tiles ? row[i] : 0u;
      sc[k] = i < tiles ? __ldg(&tile_scene[i]) : 0xffffffffu;
    }
    const uint32_t before = (i0 > 0 && i0 <= tiles) ? __ldg(&tile_scene[i0 - 1]) : 0xffffffffu;
    const uint32_t after = i0 + kScanItems < tiles ? __ldg(&tile_scene[i0 + kScanItems]) : 0xffffffffu;
    // the thread's own inclusive scan, restarting at each head (the first tile of a scene)
    uint32_t x[kScanItems], acc = 0;
    bool fl = false;   // a head among the thread's tiles so far
    int first_head = kScanItems;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
      const uint32_t i = i0 + k;
      const bool head = i < tiles && (i == 0 || sc[k] != (k ? sc[k - 1] : before));
      if (head) {
        acc = v[k];
        if (!fl) first_head = k;
        fl = true;
      } else {
        acc += v[k];
      }
      x[k] = acc;
    }
    // inclusive segmented scan of the threads' (last segment sum, has head) within the warp
    uint32_t xi = acc, fi = fl ? 1u : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, xi, o);
      const uint32_t g = __shfl_up_sync(0xffffffffu, fi, o);
      if (lane >= o && !fi) { xi += y; fi = g; }
    }
    if (lane == 31) { warp_sum[warp] = xi; warp_head[warp] = fi; }
    cta_sync();
    // what flows into the warp: the carry, then the earlier warps in order
    uint32_t p = carry;
    for (int w = 0; w < warp; w++) p = warp_head[w] ? warp_sum[w] : p + warp_sum[w];
    // what flows into this thread: the warp's inflow, then the earlier lanes of the warp
    const uint32_t e = __shfl_up_sync(0xffffffffu, xi, 1), ef = __shfl_up_sync(0xffffffffu, fi, 1);
    const uint32_t in = lane == 0 ? p : (ef ? e : p + e);
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
      const uint32_t i = i0 + k;
      if (i < tiles) {
        const uint32_t xk = k < first_head ? in + x[k] : x[k];
        row[i] = xk - v[k];
        const bool tail = i + 1 == tiles || sc[k] != (k + 1 < kScanItems ? sc[k + 1] : after);
        if (tail) seg_total[(size_t)sc[k] * 256 + d] = xk;
        x[k] = xk;
      }
    }
    cta_sync();   // every thread has read carry and the warp sums
    const uint32_t last = min(b + kRound, tiles) - 1;  // the round's last tile: its segment goes on
#pragma unroll
    for (int k = 0; k < kScanItems; k++)
      if (i0 + k == last) carry = x[k];
    cta_sync();
  }
}

// Stable scatter of one pass. Warp w of a tile owns the kSortTile / kWarps consecutive keys from
// tile * kSortTile + w * kSeg; it counts their digits (one add per distinct digit and round, by the
// group's lowest lane), a per-digit prefix over the warps turns the counts into each warp's first
// position, and a second walk over the same keys stores each at that position plus its rank among
// the earlier lanes of its round with the same digit. The rank order is (warp, round, lane), which is
// the keys' order in the tile, so equal digits keep their input order. vin == nullptr stands for the
// identity (the value of key e is e). SEG: the segmented sort, where a tile's digit bases are its
// scene's segment start plus the exclusive scan of that scene's digit totals.
// Four CTAs per SM (64 registers; the unsegmented form spills 20 B): the pass is latency-bound, and
// that occupancy made the mixed scene's sort phase 10 % faster than the compiler's 76-91 registers.
template <bool SEG>
__global__ void __launch_bounds__(kCtaThreads, 4) k_radix_scatter(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                                                              uint32_t* kout, uint32_t* vout, uint32_t n, int shift,
                                                              const uint32_t* __restrict__ hist, const uint32_t* __restrict__ digit_total,
                                                              uint32_t tiles, const uint32_t* __restrict__ tile_scene,
                                                              const uint32_t* __restrict__ seg_total, const TickScene* ts) {
  constexpr int kSeg = kSortTile / kWarps;   // 512 keys per warp, kItems rounds of 32
  static_assert(kSeg == kItems * 32, "a warp's segment is kItems rounds of 32 keys");
  __shared__ uint32_t dbase[256];
  __shared__ uint32_t woff[kWarps][256];
  __shared__ uint32_t wsum[kWarps];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // exclusive scan of the digit totals (same in every CTA)
  if (!SEG) {
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
  const unsigned lt_mask = (1u << lane) - 1u;
  for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    for (int w = 0; w < kWarps; w++) woff[w][tid] = 0;
    uint32_t sv = 0, sx = 0, sbase = 0;   // SEG: this digit's total in the tile's scene, its inclusive scan
    if (SEG) {
      const uint32_t scene = __ldg(&tile_scene[tile]);
      sbase = ts[scene].seg_base;
      sv = __ldg(&seg_total[(size_t)scene * 256 + tid]);
      sx = sv;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, sx, o);
        if (lane >= o) sx += y;
      }
      if (lane == 31) wsum[warp] = sx;
    }
    cta_sync();
    const uint32_t wbase = tile * kSortTile + (uint32_t)warp * kSeg;
    uint32_t key[kItems], val[kItems];
    // SEG: the warp's keys and values are all loaded before the counting (batched substep -0.2 %;
    // the unsegmented form spills more that way and loads them round by round)
    if (SEG) {
#pragma unroll
      for (int r = 0; r < kItems; r++) {
        const uint32_t e = wbase + r * 32 + lane;
        const bool ok = e < n;
        key[r] = ok ? kin[e] : 0u;
        val[r] = ok ? (vin ? vin[e] : e) : 0u;
      }
    }
    // 1. the warp's digit counts
#pragma unroll
    for (int r = 0; r < kItems; r++) {
      const uint32_t e = wbase + r * 32 + lane;
      const bool ok = e < n;
      if (!SEG) {
        key[r] = ok ? kin[e] : 0u;
        val[r] = ok ? (vin ? vin[e] : e) : 0u;
      }
      const uint32_t d = ok ? (key[r] >> shift) & 255u : 256u;
      const unsigned peers = __match_any_sync(0xffffffffu, d);
      if (ok && (peers & lt_mask) == 0u) woff[warp][d] += (uint32_t)__popc(peers);
      __syncwarp();
    }
    cta_sync();
    // 2. per digit: the first position of each warp's keys (tile base of the digit from the scan)
    {
      uint32_t db;
      if (SEG) {
        uint32_t pre = 0;
        for (int w = 0; w < warp; w++) pre += wsum[w];
        db = sbase + pre + sx - sv;
      } else {
        db = dbase[tid];
      }
      uint32_t acc = db + hist[tid * tiles + tile];
#pragma unroll
      for (int w = 0; w < kWarps; w++) {
        const uint32_t c = woff[w][tid];
        woff[w][tid] = acc;
        acc += c;
      }
    }
    cta_sync();
    // 3. ranks and stores, in the same order as the counts
#pragma unroll
    for (int r = 0; r < kItems; r++) {
      const uint32_t e = wbase + r * 32 + lane;
      const bool ok = e < n;
      const uint32_t d = ok ? (key[r] >> shift) & 255u : 256u;
      const unsigned peers = __match_any_sync(0xffffffffu, d);
      const uint32_t rank = (uint32_t)__popc(peers & lt_mask);
      const uint32_t at = ok ? woff[warp][d] : 0u;
      __syncwarp();
      if (ok) {
        kout[at + rank] = key[r];
        vout[at + rank] = val[r];
        if (rank == 0) woff[warp][d] = at + (uint32_t)__popc(peers);
      }
      __syncwarp();
    }
    cta_sync();   // woff is cleared for the next tile
  }
}

// starts of every bin of every sorting scene: lower_bound in the sorted keys of its segment. Every
// stride-th key (stride = ceil(n / kStartSamples)) is first loaded into shared memory by the whole CTA
// with independent loads; a bin's search narrows to one run of stride keys there and continues in
// global memory only inside that run (11 dependent global loads instead of 21 for 2.2 M keys).
constexpr uint32_t kStartSamples = 1024;
__global__ void __launch_bounds__(256) k_scene_starts(TickInfo t, const uint32_t* __restrict__ skeys) {
  __shared__ uint32_t smp[kStartSamples];
  const TickScene& ts = t.ts[blockIdx.y];
  if (!(ts.flags & F_GATHER)) return;
  const uint32_t nb = ts.prm->num_blocks;
  if (blockIdx.x * blockDim.x > nb) return;          // no bin of this scene for the CTA
  uint32_t* starts = ts.starts;
  const uint32_t* seg = skeys + ts.seg_base;
  const uint32_t n = (uint32_t)ts.n;
  const uint32_t stride = (n + kStartSamples - 1) / kStartSamples;   // 0 only when n == 0
  const uint32_t m = stride ? (n + stride - 1) / stride : 0;        // samples: seg[j * stride], j < m
  for (uint32_t j = threadIdx.x; j < m; j += blockDim.x) smp[j] = __ldg(&seg[j * stride]);
  __syncthreads();
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k <= nb; k += gridDim.x * blockDim.x) {
    const uint32_t target = ts.bin_base + k;
    uint32_t a = 0, b = m;                           // the first sample >= target (m: none)
    while (a < b) {
      const uint32_t mid = (a + b) >> 1;
      if (smp[mid] < target) a = mid + 1; else b = mid;
    }
    // seg[(a - 1) * stride] < target <= seg[a * stride]: the bound is in [(a - 1) * stride + 1, a * stride]
    uint32_t lo = a ? (a - 1) * stride + 1 : 0, hi = min(a * stride, n);
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (__ldg(&seg[mid]) < target) lo = mid + 1; else hi = mid;
    }
    starts[k] = lo;
  }
}

// The block binning of one small scene by one CTA in a single pass over all bins (at most 512 bins
// and 32768 keys, which fit in shared memory with 32 warps' counters). It ranks the keys as
// k_radix_scatter does, per warp over a contiguous segment, so the order is the stable one of the
// radix sort; the scan over the bins gives the scene's starts (scan.js:288-306) directly.
constexpr int kSmallThreads = 1024;
constexpr int kSmallWarps = kSmallThreads / 32;

__global__ void __launch_bounds__(kSmallThreads, 1) k_small_sort(const uint32_t* __restrict__ kin, uint32_t n,
                                                                 uint32_t bins, uint32_t* kout, uint32_t* vout,
                                                                 uint32_t* starts) {
  extern __shared__ uint32_t ss[];
  __shared__ uint32_t wsum[kSmallWarps];
  uint32_t* keys = ss;                                 // n keys
  const uint32_t row = bins + 1;                       // bin `bins`: lanes past the end (never counted)
  uint32_t* cnt = ss + n;                              // kSmallWarps x row counters
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (uint32_t i = tid; i < n; i += kSmallThreads) {
    const uint32_t k = kin[i];
    keys[i] = k < bins ? k : bins - 1;                 // block keys are < bins; kept in range regardless
  }
  for (uint32_t i = tid; i < (uint32_t)kSmallWarps * row; i += kSmallThreads) cnt[i] = 0;
  __syncthreads();
  const uint32_t seg = ((n + kSmallWarps - 1) / kSmallWarps + 31u) & ~31u;   // whole rounds of 32
  const uint32_t wb = (uint32_t)warp * seg, we = min(n, wb + seg);
  const unsigned lt_mask = (1u << lane) - 1u;
  uint32_t* wc = cnt + (uint32_t)warp * row;
  // 1. the warp's bin counts
  for (uint32_t base = wb; base < wb + seg; base += 32) {
    const uint32_t e = base + lane;
    const bool ok = e < we;
    const uint32_t d = ok ? keys[e] : bins;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    if (ok && (peers & lt_mask) == 0u) wc[d] += (uint32_t)__popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // 2. starts: exclusive scan of the bin totals (thread b: bin b); then each warp's first position
  uint32_t tot = 0;
  if ((uint32_t)tid < bins)
    for (int w = 0; w < kSmallWarps; w++) tot += cnt[(uint32_t)w * row + tid];
  uint32_t x = tot;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[warp] = x;
  __syncthreads();
  uint32_t pre = 0;
  for (int w = 0; w < warp; w++) pre += wsum[w];
  if ((uint32_t)tid < bins) {
    uint32_t acc = pre + x - tot;
    starts[tid] = acc;
    for (int w = 0; w < kSmallWarps; w++) {
      const uint32_t c = cnt[(uint32_t)w * row + tid];
      cnt[(uint32_t)w * row + tid] = acc;
      acc += c;
    }
  }
  if (tid == 0) starts[bins] = n;
  __syncthreads();
  // 3. ranks and stores, in the order of the counts
  for (uint32_t base = wb; base < wb + seg; base += 32) {
    const uint32_t e = base + lane;
    const bool ok = e < we;
    const uint32_t d = ok ? keys[e] : bins;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const uint32_t rank = (uint32_t)__popc(peers & lt_mask);
    const uint32_t at = ok ? wc[d] : 0u;
    __syncwarp();
    if (ok) {
      kout[at + rank] = d;
      vout[at + rank] = e;
      if (rank == 0) wc[d] = at + (uint32_t)__popc(peers);
    }
    __syncwarp();
  }
}

// Opts k_small_sort in to the dynamic shared memory of its largest case (about 192 KB). The
// attribute belongs to the device that is current, so every world calls this on its own device.
cudaError_t configure_sort_kernels() {
  return cudaFuncSetAttribute(k_small_sort, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)((kSmallSortMaxN + (uint32_t)kSmallWarps * (kSmallSortMaxBins + 1)) *
                                    sizeof(uint32_t)));
}

bool launch_sort(const TickInfo& t, const SortInfo& s, const uint32_t** perm_out, const uint32_t** keys_out,
                 int grid_ctas, cudaStream_t st) {
  *perm_out = s.vals_a;
  *keys_out = s.keys_a;
  if (s.n == 0) return false;
  if (s.keys_in && s.starts_out && small_sort_ok(s.n, s.bins, true)) {
    // the shared-memory opt-in of the largest case was set on this device by configure_sort_kernels()
    const int smem = (int)((s.n + (uint32_t)kSmallWarps * (s.bins + 1)) * sizeof(uint32_t));
    k_small_sort<<<1, kSmallThreads, smem, st>>>(s.keys_in, s.n, s.bins, s.keys_a, s.vals_a, s.starts_out);
    return true;
  }
  const uint32_t tiles = (s.n + kSortTile - 1) / kSortTile;
  if (!s.keys_in) {
    int ctas = (int)std::min<uint32_t>(tiles, (uint32_t)grid_ctas);
    k_sort_init<<<ctas, kCtaThreads, 0, st>>>(t, s.keys_a, s.vals_a, s.tile_scene, s.sentinel, tiles, s.hist);
  }
  uint32_t *ka = s.keys_a, *va = s.vals_a, *kb = s.keys_b, *vb = s.vals_b;
  for (int p = 0; p < s.passes; p++) {
    const int shift = p * kRadixBits;
    int ctas = (int)std::min<uint32_t>(tiles, (uint32_t)grid_ctas);
    const uint32_t* kin = (p == 0 && s.keys_in) ? s.keys_in : ka;
    const uint32_t* vin = (p == 0 && s.keys_in) ? nullptr : va;
    if (p > 0 || s.keys_in) k_radix_hist<<<ctas, kCtaThreads, 0, st>>>(kin, s.n, shift, s.hist, tiles);
    if (s.keys_in) {
      k_radix_scan<<<256, kCtaThreads, 0, st>>>(s.hist, tiles, s.digit_total);
      k_radix_scatter<false><<<ctas, kCtaThreads, 0, st>>>(kin, vin, kb, vb, s.n, shift, s.hist, s.digit_total, tiles,
                                                          nullptr, nullptr, nullptr);
    } else {   // segmented: the concatenation of the sorting scenes, each sorted within its own tiles
      k_radix_scan_seg<<<256, kCtaThreads, 0, st>>>(s.hist, tiles, s.tile_scene, s.seg_total);
      k_radix_scatter<true><<<ctas, kCtaThreads, 0, st>>>(kin, vin, kb, vb, s.n, shift, s.hist, nullptr, tiles,
                                                         s.tile_scene, s.seg_total, t.ts);
    }
    uint32_t* tk = ka; ka = kb; kb = tk;
    uint32_t* tv = va; va = vb; vb = tv;
  }
  *perm_out = va;
  *keys_out = ka;
  return false;
}

void launch_scene_starts_all(const TickInfo& t, const uint32_t* sorted_keys, uint32_t max_blocks, cudaStream_t st) {
  if (t.nscenes == 0) return;
  dim3 grid((unsigned)std::min<uint32_t>((max_blocks + 1 + 255) / 256, 1024u), (unsigned)t.nscenes);
  k_scene_starts<<<grid, 256, 0, st>>>(t, sorted_keys);
}

}  // namespace si

// ------------------------------------------------------------------ allocation-free block sort
// The block binning of _sort() (keys, stable order, starts) for positions the caller already holds
// on the device, with every intermediate buffer in one file-scope device array instead of memory
// from cudaMalloc. For callers that must not allocate device memory: a host that has handed the
// GPU's memory to its own pool, a stream that is being recorded into a CUDA graph, or a frame loop
// that cannot afford the device-wide synchronisation cudaFree implies.
namespace si {

constexpr int64_t kNoAllocMaxParticles = 262144;   // the reference MPM's default capacity
constexpr int64_t kNoAllocTiles = (kNoAllocMaxParticles + kSortTile - 1) / kSortTile;
// two (key, index) ping-pong pairs, the per-tile digit histogram and the digit totals
constexpr int64_t kNoAllocWords = 4 * kNoAllocMaxParticles + 256 * kNoAllocTiles + 256;
static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoAllocWords];

__global__ void k_na_keys(const float* __restrict__ x, int64_t stride, int32_t n, uint32_t num_blocks,
                          uint32_t* keys_out, uint32_t* skeys, uint32_t* svals) {
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float* p = x + (int64_t)i * stride;
    const uint32_t k = block_key(p[0], p[1], p[2], num_blocks);   // the key of si_mpm_sort, one definition
    keys_out[i] = k;
    skeys[i] = k;
    svals[i] = (uint32_t)i;
  }
}

__global__ void k_na_starts(const uint32_t* __restrict__ skeys, int32_t n, uint32_t num_blocks, uint32_t* starts) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k <= num_blocks; k += gridDim.x * blockDim.x) {
    uint32_t lo = 0, hi = (uint32_t)n;
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (__ldg(&skeys[mid]) < k) lo = mid + 1; else hi = mid;
    }
    starts[k] = lo;
  }
}

}  // namespace si

extern "C" int si_fail_c(int code, const char* msg);

extern "C" int si_block_sort_noalloc(const float* x, int64_t stride_floats, int32_t n, const int32_t dims[3],
                                     uint32_t* keys, uint32_t* perm, uint32_t* starts, void* stream) {
  using namespace si;
  if (n < 0 || (n > 0 && (!x || !keys || !perm)) || !dims || !starts || stride_floats < 3)
    return si_fail_c(SI_EINVAL, "si_block_sort_noalloc: bad argument (null pointer, n < 0 or stride < 3)");
  if (n > kNoAllocMaxParticles)
    return si_fail_c(SI_EINVAL, "si_block_sort_noalloc: n exceeds the fixed scratch capacity of 262144 particles");
  int32_t bmax = 0;
  for (int a = 0; a < 3; a++) {
    if (dims[a] <= 0 || dims[a] > 4096) return si_fail_c(SI_EINVAL, "si_block_sort_noalloc: dims must be in [1, 4096]");
    bmax = std::max(bmax, (dims[a] + 3) / 4);
  }
  uint32_t bpow = 1;
  while ((int32_t)bpow < bmax) bpow <<= 1;
  const uint32_t nb = bpow * bpow * bpow;   // numBlocks of mpm.js:119-121
  // set-up, once per device and with that device current: the array's device address
  static std::mutex mu;
  static uint32_t* base[64] = {nullptr};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return si_fail_c(SI_EDEVICE, "si_block_sort_noalloc: no current CUDA device");
  uint32_t* scratch = nullptr;
  {
    std::lock_guard<std::mutex> g(mu);
    if (!base[dev]) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess) {
        cudaGetLastError();
        return si_fail_c(SI_EDEVICE, "si_block_sort_noalloc: cudaGetSymbolAddress of the scratch array failed");
      }
      base[dev] = static_cast<uint32_t*>(p);
    }
    scratch = base[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int ctas = 1024;
  if (n == 0) {
    k_na_starts<<<(unsigned)std::min<uint64_t>((nb + 256) / 256, 4096), 256, 0, st>>>(scratch, 0, nb, starts);
    return cudaGetLastError() == cudaSuccess ? SI_OK : si_fail_c(SI_EDEVICE, "si_block_sort_noalloc: launch failed");
  }
  uint32_t* ka = scratch;
  uint32_t* va = scratch + kNoAllocMaxParticles;
  uint32_t* kb = scratch + 2 * kNoAllocMaxParticles;
  uint32_t* vb = scratch + 3 * kNoAllocMaxParticles;
  uint32_t* hist = scratch + 4 * kNoAllocMaxParticles;
  uint32_t* digit_total = hist + 256 * kNoAllocTiles;
  k_na_keys<<<(unsigned)std::min<int64_t>((n + 255) / 256, ctas), 256, 0, st>>>(x, stride_floats, n, nb, keys, ka, va);
  int bits = 1;
  while (bits < 32 && (1ull << bits) < (uint64_t)std::max<uint32_t>(nb, 2u)) bits++;
  const int passes = (bits + kRadixBits - 1) / kRadixBits;
  const uint32_t tiles = ((uint32_t)n + kSortTile - 1) / kSortTile;
  for (int p = 0; p < passes; p++) {
    const int shift = p * kRadixBits;
    k_radix_hist<<<tiles, kCtaThreads, 0, st>>>(ka, (uint32_t)n, shift, hist, tiles);
    k_radix_scan<<<256, kCtaThreads, 0, st>>>(hist, tiles, digit_total);
    k_radix_scatter<false><<<tiles, kCtaThreads, 0, st>>>(ka, va, kb, vb, (uint32_t)n, shift, hist, digit_total, tiles,
                                                         nullptr, nullptr, nullptr);
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  k_na_starts<<<(unsigned)std::min<uint64_t>((nb + 256) / 256, 4096), 256, 0, st>>>(ka, n, nb, starts);
  if (cudaMemcpyAsync(perm, va, sizeof(uint32_t) * (size_t)n, cudaMemcpyDeviceToDevice, st) != cudaSuccess) {
    cudaGetLastError();
    return si_fail_c(SI_EDEVICE, "si_block_sort_noalloc: copy of the order failed");
  }
  return cudaGetLastError() == cudaSuccess ? SI_OK : si_fail_c(SI_EDEVICE, "si_block_sort_noalloc: launch failed");
}

// ------------------------------------------------------------------ SpatialGrid (src/prims/grid.js)
// Uniform-grid neighbour binning of arbitrary points: cell = gridIndex(gridCoord(p)) (grid.js:14-20,
// x-fastest), then the same stable radix sort as the block sort, and start[] = the first sorted slot
// of every cell (numCells + 1 entries). The reference ranks points within a cell by atomic arrival
// (any order); the stable sort keeps them in index order, one of those orders, always the same.
#include "si_runtime.h"

struct si_spatial {
  si_world* w = nullptr;
  int64_t max_count = 0, count = 0;
  int32_t dims[3] = {1, 1, 1};
  uint32_t cells = 1;
  float origin[3] = {0, 0, 0};
  float inv = 1.0f;
  uint32_t *ka = nullptr, *va = nullptr, *kb = nullptr, *vb = nullptr, *hist = nullptr, *digit_total = nullptr;
  uint32_t* start = nullptr;
  uint32_t* order = nullptr;   // points to va or vb after a build
  float4* pos = nullptr;       // staging of host positions
  bool destroyed = false;
};

namespace si {
// gridCoord + gridIndex, grid.js:14-20: clamp(vec3i(floor((p - origin) * inv)), 0, dims - 1)
__global__ void k_spatial_cells(const float4* __restrict__ pos, int64_t n, float o0, float o1, float o2, float inv,
                                int32_t d0, int32_t d1, int32_t d2, uint32_t* keys, uint32_t* vals) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float4 p = pos[i];
    const int32_t cx = min(max(__float2int_rz(floorf((p.x - o0) * inv)), 0), d0 - 1);
    const int32_t cy = min(max(__float2int_rz(floorf((p.y - o1) * inv)), 0), d1 - 1);
    const int32_t cz = min(max(__float2int_rz(floorf((p.z - o2) * inv)), 0), d2 - 1);
    keys[i] = (uint32_t)cx + (uint32_t)d0 * ((uint32_t)cy + (uint32_t)d1 * (uint32_t)cz);
    vals[i] = (uint32_t)i;
  }
}

__global__ void k_spatial_gather(const float* __restrict__ src, float* dst, const uint32_t* __restrict__ order,
                                 int64_t n, int32_t width) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * width; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = t / width;
    dst[t] = src[(int64_t)order[k] * width + (t - k * width)];
  }
}
}  // namespace si

static int spatial_sort(si_spatial* g, const float4* pos, int64_t n) {
  using namespace si;
  cudaStream_t st = g->w->st;
  g->count = n;
  if (n > 0) {
    const unsigned ctas = (unsigned)std::min<int64_t>((n + 255) / 256, 4096);
    k_spatial_cells<<<ctas, 256, 0, st>>>(pos, n, g->origin[0], g->origin[1], g->origin[2], g->inv, g->dims[0],
                                          g->dims[1], g->dims[2], g->ka, g->va);
    int bits = 1;
    while (bits < 32 && (1ull << bits) < (uint64_t)std::max<uint32_t>(g->cells, 2u)) bits++;
    const int passes = (bits + kRadixBits - 1) / kRadixBits;
    const uint32_t tiles = ((uint32_t)n + kSortTile - 1) / kSortTile;
    uint32_t *ka = g->ka, *va = g->va, *kb = g->kb, *vb = g->vb;
    for (int p = 0; p < passes; p++) {
      k_radix_hist<<<tiles, kCtaThreads, 0, st>>>(ka, (uint32_t)n, p * kRadixBits, g->hist, tiles);
      k_radix_scan<<<256, kCtaThreads, 0, st>>>(g->hist, tiles, g->digit_total);
      k_radix_scatter<false><<<tiles, kCtaThreads, 0, st>>>(ka, va, kb, vb, (uint32_t)n, p * kRadixBits, g->hist,
                                                            g->digit_total, tiles, nullptr, nullptr, nullptr);
      std::swap(ka, kb);
      std::swap(va, vb);
    }
    g->order = va;
    k_na_starts<<<(unsigned)std::min<uint64_t>(((uint64_t)g->cells + 256) / 256, 65535), 256, 0, st>>>(
        ka, (int32_t)n, g->cells, g->start);
  } else {
    g->order = g->va;
    k_na_starts<<<(unsigned)std::min<uint64_t>(((uint64_t)g->cells + 256) / 256, 65535), 256, 0, st>>>(
        g->ka, 0, g->cells, g->start);
  }
  return cudaGetLastError() == cudaSuccess ? SI_OK : si_fail_c(SI_EDEVICE, "SpatialGrid.build: launch failed");
}

#define SG_GUARD(g)                                                                     \
  if (!(g)) return si_fail_c(SI_EINVAL, "null SpatialGrid");                            \
  std::lock_guard<std::recursive_mutex> sg_lock_((g)->w->api_mu);                       \
  if ((g)->destroyed || (g)->w->destroyed) return si_fail_c(SI_EDESTROYED, "SpatialGrid: it was destroyed")

extern "C" {

int si_spatial_create(si_world* w, int64_t max_count, const double mn[3], const double mx[3], double cell_size,
                      si_spatial** out) {
  if (!w || !mn || !mx || !out) return si_fail_c(SI_EINVAL, "SpatialGrid: null argument");
  if (max_count < 0 || max_count > ((int64_t)1 << 31) - 1) return si_fail_c(SI_EINVAL, "SpatialGrid: bad maxCount");
  if (!(cell_size > 0)) return si_fail_c(SI_EINVAL, "SpatialGrid: cellSize must be > 0");
  std::lock_guard<std::recursive_mutex> lock(w->api_mu);
  if (w->destroyed) return si_fail_c(SI_EDESTROYED, "the world was destroyed");
  auto* g = new si_spatial();
  g->w = w;
  g->max_count = max_count;
  uint64_t cells = 1;
  for (int a = 0; a < 3; a++) {   // grid.js:31-33
    g->dims[a] = (int32_t)std::max(1.0, std::ceil((mx[a] - mn[a]) / cell_size));
    g->origin[a] = (float)mn[a];
    cells *= (uint64_t)g->dims[a];
  }
  if (cells > (1u << 26)) {
    delete g;
    return si_fail_c(SI_EINVAL, "SpatialGrid: too many cells; increase cellSize");
  }
  g->cells = (uint32_t)cells;
  g->inv = (float)(1.0 / cell_size);
  cudaStream_t st = w->st;
  const size_t n = (size_t)std::max<int64_t>(max_count, 1);
  const size_t tiles = (n + si::kSortTile - 1) / si::kSortTile;
  cudaError_t e = cudaSuccess;
  for (uint32_t** p : {&g->ka, &g->va, &g->kb, &g->vb})
    if (e == cudaSuccess) e = cudaMallocAsync((void**)p, n * 4, st);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&g->hist, 256 * tiles * 4, st);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&g->digit_total, 256 * 4, st);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&g->start, ((size_t)cells + 1) * 4, st);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&g->pos, n * 16, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(g->start, 0, ((size_t)cells + 1) * 4, st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    for (void* p : {(void*)g->ka, (void*)g->va, (void*)g->kb, (void*)g->vb, (void*)g->hist, (void*)g->digit_total,
                    (void*)g->start, (void*)g->pos})
      if (p) cudaFreeAsync(p, st);
    delete g;
    return si_fail_c(e == cudaErrorMemoryAllocation ? SI_ENOMEM : SI_EDEVICE, "SpatialGrid: device allocation failed");
  }
  g->order = g->va;
  *out = g;
  return SI_OK;
}

int si_spatial_destroy(si_spatial* g) {
  if (!g) return si_fail_c(SI_EINVAL, "null SpatialGrid");
  {
    std::lock_guard<std::recursive_mutex> lock(g->w->api_mu);
    if (!g->destroyed && !g->w->destroyed) {
      for (void* p : {(void*)g->ka, (void*)g->va, (void*)g->kb, (void*)g->vb, (void*)g->hist, (void*)g->digit_total,
                      (void*)g->start, (void*)g->pos})
        if (p) cudaFreeAsync(p, g->w->st);
      cudaStreamSynchronize(g->w->st);
    }
    g->destroyed = true;
  }
  delete g;
  return SI_OK;
}

int si_spatial_info(const si_spatial* g, int32_t dims[3], int64_t* num_cells, int64_t* count) {
  if (!g) return si_fail_c(SI_EINVAL, "null SpatialGrid");
  if (dims) for (int a = 0; a < 3; a++) dims[a] = g->dims[a];
  if (num_cells) *num_cells = g->cells;
  if (count) *count = g->count;
  return SI_OK;
}

int si_spatial_build(si_spatial* g, const float* pos, int64_t count) {
  SG_GUARD(g);
  if (count < 0 || (count && !pos)) return si_fail_c(SI_EINVAL, "SpatialGrid.build: bad positions");
  if (count > g->max_count) return si_fail_c(SI_EINVAL, "SpatialGrid.build: points exceed maxCount");
  if (count && cudaMemcpyAsync(g->pos, pos, (size_t)count * 16, cudaMemcpyHostToDevice, g->w->st) != cudaSuccess)
    return si_fail_c(SI_EDEVICE, "SpatialGrid.build: upload failed");
  return spatial_sort(g, g->pos, count);
}

int si_spatial_build_mpm(si_spatial* g, const si_mpm* h) {
  SG_GUARD(g);
  if (!h || h->destroyed) return si_fail_c(SI_EINVAL, "SpatialGrid.build: no simulation");
  if (h->w != g->w) return si_fail_c(SI_EINVAL, "SpatialGrid.build: the simulation belongs to another world");
  if (h->count > g->max_count) return si_fail_c(SI_EINVAL, "SpatialGrid.build: points exceed maxCount");
  return spatial_sort(g, h->pbuf[h->pcur], h->count);
}

int si_spatial_read(si_spatial* g, uint32_t* order, uint32_t* start) {
  SG_GUARD(g);
  cudaStream_t st = g->w->st;
  if (order && g->count &&
      cudaMemcpyAsync(order, g->order, (size_t)g->count * 4, cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return si_fail_c(SI_EDEVICE, "SpatialGrid: read failed");
  if (start && cudaMemcpyAsync(start, g->start, ((size_t)g->cells + 1) * 4, cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return si_fail_c(SI_EDEVICE, "SpatialGrid: read failed");
  return cudaStreamSynchronize(st) == cudaSuccess ? SI_OK : si_fail_c(SI_EDEVICE, "SpatialGrid: read failed");
}

int si_spatial_gather(si_spatial* g, const float* src, float* dst, int32_t width) {
  SG_GUARD(g);
  if (width <= 0 || (g->count && (!src || !dst))) return si_fail_c(SI_EINVAL, "SpatialGrid.gather: bad arguments");
  if (!g->count) return SI_OK;
  cudaStream_t st = g->w->st;
  const size_t bytes = (size_t)g->count * (size_t)width * 4;
  float *ds = nullptr, *dd = nullptr;
  if (cudaMallocAsync((void**)&ds, bytes, st) != cudaSuccess || cudaMallocAsync((void**)&dd, bytes, st) != cudaSuccess) {
    cudaGetLastError();
    if (ds) cudaFreeAsync(ds, st);
    return si_fail_c(SI_ENOMEM, "SpatialGrid.gather: device allocation failed");
  }
  cudaMemcpyAsync(ds, src, bytes, cudaMemcpyHostToDevice, st);
  const int64_t total = g->count * width;
  si::k_spatial_gather<<<(unsigned)std::min<int64_t>((total + 255) / 256, 8192), 256, 0, st>>>(ds, dd, g->order,
                                                                                             g->count, width);
  cudaMemcpyAsync(dst, dd, bytes, cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(ds, st);
  cudaFreeAsync(dd, st);
  return cudaStreamSynchronize(st) == cudaSuccess ? SI_OK : si_fail_c(SI_EDEVICE, "SpatialGrid.gather failed");
}

}  // extern "C"
