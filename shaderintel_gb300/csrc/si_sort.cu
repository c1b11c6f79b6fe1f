// si_sort.cu — the block sort of mpm.js:563-577/614-621 for one tick of many scenes.
//
// The reference counts keys with global atomics, so the order inside a block depends on atomic
// timing. Here the particles of every sorting scene are concatenated with key = bin_base + block key
// and sorted by a stable LSD radix sort (8-bit digits; per pass: tile histograms, a scan per digit,
// a stable scatter ranked with warp match + shared-memory prefixes). It is deterministic, has no
// waits between CTAs, and yields the reference's counts and starts exactly; each scene's particles
// stay inside its own segment because the bin ranges are ordered like the segments.
#include <algorithm>
#include <mutex>

#include "si_cuda.h"
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
    const float fx = fminf(fmaxf(p[0], 0.0f), 16777216.0f), fy = fminf(fmaxf(p[1], 0.0f), 16777216.0f);
    const float fz = fminf(fmaxf(p[2], 0.0f), 16777216.0f);
    const uint32_t bx = ((uint32_t)fx) / 4u, by = ((uint32_t)fy) / 4u, bz = ((uint32_t)fz) / 4u;
    auto part = [](uint32_t v) {
      v &= 0x3ffu;
      v = (v | (v << 16)) & 0x030000ffu;
      v = (v | (v << 8)) & 0x0300f00fu;
      v = (v | (v << 4)) & 0x030c30c3u;
      v = (v | (v << 2)) & 0x09249249u;
      return v;
    };
    uint32_t k = part(bx) | (part(by) << 1) | (part(bz) << 2);
    k = k < num_blocks ? k : num_blocks - 1u;
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
    k_radix_scatter<<<tiles, kCtaThreads, 0, st>>>(ka, va, kb, vb, (uint32_t)n, shift, hist, digit_total, tiles);
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
