// Value-block slot assignment that allocates nothing.
//
// Same result as the slot scan inside msbg_gpu_set_refinement_map
// (context.cu): slot[bid] = rank of bid among the level-0 blocks in ascending
// bid order, -1 for every other block; activeBids[rank] = bid; *count = number
// of level-0 blocks.  It exists for callers that cannot allocate device memory
// at all (an allocator owned by another runtime, a memory budget fixed up
// front, code paths that must not call cudaMalloc/cudaFree): it needs no
// context, allocates nothing, and keeps its only scratch -- the per-tile partial
// sums of the scan -- in the file-scope device array below.
//
// Scratch rules:
//   * g_slotScanPartials lives on every device that loads this library, for the
//     life of the process (kNoAllocMaxTiles int64 values, 32 KiB).
//   * Host code cannot use the array's name as a device address, so the first
//     call on each device looks its address up with cudaGetSymbolAddress (with
//     that device current) and caches it.  Make that first call before any
//     stream capture.
//   * Every call reuses the same array.  The kernels overwrite every partial they
//     read, so nothing has to be cleared between calls, but two calls whose
//     kernels overlap on the GPU (different streams, no ordering) race on it.
#include <mutex>

#include "internal.cuh"

namespace {

constexpr int kThreads = 512;
constexpr int kItems = 8;
constexpr int kTile = kThreads * kItems;           // blocks per scan tile
constexpr int64_t kNoAllocMaxBlocks = (int64_t)1 << 24;
constexpr int64_t kNoAllocMaxTiles = kNoAllocMaxBlocks / kTile;  // 4096

static_assert(MSBG_GPU_NOALLOC_MAX_BLOCKS == kNoAllocMaxBlocks, "header and library disagree");

// The scratch: one partial sum per scan tile (exclusive prefix after phase 2).
__device__ __align__(256) int64_t g_slotScanPartials[kNoAllocMaxTiles];

__device__ __forceinline__ int64_t warpIncl(int64_t v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// exclusive prefix of v over the CTA; *total = CTA sum
__device__ int64_t ctaExclusive(int64_t v, int64_t *total) {
  __shared__ int64_t ws[kThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t inc = warpIncl(v);
  if (lane == 31) ws[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    int64_t s = lane < kThreads / 32 ? ws[lane] : 0;
    s = warpIncl(s);
    if (lane < kThreads / 32) ws[lane] = s;
  }
  __syncthreads();
  const int64_t off = warp ? ws[warp - 1] : 0;
  *total = ws[kThreads / 32 - 1];
  __syncthreads();
  return off + inc - v;
}

__global__ void kTileCounts(const int32_t *__restrict__ levels, int64_t n, int64_t *__restrict__ part) {
  const int64_t base = (int64_t)blockIdx.x * kTile;
  int64_t c = 0;
#pragma unroll
  for (int k = 0; k < kItems; k++) {
    const int64_t i = base + (int64_t)k * kThreads + threadIdx.x;
    if (i < n) c += levels[i] == 0;
  }
  int64_t tot;
  ctaExclusive(c, &tot);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

__global__ void kTileOffsets(int64_t *part, int64_t nTiles, int64_t *count) {
  int64_t carry = 0;
  for (int64_t c0 = 0; c0 < nTiles; c0 += kThreads) {
    const int64_t i = c0 + threadIdx.x;
    const int64_t v = i < nTiles ? part[i] : 0;
    int64_t tot;
    const int64_t ex = ctaExclusive(v, &tot);
    if (i < nTiles) part[i] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0) *count = carry;
}

__global__ void kTileSlots(const int32_t *__restrict__ levels, int64_t n, const int64_t *__restrict__ part,
                           int32_t *__restrict__ slot, int32_t *__restrict__ active) {
  const int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kItems;
  int v[kItems];
  int64_t s = 0;
#pragma unroll
  for (int k = 0; k < kItems; k++) {
    const int64_t i = base + k;
    v[k] = (i < n && levels[i] == 0) ? 1 : 0;
    s += v[k];
  }
  int64_t tot;
  int64_t off = ctaExclusive(s, &tot) + part[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kItems; k++) {
    const int64_t i = base + k;
    if (i < n) {
      if (v[k]) {
        slot[i] = (int32_t)off;
        active[off] = (int32_t)i;
        off++;
      } else {
        slot[i] = -1;
      }
    }
  }
}

// Device address of the scratch array, looked up once per device.
constexpr int kMaxDevices = 64;
std::mutex g_scratchLock;
int64_t *g_scratchPtr[kMaxDevices] = {};

int scratchFor(int dev, int64_t **out) {
  std::lock_guard<std::mutex> lk(g_scratchLock);
  if (!g_scratchPtr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_slotScanPartials);
    if (e != cudaSuccess || !p) return MSBG_GPU_ERR_CUDA;
    g_scratchPtr[dev] = (int64_t *)p;
  }
  *out = g_scratchPtr[dev];
  return MSBG_GPU_OK;
}

}  // namespace

extern "C" int msbg_gpu_assign_slots_noalloc(const int32_t *dLevels, int64_t nBlocks, int32_t *dSlot,
                                             int32_t *dActiveBids, int64_t *dCount, void *cudaStream) {
  if (!dSlot || !dActiveBids || !dCount || nBlocks < 0 || (nBlocks > 0 && !dLevels))
    return MSBG_GPU_ERR_ARG;
  if (nBlocks > kNoAllocMaxBlocks) return MSBG_GPU_ERR_CAPACITY;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return MSBG_GPU_ERR_CUDA;
  int64_t *part = nullptr;
  const int rc = scratchFor(dev, &part);
  if (rc != MSBG_GPU_OK) return rc;
  // An error that earlier, unrelated work left in the runtime is not this call's:
  // report it without launching and leave it for its owner to read.
  if (cudaPeekAtLastError() != cudaSuccess) return MSBG_GPU_ERR_CUDA;
  cudaStream_t st = (cudaStream_t)cudaStream;
  const int64_t nTiles = (nBlocks + kTile - 1) / kTile;
  if (nTiles > 0) kTileCounts<<<(unsigned)nTiles, kThreads, 0, st>>>(dLevels, nBlocks, part);
  kTileOffsets<<<1, kThreads, 0, st>>>(part, nTiles, dCount);
  if (nTiles > 0) kTileSlots<<<(unsigned)nTiles, kThreads, 0, st>>>(dLevels, nBlocks, part, dSlot, dActiveBids);
  return cudaGetLastError() == cudaSuccess ? MSBG_GPU_OK : MSBG_GPU_ERR_CUDA;
}
