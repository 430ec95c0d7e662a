// Context lifecycle, block pool, refinement map and the ABI glue of msbg_gpu.
//
// Reference counterparts:
//   MultiresSparseGrid::create/destroy          src/msbg.cpp:116-1106
//   regularizeRefinementMap                     src/msbg.cpp:1202-1423
//   setRefinementMap (levelMg 0 BlockInfo)      src/msbg.cpp:1428-2165
//   demo active marking / allocation            src/msbg_demo.cpp:339-511
//   BlockPool (monotonic fixed-size blocks)     src/blockpool.cpp:237-351
// The block pool here is one payload slab per channel, [nActive][bs^3], whose
// slots are handed out by an exclusive scan over the level map (ascending bid,
// the order of the demo's activeBlocks list) instead of an atomic bump pointer.
#include <stdarg.h>
#include <string.h>

#include <cmath>

#include "internal.cuh"
#include "poisson.cuh"

namespace msbg {

int fail(msbg_gpu_ctx *ctx, int code, const char *fmt, ...) {
  if (ctx) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    ctx->err = buf;
  }
  return code;
}

int cudaFail(msbg_gpu_ctx *ctx, cudaError_t e, const char *what) {
  return fail(ctx, e == cudaErrorMemoryAllocation ? MSBG_GPU_ERR_NOMEM : MSBG_GPU_ERR_CUDA,
              "%s: %s", what, cudaGetErrorString(e));
}

// ---------------------------------------------------------------------------------
// Exclusive scan of 0/1 flags (int32) into int64 offsets.  Three phases: per-CTA
// sums, a single-CTA scan of those sums, per-CTA scan plus offset.  The partial
// sums live in ctx->dScanPartial (sized for nBlocks at create time).
// ---------------------------------------------------------------------------------
constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;  // per thread
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int64_t warpInclusive(int64_t v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Block-wide exclusive scan of one value per thread; returns exclusive prefix,
// *total receives the block sum.
__device__ int64_t blockExclusive(int64_t v, int64_t *total) {
  __shared__ int64_t warpSums[kScanThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t inc = warpInclusive(v);
  if (lane == 31) warpSums[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    int64_t s = lane < (kScanThreads / 32) ? warpSums[lane] : 0;
    s = warpInclusive(s);
    if (lane < (kScanThreads / 32)) warpSums[lane] = s;
  }
  __syncthreads();
  const int64_t warpOff = warp ? warpSums[warp - 1] : 0;
  *total = warpSums[kScanThreads / 32 - 1];
  __syncthreads();
  return warpOff + inc - v;
}

// FLAGS: scan the 0/1 flags of the inputs (in[i] != 0); otherwise the values
// themselves (non-negative counts).
template <bool FLAGS>
__device__ __forceinline__ int64_t scanItem(int32_t v) {
  if constexpr (FLAGS) return v != 0; else return (int64_t)v;
}

template <bool FLAGS>
__global__ void kScanReduce(const int32_t *__restrict__ in, int64_t n, int64_t *__restrict__ part) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  int64_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    const int64_t i = base + (int64_t)k * kScanThreads + threadIdx.x;
    if (i < n) s += scanItem<FLAGS>(in[i]);
  }
  int64_t tot;
  blockExclusive(s, &tot);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

__global__ void kScanPartials(int64_t *part, int64_t nPart, int64_t *total) {
  // single CTA, sequential over chunks of kScanThreads
  int64_t carry = 0;
  for (int64_t c = 0; c < nPart; c += kScanThreads) {
    const int64_t i = c + threadIdx.x;
    const int64_t v = i < nPart ? part[i] : 0;
    int64_t tot;
    const int64_t ex = blockExclusive(v, &tot);
    if (i < nPart) part[i] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0) *total = carry;
}

template <bool FLAGS>
__global__ void kScanApply(const int32_t *__restrict__ in, int64_t n, const int64_t *__restrict__ part,
                           int64_t *__restrict__ out) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int64_t v[kScanItems];
  int64_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    const int64_t i = base + k;
    v[k] = i < n ? scanItem<FLAGS>(in[i]) : 0;
    s += v[k];
  }
  int64_t tot;
  int64_t ex = blockExclusive(s, &tot) + part[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    const int64_t i = base + k;
    if (i < n) out[i] = ex;
    ex += v[k];
  }
}

template <bool FLAGS>
static int exclusiveScanT(msbg_gpu_ctx *ctx, const int32_t *dIn, int64_t n, int64_t *dOut, int64_t *dTotal,
                          int64_t *dPartial) {
  const int64_t nPart = (n + kScanTile - 1) / kScanTile;
  MSBG_LAUNCH(ctx, kScanReduce<FLAGS>, (unsigned)nPart, kScanThreads, 0, dIn, n, dPartial);
  MSBG_LAUNCH(ctx, kScanPartials, 1, kScanThreads, 0, dPartial, nPart, dTotal);
  MSBG_LAUNCH(ctx, kScanApply<FLAGS>, (unsigned)nPart, kScanThreads, 0, dIn, n, dPartial, dOut);
  return MSBG_GPU_OK;
}

int exclusiveScanFlagsWith(msbg_gpu_ctx *ctx, const int32_t *dIn, int64_t n, int64_t *dOut,
                           int64_t *dTotal, int64_t *dPartial) {
  return exclusiveScanT<true>(ctx, dIn, n, dOut, dTotal, dPartial);
}

int exclusiveScanCounts(msbg_gpu_ctx *ctx, const int32_t *dIn, int64_t n, int64_t *dOut, int64_t *dTotal) {
  return exclusiveScanT<false>(ctx, dIn, n, dOut, dTotal, ctx->dScanPartial);
}

int64_t scanPartialCount(int64_t n) { return (n + kScanTile - 1) / kScanTile; }

int exclusiveScanFlags(msbg_gpu_ctx *ctx, const int32_t *dIn, int64_t n, int64_t *dOut,
                       int64_t *dTotal) {
  return exclusiveScanFlagsWith(ctx, dIn, n, dOut, dTotal, ctx->dScanPartial);
}

__global__ void kReadSmall(const uint32_t *__restrict__ src, int nWords, uint32_t *__restrict__ hDst) {
  for (int i = threadIdx.x; i < nWords; i += blockDim.x) hDst[i] = src[i];
}

int readSmall(msbg_gpu_ctx *ctx, void *hDst, const void *dSrc, size_t bytes) {
  if (bytes > kSmallReadBytes || (bytes & 3) || ((uintptr_t)dSrc & 3))
    return fail(ctx, MSBG_GPU_ERR_ARG, "readSmall: %zu bytes", bytes);
  if (bytes) MSBG_LAUNCH(ctx, kReadSmall, 1, 32, 0, (const uint32_t *)dSrc, (int)(bytes / 4), (uint32_t *)ctx->hSmall);
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (bytes) memcpy(hDst, ctx->hSmall, bytes);
  return MSBG_GPU_OK;
}

int copyAsyncSplit(msbg_gpu_ctx *ctx, void *dst, const void *src, size_t bytes, cudaMemcpyKind kind) {
  constexpr size_t kSplitBytes = size_t(64) << 20;
  if (bytes < kSplitBytes) {
    MSBG_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, kind, ctx->stream));
    return MSBG_GPU_OK;
  }
  if (!ctx->copyStream) {
    MSBG_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copyStream, cudaStreamNonBlocking));
    for (auto &e : ctx->copyEv) MSBG_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  const size_t half = (bytes / 2 + 4095) & ~size_t(4095);
  MSBG_CUDA(ctx, cudaEventRecord(ctx->copyEv[0], ctx->stream));
  MSBG_CUDA(ctx, cudaStreamWaitEvent(ctx->copyStream, ctx->copyEv[0], 0));
  MSBG_CUDA(ctx, cudaMemcpyAsync((char *)dst + half, (const char *)src + half, bytes - half, kind, ctx->copyStream));
  MSBG_CUDA(ctx, cudaMemcpyAsync(dst, src, half, kind, ctx->stream));
  MSBG_CUDA(ctx, cudaEventRecord(ctx->copyEv[1], ctx->copyStream));
  MSBG_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->copyEv[1], 0));
  return MSBG_GPU_OK;
}

int ensureTmpSlab(msbg_gpu_ctx *ctx, size_t bytes) {
  if (ctx->tmpSlabBytes >= bytes) return MSBG_GPU_OK;
  if (ctx->dTmpSlab) MSBG_CUDA(ctx, cudaFree(ctx->dTmpSlab));
  ctx->dTmpSlab = nullptr;
  ctx->tmpSlabBytes = 0;
  MSBG_CUDA(ctx, cudaMalloc(&ctx->dTmpSlab, bytes));
  ctx->tmpSlabBytes = bytes;
  return MSBG_GPU_OK;
}

// ---------------------------------------------------------------------------------
// Layout kernels
// ---------------------------------------------------------------------------------
struct GridGeom {
  int sx, sy, sz, nbx, nby, nbz, log2bs;
  float domMin[3], domMax[3];
};

__device__ __forceinline__ bool pointValid(const GridGeom &g, float px, float py, float pz) {
  if (px < g.domMin[0] || px > g.domMax[0] || py < g.domMin[1] || py > g.domMax[1] ||
      pz < g.domMin[2] || pz > g.domMax[2])
    return false;
  const int ix = (int)px, iy = (int)py, iz = (int)pz;
  return ix >= 0 && ix < g.sx && iy >= 0 && iy < g.sy && iz >= 0 && iz < g.sz;
}

// Active-block marking (src/msbg_demo.cpp:349-384): every block of the point's
// rScan box [trunc(p/bs - r/bs), trunc(p/bs + r/bs)] clamped to the grid.
__global__ void kMarkPoints(const float *__restrict__ pts, int64_t n, GridGeom g, float rScanBsx,
                            int32_t *__restrict__ mark, unsigned long long *nValid) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool ok = false;
  if (i < n) {
    const float px = pts[3 * i], py = pts[3 * i + 1], pz = pts[3 * i + 2];
    ok = pointValid(g, px, py, pz);
    if (ok) {
      const float scale = 1.0f / (float)(1 << g.log2bs);
      const float bx = __fmul_rn(px, scale), by = __fmul_rn(py, scale), bz = __fmul_rn(pz, scale);
      const int x1 = max((int)__fsub_rn(bx, rScanBsx), 0), x2 = min((int)__fadd_rn(bx, rScanBsx), g.nbx - 1);
      const int y1 = max((int)__fsub_rn(by, rScanBsx), 0), y2 = min((int)__fadd_rn(by, rScanBsx), g.nby - 1);
      const int z1 = max((int)__fsub_rn(bz, rScanBsx), 0), z2 = min((int)__fadd_rn(bz, rScanBsx), g.nbz - 1);
      for (int k = z1; k <= z2; k++)
        for (int j = y1; j <= y2; j++)
          for (int l = x1; l <= x2; l++) mark[((int64_t)k * g.nby + j) * g.nbx + l] = 1;
    }
  }
  const unsigned b = __ballot_sync(0xffffffffu, ok);
  if ((threadIdx.x & 31) == 0 && b) atomicAdd(nValid, (unsigned long long)__popc(b));
}

__global__ void kLevelsFromMarks(const int32_t *__restrict__ mark, int64_t n, int coarsest,
                                 int32_t *__restrict__ levels) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) levels[i] = mark[i] ? 0 : coarsest;
}

__global__ void kFillInt(int32_t *p, int64_t n, int32_t v) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

// Band levels: atomicMin(level, l) over the rBand box of every valid point.
__global__ void kBandLevels(const float *__restrict__ pts, int64_t n, GridGeom g, float rBsx, int level,
                            int32_t *__restrict__ levels) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float px = pts[3 * i], py = pts[3 * i + 1], pz = pts[3 * i + 2];
  if (!pointValid(g, px, py, pz)) return;
  const float scale = 1.0f / (float)(1 << g.log2bs);
  const float bx = __fmul_rn(px, scale), by = __fmul_rn(py, scale), bz = __fmul_rn(pz, scale);
  const int x1 = max((int)__fsub_rn(bx, rBsx), 0), x2 = min((int)__fadd_rn(bx, rBsx), g.nbx - 1);
  const int y1 = max((int)__fsub_rn(by, rBsx), 0), y2 = min((int)__fadd_rn(by, rBsx), g.nby - 1);
  const int z1 = max((int)__fsub_rn(bz, rBsx), 0), z2 = min((int)__fadd_rn(bz, rBsx), g.nbz - 1);
  for (int k = z1; k <= z2; k++)
    for (int j = y1; j <= y2; j++)
      for (int l = x1; l <= x2; l++) {
        int32_t *p = &levels[((int64_t)k * g.nby + j) * g.nbx + l];
        if (*p > level) atomicMin(p, level);
      }
}

// One pass ll of regularizeRefinementMap (src/msbg.cpp:1323-1369): a block at
// level >= ll whose finest 26-neighbour is at ll-1 becomes ll.
__global__ void kRegularizePass(const int32_t *__restrict__ src, int32_t *__restrict__ dst, int nbx,
                                int nby, int nbz, int nLevels, int ll) {
  const int64_t bid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nB = (int64_t)nbx * nby * nbz;
  if (bid >= nB) return;
  const int bx = (int)(bid % nbx), by = (int)((bid / nbx) % nby), bz = (int)(bid / ((int64_t)nbx * nby));
  int level = src[bid];
  if (level >= ll) {
    int finest = nLevels - 1;
    for (int dz = -1; dz <= 1; dz++) {
      const int z = bz + dz;
      if (z < 0 || z >= nbz) continue;
      for (int dy = -1; dy <= 1; dy++) {
        const int y = by + dy;
        if (y < 0 || y >= nby) continue;
        for (int dx = -1; dx <= 1; dx++) {
          const int x = bx + dx;
          if (x < 0 || x >= nbx || (!dx && !dy && !dz)) continue;
          finest = min(finest, src[((int64_t)z * nby + y) * nbx + x]);
        }
      }
    }
    if (finest == ll - 1) level = ll;
  }
  dst[bid] = level;
}

// BlockInfo flags of setRefinementMap for levelMg 0 (src/msbg.cpp:1632-1720),
// followed by the demo allocation loop's BLK_EXISTS on level-0 blocks
// (src/msbg_demo.cpp:477-491).  Also the per-level histogram.
__global__ void kBlockFlags(const int32_t *__restrict__ levels, uint16_t *__restrict__ flags, int nbx,
                            int nby, int nbz, unsigned long long *perLevel) {
  const int64_t bid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nB = (int64_t)nbx * nby * nbz;
  if (bid >= nB) return;
  const int bx = (int)(bid % nbx), by = (int)((bid / nbx) % nby), bz = (int)(bid / ((int64_t)nbx * nby));
  uint16_t f = 0;
  if (bx == 0 || bx == nbx - 1 || by == 0 || by == nby - 1 || bz == 0 || bz == nbz - 1)
    f |= MSBG_GPU_BLK_DOM_BORDER;
  const int level = levels[bid];
  int lmax = 0, lmin = 1 << 20;
  for (int dz = -1; dz <= 1; dz++) {
    const int z = bz + dz;
    if (z < 0 || z >= nbz) continue;
    for (int dy = -1; dy <= 1; dy++) {
      const int y = by + dy;
      if (y < 0 || y >= nby) continue;
      for (int dx = -1; dx <= 1; dx++) {
        const int x = bx + dx;
        if (x < 0 || x >= nbx || (!dx && !dy && !dz)) continue;
        const int l2 = levels[((int64_t)z * nby + y) * nbx + x];
        lmax = max(lmax, l2);
        lmin = min(lmin, l2);
      }
    }
  }
  if (lmax > level) f |= MSBG_GPU_BLK_FINE_COARSE;
  if (lmin < level) f |= MSBG_GPU_BLK_COARSE_FINE;
  if (!(f & (MSBG_GPU_BLK_FINE_COARSE | MSBG_GPU_BLK_COARSE_FINE))) f |= MSBG_GPU_BLK_UNIFORM_EMPTY;
  if (level == 0) f |= MSBG_GPU_BLK_EXISTS;
  flags[bid] = f;
  if (level >= 0 && level < 8) atomicAdd(&perLevel[level], 1ull);
}

__global__ void kValueFlags(const int32_t *__restrict__ levels, int64_t n, int32_t *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = levels[i] == 0;
}

// slot[bid] = exclusive-scan offset for value blocks, -1 otherwise; active list.
__global__ void kAssignSlots(const int32_t *__restrict__ levels, const int64_t *__restrict__ off,
                             int64_t n, int32_t *__restrict__ slot, int32_t *__restrict__ active) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (levels[i] == 0) {
    slot[i] = (int32_t)off[i];
    active[off[i]] = (int32_t)i;
  } else {
    slot[i] = -1;
  }
}

__device__ __forceinline__ int blockColor8(int bx, int by, int bz) {
  return (bx & 1) + ((by & 1) << 1) + ((bz & 1) << 2);  // src/msbg.h:642-646
}

__global__ void kColorFlags(const int32_t *__restrict__ active, int64_t nAct, int nbx, int nby, int color,
                            int32_t *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nAct) return;
  const int bid = active[i];
  const int bx = bid % nbx, by = (bid / nbx) % nby, bz = bid / (nbx * nby);
  out[i] = blockColor8(bx, by, bz) == color;
}

// The colour's list starts after the lists of the lower colours, whose lengths the
// earlier scans left in colTot[0..color-1] on the device.
__global__ void kColorScatter(const int32_t *__restrict__ active, const int32_t *__restrict__ flag,
                              const int64_t *__restrict__ off, int64_t nAct, const int64_t *__restrict__ colTot,
                              int color, int32_t *__restrict__ colorBids) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nAct || !flag[i]) return;
  int64_t base = 0;
  for (int c = 0; c < color; c++) base += colTot[c];
  colorBids[base + off[i]] = active[i];
}

}  // namespace msbg

using namespace msbg;

// =====================================================================================
// ABI
// =====================================================================================

static float quant24(float x) {
  // 24-bit particle position quantisation of the domain limits
  // (src/sbg.cpp:262-316 with PARTICLE_QUANT_POS, src/msbgcell.h:74, src/msbgcell.h:138)
  const double scale = ((1 << 24) - 1) * (1.0 / 32768.0);
  return (float)((int32_t)std::floor(scale * x + 0.5) / scale);
}

static bool isPow2(int v) { return v > 0 && (v & (v - 1)) == 0; }

extern "C" int msbg_gpu_create(msbg_gpu_ctx **out, int sx, int sy, int sz, int bsx, int nLevels,
                               int storage, int64_t capacityBlocks) {
  if (!out) return MSBG_GPU_ERR_ARG;
  *out = nullptr;
  if (!isPow2(bsx) || bsx < 8 || bsx > 32 || sx <= 0 || sy <= 0 || sz <= 0 || sx % bsx ||
      sy % bsx || sz % bsx || nLevels < 1 || nLevels > 5 || storage < 0 || storage > 3)
    return MSBG_GPU_ERR_ARG;
  msbg_gpu_ctx *ctx = new msbg_gpu_ctx();
  ctx->sx = sx; ctx->sy = sy; ctx->sz = sz; ctx->bsx = bsx;
  ctx->log2bs = 0;
  while ((1 << ctx->log2bs) < bsx) ctx->log2bs++;
  ctx->nbx = sx / bsx; ctx->nby = sy / bsx; ctx->nbz = sz / bsx;
  ctx->nLevels = nLevels;
  ctx->nBlocks = (int64_t)ctx->nbx * ctx->nby * ctx->nbz;
  ctx->voxPerBlock = (int64_t)bsx * bsx * bsx;
  ctx->capacityLimit = capacityBlocks > 0 ? capacityBlocks : ctx->nBlocks;
  const float beps = 0.005f;
  const int s[3] = {sx, sy, sz};
  for (int k = 0; k < 3; k++) {
    ctx->domMin[k] = quant24(0.0f + beps);
    ctx->domMax[k] = quant24((float)s[k] - beps);
  }
  if (ctx->nBlocks > (int64_t)0x7fffffff) {
    delete ctx;
    return MSBG_GPU_ERR_ARG;
  }
  const size_t nB = (size_t)ctx->nBlocks;
  const int64_t nPart = (ctx->nBlocks + kScanTile - 1) / kScanTile + 1;
  cudaError_t e = cudaSuccess;
#define ALLOC(p, bytes) \
  if (e == cudaSuccess) e = cudaMalloc((void **)&(p), (bytes))
  ALLOC(ctx->dMark, nB * 4);
  ALLOC(ctx->dLevels, nB * 4);
  ALLOC(ctx->dLevelsTmp, nB * 4);
  ALLOC(ctx->dFlags, nB * 2);
  ALLOC(ctx->dSlot, nB * 4);
  ALLOC(ctx->dActive, nB * 4);
  ALLOC(ctx->dColorBids, nB * 4);
  ALLOC(ctx->dScanPartial, (size_t)nPart * 8);
  ALLOC(ctx->dCounters, kNumCounters * 8);
  ALLOC(ctx->dStatus, 16);
#undef ALLOC
  if (e == cudaSuccess) e = cudaMallocHost((void **)&ctx->hCounters, kNumCounters * 8);
  if (e == cudaSuccess) e = cudaMallocHost((void **)&ctx->hSmall, kSmallReadBytes);
  if (e == cudaSuccess) {
    // per-call scratch (splat lists, list copies) comes from the device's
    // stream-ordered pool: keep what it has allocated for the next call instead of
    // returning it at every synchronization (a property of this process's pool)
    int dev = 0;
    cudaMemPool_t pool;
    uint64_t keep = ~0ull;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetDefaultMemPool(&pool, dev);
    if (e == cudaSuccess) e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  for (int i = 0; i < kMaxEvents && e == cudaSuccess; i++) e = cudaEventCreate(&ctx->ev[i]);
  for (int i = 0; i < 8 && e == cudaSuccess; i++) e = cudaEventCreate(&ctx->stageEv[i]);
  if (e == cudaSuccess) e = cudaMemset(ctx->dMark, 0, nB * 4);
  if (e == cudaSuccess) e = cudaMemset(ctx->dCounters, 0, kNumCounters * 8);
  if (e == cudaSuccess) e = cudaMemset(ctx->dStatus, 0, 16);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    msbg_gpu_destroy(ctx);
    return e == cudaErrorMemoryAllocation ? MSBG_GPU_ERR_NOMEM : MSBG_GPU_ERR_CUDA;
  }
  ctx->ch[0].exists = true;
  ctx->ch[0].storage = storage;
  *out = ctx;
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_destroy(msbg_gpu_ctx *ctx) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  cudaStreamSynchronize(ctx->stream);
  cudaFree(ctx->dMark); cudaFree(ctx->dLevels); cudaFree(ctx->dLevelsTmp); cudaFree(ctx->dFlags);
  cudaFree(ctx->dSlot); cudaFree(ctx->dActive); cudaFree(ctx->dColorBids);
  if (ctx->dListMark) cudaFree(ctx->dListMark);
  if (ctx->dListBids) cudaFree(ctx->dListBids);
  cudaFree(ctx->dScanPartial); cudaFree(ctx->dCounters); cudaFree(ctx->dStatus);
  if (ctx->hCounters) cudaFreeHost(ctx->hCounters);
  if (ctx->hSmall) cudaFreeHost(ctx->hSmall);
  for (auto &c : ctx->ch) {
    if (c.d) cudaFree(c.d);
    if (c.cache) cudaFree(c.cache);
    for (auto &gr : c.sweepGraphs) cudaGraphExecDestroy(gr.exec);
    c.sweepGraphs.clear();
  }
  if (ctx->dTmpSlab) cudaFree(ctx->dTmpSlab);
  if (ctx->dPts) cudaFree(ctx->dPts);
  msbg::batchFree(ctx->batch);
  msbg::levelChannelsFree(ctx->levelCh);
  msbg::warmNetFree(ctx->warmnet);
  msbg::poissonFree(ctx->poisson);
  for (auto &ev : ctx->ev) if (ev) cudaEventDestroy(ev);
  for (auto &ev : ctx->stageEv) if (ev) cudaEventDestroy(ev);
  for (auto &ev : ctx->copyEv) if (ev) cudaEventDestroy(ev);
  if (ctx->copyStream) {
    cudaStreamSynchronize(ctx->copyStream);
    cudaStreamDestroy(ctx->copyStream);
  }
  if (ctx->captureStream) cudaStreamDestroy(ctx->captureStream);
  for (cudaStream_t st : {ctx->h2dStream, ctx->d2hStream})
    if (st) {
      cudaStreamSynchronize(st);
      cudaStreamDestroy(st);
    }
  for (int i = 0; i < 2; i++) {
    if (ctx->dPtsQ[i]) cudaFree(ctx->dPtsQ[i]);
    if (ctx->ptsQReady[i]) cudaEventDestroy(ctx->ptsQReady[i]);
    if (ctx->ptsQFree[i]) cudaEventDestroy(ctx->ptsQFree[i]);
  }
  if (ctx->dStageOut) cudaFree(ctx->dStageOut);
  if (ctx->stageOutReady) cudaEventDestroy(ctx->stageOutReady);
  if (ctx->stageOutFree) cudaEventDestroy(ctx->stageOutFree);
  delete ctx;
  return MSBG_GPU_OK;
}

extern "C" const char *msbg_gpu_last_error(const msbg_gpu_ctx *ctx) {
  return ctx ? ctx->err.c_str() : "null context";
}

extern "C" int msbg_gpu_set_stream(msbg_gpu_ctx *ctx, void *stream) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  ctx->stream = (cudaStream_t)stream;
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_synchronize(msbg_gpu_ctx *ctx) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_channel_create(msbg_gpu_ctx *ctx, int chan, int storage) {
  if (!ctx || chan < 0 || chan >= kMaxChannels || storage < 0 || storage > 3)
    return MSBG_GPU_ERR_ARG;
  Channel &c = ctx->ch[chan];
  if (c.exists && c.storage != storage && c.d) {
    MSBG_CUDA(ctx, cudaFree(c.d));
    c.d = nullptr;
    c.capBlocks = 0;
  }
  c.exists = true;
  c.storage = storage;
  if (ctx->layoutValid && ctx->nActive > 0 && c.capBlocks < (size_t)ctx->nActive) {
    if (c.d) MSBG_CUDA(ctx, cudaFree(c.d));
    c.d = nullptr;
    MSBG_CUDA(ctx, cudaMalloc(&c.d, (size_t)ctx->nActive * ctx->voxPerBlock * storageBytes(storage)));
    c.capBlocks = (size_t)ctx->nActive;
  }
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_mark_points(msbg_gpu_ctx *ctx, const float *dPts, int64_t n, float rScan) {
  if (!ctx || (n > 0 && !dPts) || n < 0 || !(rScan >= 0)) return MSBG_GPU_ERR_ARG;
  GridGeom g{ctx->sx, ctx->sy, ctx->sz, ctx->nbx, ctx->nby, ctx->nbz, ctx->log2bs,
             {ctx->domMin[0], ctx->domMin[1], ctx->domMin[2]},
             {ctx->domMax[0], ctx->domMax[1], ctx->domMax[2]}};
  const float rScanBsx = rScan / (float)ctx->bsx;
  MSBG_CUDA(ctx, cudaMemsetAsync(ctx->dCounters, 0, 8, ctx->stream));
  if (n > 0)
    MSBG_LAUNCH(ctx, kMarkPoints, gridFor(n, 256), 256, 0, dPts, n, g, rScanBsx, ctx->dMark,
                (unsigned long long *)ctx->dCounters);
  ctx->layoutValid = false;
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_levels_from_marks(msbg_gpu_ctx *ctx) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  MSBG_LAUNCH(ctx, kLevelsFromMarks, gridFor(ctx->nBlocks, 256), 256, 0, ctx->dMark, ctx->nBlocks,
              ctx->nLevels - 1, ctx->dLevels);
  // marks are consumed: clear them for the next layout
  MSBG_CUDA(ctx, cudaMemsetAsync(ctx->dMark, 0, (size_t)ctx->nBlocks * 4, ctx->stream));
  ctx->layoutValid = false;
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_levels_from_bands(msbg_gpu_ctx *ctx, const float *dPts, int64_t n,
                                          const float *hBands, int nBands) {
  if (!ctx || !hBands || nBands < 1 || nBands > ctx->nLevels - 1 || n < 0 || (n && !dPts))
    return MSBG_GPU_ERR_ARG;
  GridGeom g{ctx->sx, ctx->sy, ctx->sz, ctx->nbx, ctx->nby, ctx->nbz, ctx->log2bs,
             {ctx->domMin[0], ctx->domMin[1], ctx->domMin[2]},
             {ctx->domMax[0], ctx->domMax[1], ctx->domMax[2]}};
  MSBG_LAUNCH(ctx, kFillInt, gridFor(ctx->nBlocks, 256), 256, 0, ctx->dLevels, ctx->nBlocks,
              ctx->nLevels - 1);
  MSBG_CUDA(ctx, cudaMemsetAsync(ctx->dCounters, 0, 8, ctx->stream));
  if (n > 0) {
    // count valid points once (marks buffer is reused as scratch and cleared)
    MSBG_LAUNCH(ctx, kMarkPoints, gridFor(n, 256), 256, 0, dPts, n, g, 0.0f, ctx->dMark,
                (unsigned long long *)ctx->dCounters);
    MSBG_CUDA(ctx, cudaMemsetAsync(ctx->dMark, 0, (size_t)ctx->nBlocks * 4, ctx->stream));
    for (int l = nBands - 1; l >= 0; l--) {
      if (!(hBands[l] >= 0)) return fail(ctx, MSBG_GPU_ERR_ARG, "band %d invalid", l);
      MSBG_LAUNCH(ctx, kBandLevels, gridFor(n, 256), 256, 0, dPts, n, g, hBands[l] / (float)ctx->bsx, l,
                  ctx->dLevels);
    }
  }
  ctx->layoutValid = false;
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_set_levels(msbg_gpu_ctx *ctx, const int32_t *hLevels) {
  if (!ctx || !hLevels) return MSBG_GPU_ERR_ARG;
  for (int64_t i = 0; i < ctx->nBlocks; i++)
    if (hLevels[i] < 0 || hLevels[i] >= ctx->nLevels)
      return fail(ctx, MSBG_GPU_ERR_ARG, "level %d of block %lld out of range", hLevels[i],
                  (long long)i);
  MSBG_CUDA(ctx, cudaMemcpyAsync(ctx->dLevels, hLevels, (size_t)ctx->nBlocks * 4,
                                 cudaMemcpyHostToDevice, ctx->stream));
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->layoutValid = false;
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_regularize_refinement_map(msbg_gpu_ctx *ctx) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  for (int ll = 1; ll <= ctx->nLevels - 2; ll++) {
    MSBG_LAUNCH(ctx, kRegularizePass, gridFor(ctx->nBlocks, 256), 256, 0, ctx->dLevels,
                ctx->dLevelsTmp, ctx->nbx, ctx->nby, ctx->nbz, ctx->nLevels, ll);
    std::swap(ctx->dLevels, ctx->dLevelsTmp);
  }
  ctx->layoutValid = false;
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_set_refinement_map(msbg_gpu_ctx *ctx, double fillValue) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  const int64_t nB = ctx->nBlocks;
  int64_t *dCnt = ctx->dCounters;
  MSBG_CUDA(ctx, cudaMemsetAsync(dCnt + 4, 0, 8 * 8, ctx->stream));
  MSBG_LAUNCH(ctx, kBlockFlags, gridFor(nB, 256), 256, 0, ctx->dLevels, ctx->dFlags, ctx->nbx,
              ctx->nby, ctx->nbz, (unsigned long long *)(dCnt + 4));
  // slot assignment: scan of (level == 0) over all blocks; dLevelsTmp holds the flags,
  // the int64 offsets go to the tmp slab.
  int rc = ensureTmpSlab(ctx, (size_t)nB * 8);
  if (rc) return rc;
  int64_t *dOff = (int64_t *)ctx->dTmpSlab;
  MSBG_LAUNCH(ctx, kValueFlags, gridFor(nB, 256), 256, 0, ctx->dLevels, nB, ctx->dLevelsTmp);
  rc = exclusiveScanFlags(ctx, ctx->dLevelsTmp, nB, dOff, dCnt + 2);
  if (rc) return rc;
  MSBG_LAUNCH(ctx, kAssignSlots, gridFor(nB, 256), 256, 0, ctx->dLevels, dOff, nB, ctx->dSlot,
              ctx->dActive);
  if ((rc = readSmall(ctx, ctx->hCounters, dCnt, 16 * 8))) return rc;  // 0..15
  const int64_t nAct = ctx->hCounters[2];
  for (int l = 0; l < 8; l++) ctx->blocksPerLevel[l] = ctx->hCounters[4 + l];
  ctx->nActParticles = ctx->hCounters[0];
  if (nAct > ctx->capacityLimit)
    return fail(ctx, MSBG_GPU_ERR_CAPACITY, "%lld value blocks exceed the pool capacity %lld",
                (long long)nAct, (long long)ctx->capacityLimit);
  // 8-color lists: stable compaction of the active list per color; each colour's
  // length stays on the device (counters kColorTot..+7), where the next colours'
  // scatters read their start, and all eight are read back once.
  int32_t *dFlag = ctx->dLevelsTmp;
  int64_t *dColTot = dCnt + kColorTot;
  if (nAct > 0) {
    for (int c = 0; c < 8; c++) {
      MSBG_LAUNCH(ctx, kColorFlags, gridFor(nAct, 256), 256, 0, ctx->dActive, nAct, ctx->nbx, ctx->nby,
                  c, dFlag);
      rc = exclusiveScanFlags(ctx, dFlag, nAct, dOff, dColTot + c);
      if (rc) return rc;
      MSBG_LAUNCH(ctx, kColorScatter, gridFor(nAct, 256), 256, 0, ctx->dActive, dFlag, dOff, nAct, dColTot,
                  c, ctx->dColorBids);
    }
    if ((rc = readSmall(ctx, ctx->hCounters + kColorTot, dColTot, 8 * 8))) return rc;
  }
  int32_t base = 0;
  for (int c = 0; c < 8; c++) {
    ctx->colorStart[c] = base;
    if (nAct > 0) base += (int32_t)ctx->hCounters[kColorTot + c];
  }
  ctx->colorStart[8] = base;
  ctx->nActive = nAct;
  ctx->layoutStamp++;
  // block pool: (re)size every channel slab to the value-block count
  for (auto &c : ctx->ch) {
    if (!c.exists) continue;
    if (c.capBlocks < (size_t)nAct || !c.d) {
      if (c.d) MSBG_CUDA(ctx, cudaFree(c.d));
      c.d = nullptr;
      c.capBlocks = 0;
      const size_t want = (size_t)(nAct > 0 ? nAct : 1);
      MSBG_CUDA(ctx, cudaMalloc(&c.d, want * ctx->voxPerBlock * storageBytes(c.storage)));
      c.capBlocks = want;
    }
  }
  ctx->layoutValid = true;
  for (int i = 0; i < kMaxChannels; i++) {
    if (!ctx->ch[i].exists) continue;
    rc = fillChannel(ctx, i, fillValue);
    if (rc) return rc;
  }
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_get_info(msbg_gpu_ctx *ctx, msbg_gpu_info *info) {
  if (!ctx || !info) return MSBG_GPU_ERR_ARG;
  MSBG_CUDA(ctx, cudaMemcpyAsync(ctx->hCounters, ctx->dCounters, 16 * 8, cudaMemcpyDeviceToHost,
                                 ctx->stream));
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  memset(info, 0, sizeof(*info));
  info->sx = ctx->sx; info->sy = ctx->sy; info->sz = ctx->sz; info->bsx = ctx->bsx;
  info->nbx = ctx->nbx; info->nby = ctx->nby; info->nbz = ctx->nbz;
  info->nLevels = ctx->nLevels;
  info->nBlocks = ctx->nBlocks;
  info->nActive = ctx->layoutValid ? ctx->nActive : 0;
  info->capacityBlocks = ctx->capacityLimit;
  for (int l = 0; l < 8; l++) info->blocksPerLevel[l] = ctx->blocksPerLevel[l];
  for (int c = 0; c < 8; c++) info->colorCount[c] = ctx->colorStart[c + 1] - ctx->colorStart[c];
  info->nActParticles = ctx->hCounters[0];
  info->nAborted = ctx->hCounters[1];
  return MSBG_GPU_OK;
}

static int needLayout(msbg_gpu_ctx *ctx) {
  if (!ctx->layoutValid) return fail(ctx, MSBG_GPU_ERR_STATE, "no block layout: call set_refinement_map");
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_get_levels(msbg_gpu_ctx *ctx, int8_t *hLevels) {
  if (!ctx || !hLevels) return MSBG_GPU_ERR_ARG;
  int32_t *tmp = nullptr;
  MSBG_CUDA(ctx, cudaMallocHost((void **)&tmp, (size_t)ctx->nBlocks * 4));
  cudaError_t e = cudaMemcpyAsync(tmp, ctx->dLevels, (size_t)ctx->nBlocks * 4, cudaMemcpyDeviceToHost,
                                  ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e == cudaSuccess)
    for (int64_t i = 0; i < ctx->nBlocks; i++) hLevels[i] = (int8_t)tmp[i];
  cudaFreeHost(tmp);
  if (e != cudaSuccess) return cudaFail(ctx, e, "get_levels");
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_get_flags(msbg_gpu_ctx *ctx, uint16_t *hFlags) {
  if (!ctx || !hFlags) return MSBG_GPU_ERR_ARG;
  int rc = needLayout(ctx);
  if (rc) return rc;
  MSBG_CUDA(ctx, cudaMemcpyAsync(hFlags, ctx->dFlags, (size_t)ctx->nBlocks * 2, cudaMemcpyDeviceToHost,
                                 ctx->stream));
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_get_active_blocks(msbg_gpu_ctx *ctx, int32_t *hBids, int64_t cap, int64_t *n) {
  if (!ctx || !n) return MSBG_GPU_ERR_ARG;
  int rc = needLayout(ctx);
  if (rc) return rc;
  *n = ctx->nActive;
  if (!hBids) return MSBG_GPU_OK;
  if (cap < ctx->nActive) return fail(ctx, MSBG_GPU_ERR_ARG, "buffer too small");
  if (ctx->nActive)
    MSBG_CUDA(ctx, cudaMemcpyAsync(hBids, ctx->dActive, (size_t)ctx->nActive * 4, cudaMemcpyDeviceToHost,
                                   ctx->stream));
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_get_slots(msbg_gpu_ctx *ctx, int32_t *hSlots) {
  if (!ctx || !hSlots) return MSBG_GPU_ERR_ARG;
  int rc = needLayout(ctx);
  if (rc) return rc;
  MSBG_CUDA(ctx, cudaMemcpyAsync(hSlots, ctx->dSlot, (size_t)ctx->nBlocks * 4, cudaMemcpyDeviceToHost,
                                 ctx->stream));
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return MSBG_GPU_OK;
}

static int checkChan(msbg_gpu_ctx *ctx, int chan) {
  if (chan < 0 || chan >= kMaxChannels || !ctx->ch[chan].exists)
    return fail(ctx, MSBG_GPU_ERR_ARG, "channel %d does not exist", chan);
  return needLayout(ctx);
}

extern "C" int msbg_gpu_upload_payload(msbg_gpu_ctx *ctx, int chan, const void *hData) {
  if (!ctx || !hData) return MSBG_GPU_ERR_ARG;
  int rc = checkChan(ctx, chan);
  if (rc) return rc;
  const size_t bytes = (size_t)ctx->nActive * ctx->voxPerBlock * storageBytes(ctx->ch[chan].storage);
  if (bytes) return copyAsyncSplit(ctx, ctx->ch[chan].d, hData, bytes, cudaMemcpyHostToDevice);
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_download_payload(msbg_gpu_ctx *ctx, int chan, void *hData) {
  if (!ctx || !hData) return MSBG_GPU_ERR_ARG;
  int rc = checkChan(ctx, chan);
  if (rc) return rc;
  const size_t bytes = (size_t)ctx->nActive * ctx->voxPerBlock * storageBytes(ctx->ch[chan].storage);
  if (bytes && (rc = copyAsyncSplit(ctx, hData, ctx->ch[chan].d, bytes, cudaMemcpyDeviceToHost))) return rc;
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_payload_ptr(msbg_gpu_ctx *ctx, int chan, void **dPtr) {
  if (!ctx || !dPtr) return MSBG_GPU_ERR_ARG;
  int rc = checkChan(ctx, chan);
  if (rc) return rc;
  *dPtr = ctx->ch[chan].d;
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_fill(msbg_gpu_ctx *ctx, int chan, double value) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  int rc = checkChan(ctx, chan);
  if (rc) return rc;
  return fillChannel(ctx, chan, value);
}

extern "C" int msbg_gpu_splat(msbg_gpu_ctx *ctx, const float *dPts, int64_t n, float rParticle,
                              float nbDist) {
  if (!ctx || n < 0 || (n && !dPts) || !(rParticle > 0) || !(nbDist >= 0)) return MSBG_GPU_ERR_ARG;
  int rc = checkChan(ctx, 0);
  if (rc) return rc;
  if ((double)(rParticle + nbDist) * 2.0 + 1.0 > (double)ctx->bsx)
    return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED, "splat box wider than a block");
  return splatRun(ctx, dPts, n, rParticle, nbDist);
}

extern "C" int msbg_gpu_particles_per_block(msbg_gpu_ctx *ctx, const float *dPts, int64_t n, int64_t *dOffsets,
                                            int32_t *dIndex, int64_t *hCount) {
  if (!ctx || n < 0 || (n > 0 && (!dPts || !dIndex)) || !dOffsets || !hCount) return MSBG_GPU_ERR_ARG;
  if (n > (int64_t)0x7fffffff) return fail(ctx, MSBG_GPU_ERR_ARG, "particles_per_block: %lld points", (long long)n);
  return particlesPerBlockRun(ctx, dPts, n, dOffsets, dIndex, hCount);
}

extern "C" int msbg_gpu_splat_finalize(msbg_gpu_ctx *ctx, float rParticle, float nbDist) {
  if (!ctx || !(rParticle > 0) || !(nbDist >= 0)) return MSBG_GPU_ERR_ARG;
  int rc = checkChan(ctx, 0);
  if (rc) return rc;
  return splatFinalizeRun(ctx, rParticle, nbDist);
}

extern "C" int msbg_gpu_apply_channel_pde_fast(msbg_gpu_ctx *ctx, int chPhi, int chTmp, int chTmp2,
                                               const int32_t *dBlockList, int64_t nBlockList, int laplTyp,
                                               int doConstrZeroOne, float densThr, float densThrTol1,
                                               float densThrTol2, int numIter, float gridSpacing, float timeStep,
                                               float velMagThr, const void *msbgVel, float lambda,
                                               float lambdaSDF, float taubinStrength, float redist,
                                               float anisDiffAlpha, int veldepOn, const float *veldepFit,
                                               int visOpt, int variant) {
  (void)chTmp; (void)chTmp2; (void)veldepFit; (void)visOpt;  // scratch is the library's own; no display
  if (!ctx || nBlockList < 0 || (nBlockList > 0 && !dBlockList)) return MSBG_GPU_ERR_ARG;
  if (numIter < 0)  // the reference's compressed-range mode (src/msbg4.cpp:136-141)
    return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED, "negative numIter (compressed value range)");
  if (gridSpacing != 1.0f)  // the reference asserts a unit spacing (src/msbg4.cpp:326)
    return fail(ctx, MSBG_GPU_ERR_ARG, "gridSpacing must be 1");
  // lambda is forced to 0 by the reference itself (src/msbg4.cpp:164); lambdaSDF serves it
  (void)lambda; (void)lambdaSDF;
  if (densThr > 0.0f || densThrTol1 > 0.0f || densThrTol2 > 0.0f || velMagThr != 0.0f || msbgVel || veldepOn ||
      taubinStrength != 0.0f || redist > 0.0f)
    return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED,
                "density constraints, velocity terms, Taubin smoothing and redistancing are not on this path");
  int rc = checkChan(ctx, chPhi);
  if (rc) return rc;
  return pdeRun(ctx, chPhi, laplTyp, doConstrZeroOne, numIter, timeStep, anisDiffAlpha, variant, dBlockList,
                nBlockList);
}

extern "C" int msbg_gpu_surface_job(msbg_gpu_ctx *ctx, const float *hPts, int64_t n, float rParticle,
                                    float nbDist, const float *hBands, int nBands, int laplTyp,
                                    int numIter, float timeStep, int variant, void *hOut,
                                    size_t hOutCap, int64_t *nActiveOut) {
  if (!ctx || n < 0 || (n && !hPts)) return MSBG_GPU_ERR_ARG;
  // stage boundaries on the stream: start, points uploaded, layout built, splat,
  // finalize, sweeps, payload downloaded
  ctx->stageCount = 0;
  auto stage = [&]() -> int {
    MSBG_CUDA(ctx, cudaEventRecord(ctx->stageEv[ctx->stageCount], ctx->stream));
    ctx->stageCount++;
    return MSBG_GPU_OK;
  };
  if (stage()) return MSBG_GPU_ERR_CUDA;
  if (ctx->ptsCap < n) {
    if (ctx->dPts) MSBG_CUDA(ctx, cudaFree(ctx->dPts));
    ctx->dPts = nullptr;
    ctx->ptsCap = 0;
    MSBG_CUDA(ctx, cudaMalloc(&ctx->dPts, (size_t)n * 12));
    ctx->ptsCap = n;
  }
  if (n) {
    int r = copyAsyncSplit(ctx, ctx->dPts, hPts, (size_t)n * 12, cudaMemcpyHostToDevice);
    if (r) return r;
  }
  int rc = stage();
  if (!rc) {
    if (nBands > 0) {
      rc = msbg_gpu_levels_from_bands(ctx, ctx->dPts, n, hBands, nBands);
    } else {
      rc = msbg_gpu_mark_points(ctx, ctx->dPts, n, rParticle + nbDist);
      if (!rc) rc = msbg_gpu_levels_from_marks(ctx);
    }
  }
  if (!rc) rc = msbg_gpu_regularize_refinement_map(ctx);
  if (!rc) rc = msbg_gpu_set_refinement_map(ctx, 1.0);
  if (!rc) rc = stage();
  if (!rc) rc = msbg_gpu_splat(ctx, ctx->dPts, n, rParticle, nbDist);
  if (!rc) rc = stage();
  if (!rc) rc = msbg_gpu_splat_finalize(ctx, rParticle, nbDist);
  if (!rc) rc = stage();
  if (!rc && numIter > 0)
    rc = pdeRun(ctx, 0, laplTyp, 1, numIter, timeStep, 0.0f, variant);
  if (!rc) rc = stage();
  if (rc) return rc;
  if (nActiveOut) *nActiveOut = ctx->nActive;
  if (hOut) {
    const size_t bytes = (size_t)ctx->nActive * ctx->voxPerBlock * storageBytes(ctx->ch[0].storage);
    if (bytes > hOutCap) return fail(ctx, MSBG_GPU_ERR_ARG, "output buffer too small (%zu < %zu)", hOutCap, bytes);
    if ((rc = copyAsyncSplit(ctx, hOut, ctx->ch[0].d, bytes, cudaMemcpyDeviceToHost))) return rc;
  }
  if ((rc = stage())) return rc;
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return MSBG_GPU_OK;
}

// The streaming form: the same job, queued.  Job k's points go up on h2dStream into one of
// two buffers (the upload waits for the splat of job k-2, the buffer's last reader); the
// compute stream waits for them and runs the layout, splat, finalise and sweeps (the host
// reads back the block count and the sweeps' status, so the call returns only when the
// compute stream has got that far), then copies the result to a device staging buffer
// (after the previous download has left it); d2hStream downloads it while the next job
// computes.  Those read-backs go through readSmall, not a copy engine: a copy would queue
// behind the previous job's download there and hold the next job's compute back by it.
extern "C" int msbg_gpu_surface_job_submit(msbg_gpu_ctx *ctx, const float *hPts, int64_t n, float rParticle,
                                           float nbDist, const float *hBands, int nBands, int laplTyp,
                                           int numIter, float timeStep, int variant, void *hOut,
                                           size_t hOutCap, int64_t *nActiveOut) {
  if (!ctx || n < 0 || (n && !hPts)) return MSBG_GPU_ERR_ARG;
  auto event = [&](cudaEvent_t &e) -> int {
    if (!e) MSBG_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return MSBG_GPU_OK;
  };
  for (cudaStream_t *st : {&ctx->h2dStream, &ctx->d2hStream})
    if (!*st) MSBG_CUDA(ctx, cudaStreamCreateWithFlags(st, cudaStreamNonBlocking));
  const int q = (int)(ctx->jobSeq & 1);
  int rc;
  if ((rc = event(ctx->ptsQReady[q])) || (rc = event(ctx->ptsQFree[q])) || (rc = event(ctx->stageOutReady)) ||
      (rc = event(ctx->stageOutFree)))
    return rc;
  if (ctx->ptsQCap[q] < n) {
    MSBG_CUDA(ctx, cudaDeviceSynchronize());  // the buffer may still be read by an earlier job
    if (ctx->dPtsQ[q]) MSBG_CUDA(ctx, cudaFree(ctx->dPtsQ[q]));
    ctx->dPtsQ[q] = nullptr;
    ctx->ptsQCap[q] = 0;
    MSBG_CUDA(ctx, cudaMalloc(&ctx->dPtsQ[q], (size_t)(n ? n : 1) * 12));
    ctx->ptsQCap[q] = n;
  }
  float *dPts = ctx->dPtsQ[q];
  if (n) {
    MSBG_CUDA(ctx, cudaStreamWaitEvent(ctx->h2dStream, ctx->ptsQFree[q], 0));
    MSBG_CUDA(ctx, cudaMemcpyAsync(dPts, hPts, (size_t)n * 12, cudaMemcpyHostToDevice, ctx->h2dStream));
  }
  MSBG_CUDA(ctx, cudaEventRecord(ctx->ptsQReady[q], ctx->h2dStream));
  MSBG_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->ptsQReady[q], 0));
  ctx->jobSeq++;
  if (nBands > 0) {
    rc = msbg_gpu_levels_from_bands(ctx, dPts, n, hBands, nBands);
  } else {
    rc = msbg_gpu_mark_points(ctx, dPts, n, rParticle + nbDist);
    if (!rc) rc = msbg_gpu_levels_from_marks(ctx);
  }
  if (!rc) rc = msbg_gpu_regularize_refinement_map(ctx);
  if (!rc) rc = msbg_gpu_set_refinement_map(ctx, 1.0);
  if (!rc) rc = msbg_gpu_splat(ctx, dPts, n, rParticle, nbDist);
  if (rc) return rc;
  MSBG_CUDA(ctx, cudaEventRecord(ctx->ptsQFree[q], ctx->stream));
  if ((rc = msbg_gpu_splat_finalize(ctx, rParticle, nbDist))) return rc;
  if (numIter > 0 && (rc = pdeRun(ctx, 0, laplTyp, 1, numIter, timeStep, 0.0f, variant))) return rc;
  if (nActiveOut) *nActiveOut = ctx->nActive;
  if (hOut) {
    const size_t bytes = (size_t)ctx->nActive * ctx->voxPerBlock * storageBytes(ctx->ch[0].storage);
    if (bytes > hOutCap) return fail(ctx, MSBG_GPU_ERR_ARG, "output buffer too small (%zu < %zu)", hOutCap, bytes);
    if (ctx->stageOutCap < bytes) {
      MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->d2hStream));  // the last download reads it
      if (ctx->dStageOut) MSBG_CUDA(ctx, cudaFree(ctx->dStageOut));
      ctx->dStageOut = nullptr;
      ctx->stageOutCap = 0;
      MSBG_CUDA(ctx, cudaMalloc(&ctx->dStageOut, bytes));
      ctx->stageOutCap = bytes;
    }
    MSBG_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->stageOutFree, 0));
    if (bytes)
      MSBG_CUDA(ctx, cudaMemcpyAsync(ctx->dStageOut, ctx->ch[0].d, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    MSBG_CUDA(ctx, cudaEventRecord(ctx->stageOutReady, ctx->stream));
    MSBG_CUDA(ctx, cudaStreamWaitEvent(ctx->d2hStream, ctx->stageOutReady, 0));
    if (bytes) MSBG_CUDA(ctx, cudaMemcpyAsync(hOut, ctx->dStageOut, bytes, cudaMemcpyDeviceToHost, ctx->d2hStream));
    MSBG_CUDA(ctx, cudaEventRecord(ctx->stageOutFree, ctx->d2hStream));
  }
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_surface_job_wait(msbg_gpu_ctx *ctx) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (ctx->h2dStream) MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->h2dStream));
  if (ctx->d2hStream) MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->d2hStream));
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_surface_job_stages(msbg_gpu_ctx *ctx, float *msOut, int cap, int *nOut) {
  if (!ctx || !msOut || cap < 0) return MSBG_GPU_ERR_ARG;
  const int n = ctx->stageCount > 1 ? ctx->stageCount - 1 : 0;
  for (int i = 0; i < n && i < cap; i++)
    MSBG_CUDA(ctx, cudaEventElapsedTime(&msOut[i], ctx->stageEv[i], ctx->stageEv[i + 1]));
  if (nOut) *nOut = n;
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_event_record(msbg_gpu_ctx *ctx, int slot) {
  if (!ctx || slot < 0 || slot >= kMaxEvents) return MSBG_GPU_ERR_ARG;
  MSBG_CUDA(ctx, cudaEventRecord(ctx->ev[slot], ctx->stream));
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_event_elapsed(msbg_gpu_ctx *ctx, int a, int b, float *ms) {
  if (!ctx || !ms || a < 0 || b < 0 || a >= kMaxEvents || b >= kMaxEvents) return MSBG_GPU_ERR_ARG;
  MSBG_CUDA(ctx, cudaEventSynchronize(ctx->ev[b]));
  MSBG_CUDA(ctx, cudaEventElapsedTime(ms, ctx->ev[a], ctx->ev[b]));
  return MSBG_GPU_OK;
}

extern "C" int64_t msbg_gpu_launch_count(const msbg_gpu_ctx *ctx) { return ctx ? ctx->launches : -1; }

extern "C" int msbg_gpu_host_alloc(void **p, size_t bytes) {
  if (!p) return MSBG_GPU_ERR_ARG;
  return cudaMallocHost(p, bytes) == cudaSuccess ? MSBG_GPU_OK : MSBG_GPU_ERR_NOMEM;
}
extern "C" int msbg_gpu_host_free(void *p) {
  return cudaFreeHost(p) == cudaSuccess ? MSBG_GPU_OK : MSBG_GPU_ERR_CUDA;
}
extern "C" int msbg_gpu_device_alloc(void **p, size_t bytes) {
  if (!p) return MSBG_GPU_ERR_ARG;
  return cudaMalloc(p, bytes) == cudaSuccess ? MSBG_GPU_OK : MSBG_GPU_ERR_NOMEM;
}
extern "C" int msbg_gpu_device_free(void *p) {
  return cudaFree(p) == cudaSuccess ? MSBG_GPU_OK : MSBG_GPU_ERR_CUDA;
}
extern "C" int msbg_gpu_copy_h2d(msbg_gpu_ctx *ctx, void *d, const void *h, size_t bytes) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  MSBG_CUDA(ctx, cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, ctx->stream));
  return MSBG_GPU_OK;
}
extern "C" int msbg_gpu_copy_d2d(msbg_gpu_ctx *ctx, void *dd, const void *ds, size_t bytes) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  MSBG_CUDA(ctx, cudaMemcpyAsync(dd, ds, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
  return MSBG_GPU_OK;
}
extern "C" int msbg_gpu_copy_d2h(msbg_gpu_ctx *ctx, void *h, const void *d, size_t bytes) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  MSBG_CUDA(ctx, cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return MSBG_GPU_OK;
}

// ---------------------------------------------------------------------------------
// diagnostics: the bounded-wait failure path without a GPU fault
// ---------------------------------------------------------------------------------
namespace msbg {
__global__ void kDiagWait(int polls, int *__restrict__ status) {
  __shared__ __align__(8) uint64_t bar;
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(&bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(a) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  bool done = false;
  for (int it = 0; it < polls && !done; it++) {  // phase 0 never completes: no arrival
    uint32_t ok;
    asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\nselp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(ok)
                 : "r"(a)
                 : "memory");
    done = ok != 0;
  }
  if (!__syncthreads_and(done) && threadIdx.x == 0) atomicOr(status, 16);
}
}  // namespace msbg

extern "C" int msbg_gpu_diag_wait_timeout(msbg_gpu_ctx *ctx, int polls) {
  if (!ctx || polls < 1 || polls > (1 << 20)) return MSBG_GPU_ERR_ARG;
  MSBG_LAUNCH(ctx, kDiagWait, 1, 32, 0, polls, ctx->dStatus);
  int st = 0;
  MSBG_CUDA(ctx, cudaMemcpyAsync(&st, ctx->dStatus, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (st) {
    MSBG_CUDA(ctx, cudaMemsetAsync(ctx->dStatus, 0, sizeof(int), ctx->stream));
    MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return fail(ctx, MSBG_GPU_ERR_TIMEOUT, "a bounded device wait timed out (status bits %d)", st);
  }
  return MSBG_GPU_OK;
}
