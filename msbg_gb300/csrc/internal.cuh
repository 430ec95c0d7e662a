// Internal declarations of the msbg_gpu library (sm_103a).  Not part of the ABI.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <string>
#include <vector>

#include "msbg_gpu.h"

namespace msbg {

struct PoissonState;
struct WarmNetState;
struct BatchState;
struct LevelChannels;
void poissonFree(PoissonState *ps);
void levelChannelsFree(LevelChannels *lc);
void warmNetFree(WarmNetState *w);
void batchFree(BatchState *b);
constexpr int kMaxChannels = 64;
// device counters of a context (int64): 0 nActParticles, 1 nAborted, 2 nActive,
// 3 scratch, 4..11 blocks per level (5, 6 reused as scan totals by the solver),
// 16..23 value blocks per 8-colour class
constexpr int kColorTot = 16;
constexpr int kNumCounters = 32;
constexpr int kMaxEvents = 16;

// A captured sequence of launches and the bytes it was captured from (kernel,
// arguments, grid): replayed while a call presents the same bytes.
struct CachedGraph {
  std::vector<unsigned char> key;
  cudaGraphExec_t exec = nullptr;
};

struct Channel {
  bool exists = false;
  int storage = MSBG_GPU_F32;
  void *d = nullptr;      // [capacity][bs^3]
  size_t capBlocks = 0;   // blocks the slab can hold
  void *cache = nullptr;  // x-face + corner-column cache of the colored sweeps
  size_t cacheBytes = 0;
  std::vector<CachedGraph> sweepGraphs;  // the colour passes of recent sweep calls (most recent last)
};

}  // namespace msbg

struct msbg_gpu_ctx {
  // geometry
  int sx, sy, sz, bsx, log2bs, nbx, nby, nbz, nLevels;
  int64_t nBlocks;
  int64_t voxPerBlock;
  float domMin[3], domMax[3];
  int64_t capacityLimit;

  cudaStream_t stream = nullptr;
  cudaEvent_t ev[msbg::kMaxEvents] = {};
  cudaEvent_t stageEv[8] = {};   // msbg_gpu_surface_job: events at its stage boundaries
  cudaStream_t copyStream = nullptr;        // second copy engine for large host transfers
  cudaStream_t captureStream = nullptr;     // stream the sweeps' launch graphs are captured on
  cudaEvent_t copyEv[2] = {};               // fork / join of a split copy
  int stageCount = 0;            // events recorded by the last surface job
  // msbg_gpu_surface_job_submit: points double-buffered and uploaded on h2dStream, the
  // result staged on the device and downloaded on d2hStream while the next job computes
  cudaStream_t h2dStream = nullptr, d2hStream = nullptr;
  float *dPtsQ[2] = {};
  int64_t ptsQCap[2] = {};
  cudaEvent_t ptsQReady[2] = {}, ptsQFree[2] = {};
  void *dStageOut = nullptr;
  size_t stageOutCap = 0;
  cudaEvent_t stageOutReady = nullptr, stageOutFree = nullptr;
  int64_t jobSeq = 0;

  // layout (device)
  int32_t *dMark = nullptr;      // [nBlocks] 0/1 (demo's blockActive as a flag)
  int32_t *dLevels = nullptr;    // [nBlocks]
  int32_t *dLevelsTmp = nullptr; // [nBlocks]
  uint16_t *dFlags = nullptr;    // [nBlocks]
  int32_t *dSlot = nullptr;      // [nBlocks]
  int32_t *dActive = nullptr;    // [nBlocks] ascending bids of value blocks
  int32_t *dColorBids = nullptr; // [nBlocks] value blocks grouped by 8-color class
  int32_t *dListMark = nullptr;  // [nBlocks] sweeps with a block list: listed blocks
  int32_t *dListBids = nullptr;  // [nBlocks] sweeps with a block list: listed value blocks by colour
  int64_t *dScanPartial = nullptr; // scan scratch
  int64_t *dCounters = nullptr;  // [kNumCounters], see kColorTot
  int64_t *hCounters = nullptr;  // pinned mirror
  int64_t *hSmall = nullptr;     // pinned, kSmallReadBytes: target of readSmall
  int *dStatus = nullptr;        // device-side error bits (bounded waits that gave up)
  bool layoutValid = false;
  int64_t nActive = 0;
  int32_t colorStart[9] = {};
  int64_t blocksPerLevel[8] = {};

  // channels
  msbg::Channel ch[msbg::kMaxChannels];
  void *dTmpSlab = nullptr;      // ping-pong / splat staging
  size_t tmpSlabBytes = 0;

  // point staging for the host-buffer entry point
  float *dPts = nullptr;
  int64_t ptsCap = 0;

  int64_t nActParticles = 0, nAborted = 0;
  int64_t launches = 0;
  int64_t layoutStamp = 0;                 // bumped by every set_refinement_map
  msbg::PoissonState *poisson = nullptr;   // solver hierarchy of the current layout
  msbg::WarmNetState *warmnet = nullptr;   // learned warm start (weights, level-1 buffers)
  msbg::BatchState *batch = nullptr;       // batched solves: volumes of the layout, graph
  msbg::LevelChannels *levelCh = nullptr;  // multi-level channels of the halo fill
  int mgPre = 2, mgPost = 2, mgTileIters = 3, mgCoarsestIter = 0;  // multigrid parameters
  float relaxOmega = 6.0f / 7.0f;  // block smoother of msbg_gpu_relax (src/msbg.cpp:814-843)
  int relaxBlockIter = 5;
  std::string err;
};

namespace msbg {

int fail(msbg_gpu_ctx *ctx, int code, const char *fmt, ...);
int cudaFail(msbg_gpu_ctx *ctx, cudaError_t e, const char *what);

#define MSBG_CUDA(ctx, call)                                  \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return msbg::cudaFail(ctx, e_, #call); \
  } while (0)

// Every kernel launch of the library goes through this macro: it counts the
// launch and checks the launch status.
#define MSBG_LAUNCH(ctx, kernel, grid, block, smem, ...)                       \
  do {                                                                         \
    kernel<<<(grid), (block), (smem), (ctx)->stream>>>(__VA_ARGS__);           \
    (ctx)->launches++;                                                         \
    cudaError_t e_ = cudaGetLastError();                                       \
    if (e_ != cudaSuccess) return msbg::cudaFail(ctx, e_, #kernel);            \
  } while (0)

inline size_t storageBytes(int storage) {
  return storage == MSBG_GPU_F32 ? 4 : storage == MSBG_GPU_F64 ? 8 : 2;
}

inline unsigned gridFor(int64_t n, int threads) {
  int64_t g = (n + threads - 1) / threads;
  if (g < 1) g = 1;
  if (g > 0x7fffffff) g = 0x7fffffff;
  return (unsigned)g;
}

// Exclusive scan of int32 flags -> int64 offsets with total in *dTotal (device).
int exclusiveScanFlags(msbg_gpu_ctx *ctx, const int32_t *dIn, int64_t n, int64_t *dOut,
                       int64_t *dTotal);
// The same with caller scratch for the per-tile partial sums (scanPartialCount(n) int64s),
// for inputs longer than the block count.
int exclusiveScanFlagsWith(msbg_gpu_ctx *ctx, const int32_t *dIn, int64_t n, int64_t *dOut,
                           int64_t *dTotal, int64_t *dPartial);
int64_t scanPartialCount(int64_t n);
// Exclusive scan of non-negative int32 counts (n <= nBlocks) -> int64 offsets, total in *dTotal.
int exclusiveScanCounts(msbg_gpu_ctx *ctx, const int32_t *dIn, int64_t n, int64_t *dOut, int64_t *dTotal);

// Host <-> device copy on the context's stream; above 64 MiB the second half goes
// through a second stream, so two copy engines move it (ordered like one copy on
// the context's stream).
int copyAsyncSplit(msbg_gpu_ctx *ctx, void *dst, const void *src, size_t bytes, cudaMemcpyKind kind);

// Read up to kSmallReadBytes (a multiple of 4) of device memory into host memory, ordered on
// the context's stream, and wait for it.  A one-warp kernel stores the words into pinned
// host memory, so the read does not queue on a copy engine behind a large download that
// another stream has in flight (the streaming surface job's payload).
constexpr size_t kSmallReadBytes = 256;
int readSmall(msbg_gpu_ctx *ctx, void *hDst, const void *dSrc, size_t bytes);

// Ensure the temp slab can hold `bytes`.
int ensureTmpSlab(msbg_gpu_ctx *ctx, size_t bytes);

// Per-file entry points used by the ABI layer.
int splatRun(msbg_gpu_ctx *ctx, const float *dPts, int64_t n, float rParticle, float nbDist);
int splatFinalizeRun(msbg_gpu_ctx *ctx, float rParticle, float nbDist);
int particlesPerBlockRun(msbg_gpu_ctx *ctx, const float *dPts, int64_t n, int64_t *dOff, int32_t *dIndex,
                         int64_t *count);
int fillChannel(msbg_gpu_ctx *ctx, int chan, double v);
// Sweeps over all value blocks (dList NULL) or the listed blocks (device block ids).
int pdeRun(msbg_gpu_ctx *ctx, int chan, int laplTyp, int constr01, int numIter, float dt,
           float anisAlpha, int variant, const int32_t *dList = nullptr, int64_t nList = 0);

// ---- storage conversions (device) ---------------------------------------------
// uint16 density: load v*(1/65535) (src/sbg.h:225-247); the sweep store rounds half
// to even (src/sbg.h:343-351), the scalar store of splat/finalize rounds half away
// from zero (src/sbg.h:271-296).
constexpr float kU16ToF = 1.0f / 65535.0f;

template <typename T> struct Store;
template <> struct Store<float> {
  static __device__ __forceinline__ float load(const float *p) { return *p; }
  static __device__ __forceinline__ void storeRNE(float *p, float v) { *p = v; }
  static __device__ __forceinline__ void storeRHA(float *p, float v) { *p = v; }
  static __device__ __forceinline__ float quant(float v) { return v; }
};
template <> struct Store<uint16_t> {
  static __device__ __forceinline__ float load(const uint16_t *p) {
    return __fmul_rn((float)*p, kU16ToF);
  }
  static __device__ __forceinline__ void storeRNE(uint16_t *p, float v) {
    *p = (uint16_t)__float2uint_rn(__fmul_rn(v, 65535.0f));
  }
  static __device__ __forceinline__ void storeRHA(uint16_t *p, float v) {
    *p = (uint16_t)roundf(__fmul_rn(v, 65535.0f));
  }
  // value after a round-half-away store and a load
  static __device__ __forceinline__ float quant(float v) {
    return __fmul_rn(roundf(__fmul_rn(v, 65535.0f)), kU16ToF);
  }
};
template <> struct Store<__half> {
  static __device__ __forceinline__ float load(const __half *p) { return __half2float(*p); }
  static __device__ __forceinline__ void storeRNE(__half *p, float v) { *p = __float2half_rn(v); }
  static __device__ __forceinline__ void storeRHA(__half *p, float v) { *p = __float2half_rn(v); }
  static __device__ __forceinline__ float quant(float v) {
    return __half2float(__float2half_rn(v));
  }
};
template <> struct Store<double> {
  static __device__ __forceinline__ double load(const double *p) { return *p; }
  static __device__ __forceinline__ void storeRNE(double *p, double v) { *p = v; }
  static __device__ __forceinline__ void storeRHA(double *p, double v) { *p = v; }
  static __device__ __forceinline__ double quant(double v) { return v; }
};

}  // namespace msbg
