// setRefinementMap's outputs beyond the per-block levels and flags (src/msbg.cpp:1428-2165):
//   _blocksExisting             blocks flagged BLK_EXISTS             (src/msbg.cpp:1682-1685)
//   _blocksFineCoarsePerLevel   blocks of level l flagged BLK_FINE_COARSE (src/msbg.cpp:1721-1727)
//   CH_DIST_FINECOARSE          per level, the distance of every cell of a fine-coarse block
//                               to the nearest coarser 26-neighbour block, clamped to
//                               dTransRes and stored as uint16(1024 d) (src/msbg.cpp:1887-1960),
//                               plus full blocks around them (src/msbg.cpp:1994-2033)
// The lists come out in ascending block id (the release fills them from per-thread parts, so
// only their contents are defined there).
#include "internal.cuh"

namespace msbg {
namespace {

constexpr uint16_t kBlkFineCoarse = MSBG_GPU_BLK_FINE_COARSE, kBlkExists = MSBG_GPU_BLK_EXISTS;

__global__ void kListFlags(const int32_t *__restrict__ levels, const uint16_t *__restrict__ flags, int64_t n,
                           int which, int level, int32_t *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = which == MSBG_GPU_LIST_EXISTING ? (flags[i] & kBlkExists) != 0
                                            : levels[i] == level && (flags[i] & kBlkFineCoarse) != 0;
}

__global__ void kListScatter(const int32_t *__restrict__ flag, const int64_t *__restrict__ off, int64_t n,
                             int32_t *__restrict__ out, int32_t *__restrict__ state) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (flag[i]) {
    if (out) out[off[i]] = (int32_t)i;
    if (state) state[i] = (int32_t)off[i];
  } else if (state) {
    state[i] = MSBG_GPU_LBLK_EMPTY;
  }
}

// Blocks of level l-1 or l without data that touch a fine-coarse block of level l: full.
__global__ void kDistFull(const int32_t *__restrict__ levels, const uint16_t *__restrict__ flags, int nbx, int nby,
                          int nbz, int level, int32_t *__restrict__ state) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= (int64_t)nbx * nby * nbz || state[b] >= 0) return;
  const int lb = levels[b];
  if (lb > level || lb < level - 1) return;
  const int bx = (int)(b % nbx), by = (int)((b / nbx) % nby), bz = (int)(b / ((int64_t)nbx * nby));
  for (int dz = -1; dz <= 1; dz++)
    for (int dy = -1; dy <= 1; dy++)
      for (int dx = -1; dx <= 1; dx++) {
        const int x = bx + dx, y = by + dy, z = bz + dz;
        if ((!dx && !dy && !dz) || x < 0 || y < 0 || z < 0 || x >= nbx || y >= nby || z >= nbz) continue;
        const int64_t b2 = ((int64_t)z * nby + y) * nbx + x;
        if (levels[b2] == level && (flags[b2] & kBlkFineCoarse)) {
          state[b] = MSBG_GPU_LBLK_FULL;
          return;
        }
      }
}

// One CTA per fine-coarse block (list[k] = its id, data block k): the distance of every
// cell centre to the nearest coarser neighbour block (distToBoxSq, src/msbg.h:3874-3886).
// The squared distances are sums of squares of multiples of 1/2, exact in FP32, so the
// result does not depend on the order of the operations.
__global__ void __launch_bounds__(256) kDistData(const int32_t *__restrict__ list, const int32_t *__restrict__ levels,
                                                 int nbx, int nby, int nbz, int level, int bs, int dTransRes,
                                                 uint16_t *__restrict__ data) {
  __shared__ float box[26][3];
  __shared__ int nbox;
  const int b = list[blockIdx.x];
  const int bx = b % nbx, by = (b / nbx) % nby, bz = (int)(b / ((int64_t)nbx * nby));
  if (threadIdx.x == 0) {
    int k = 0;
    for (int dz = -1; dz <= 1; dz++)
      for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++) {
          const int x = bx + dx, y = by + dy, z = bz + dz;
          if ((!dx && !dy && !dz) || x < 0 || y < 0 || z < 0 || x >= nbx || y >= nby || z >= nbz) continue;
          if (levels[((int64_t)z * nby + y) * nbx + x] <= level) continue;
          box[k][0] = (float)x; box[k][1] = (float)y; box[k][2] = (float)z;
          k++;
        }
    nbox = k;
  }
  __syncthreads();
  const int vpb = bs * bs * bs;
  uint16_t *d = data + (int64_t)blockIdx.x * vpb;
  for (int v = threadIdx.x; v < vpb; v += blockDim.x) {
    const int x1 = bx * bs + v % bs, y1 = by * bs + (v / bs) % bs, z1 = bz * bs + v / (bs * bs);
    const float p[3] = {x1 + 0.5f, y1 + 0.5f, z1 + 0.5f};
    float d2 = 1e20f;
    for (int i = 0; i < nbox; i++) {
      float s2 = 0.0f;
#pragma unroll
      for (int a = 0; a < 3; a++) {
        const float lo = __fsub_rn(__fmul_rn(box[i][a], (float)bs), p[a]);
        const float hi = __fsub_rn(p[a], __fmul_rn(__fadd_rn(box[i][a], 1.0f), (float)bs));
        float m = lo > 0.0f ? lo : 0.0f;
        m = m > hi ? m : hi;
        s2 = __fadd_rn(s2, __fmul_rn(m, m));
      }
      d2 = fminf(d2, s2);
    }
    float dist = __fsqrt_rn(d2);
    if (dist < 0.0f || dist > (float)dTransRes) dist = (float)dTransRes;
    d[v] = (uint16_t)(dist * 1024.0f);
  }
}

// flag -> exclusive scan -> scatter; returns the count (synchronizes).
int compactBlocks(msbg_gpu_ctx *ctx, int which, int level, int32_t *dList, int32_t *dState, int64_t *count) {
  const int64_t nB = ctx->nBlocks;
  int rc = ensureTmpSlab(ctx, (size_t)nB * 12 + 64);
  if (rc) return rc;
  int32_t *flag = (int32_t *)ctx->dTmpSlab;
  int64_t *off = (int64_t *)((char *)ctx->dTmpSlab + (((size_t)nB * 4 + 15) & ~size_t(15)));
  MSBG_LAUNCH(ctx, kListFlags, gridFor(nB, 256), 256, 0, ctx->dLevels, ctx->dFlags, nB, which, level, flag);
  if ((rc = exclusiveScanFlags(ctx, flag, nB, off, ctx->dCounters + 3))) return rc;
  MSBG_LAUNCH(ctx, kListScatter, gridFor(nB, 256), 256, 0, flag, off, nB, dList, dState);
  int64_t n = 0;
  MSBG_CUDA(ctx, cudaMemcpyAsync(&n, ctx->dCounters + 3, 8, cudaMemcpyDeviceToHost, ctx->stream));
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  *count = n;
  return MSBG_GPU_OK;
}

}  // namespace
}  // namespace msbg

using namespace msbg;

extern "C" int msbg_gpu_get_block_list(msbg_gpu_ctx *ctx, int which, int level, int32_t *dBids, int64_t *hCount) {
  if (!ctx || !dBids || !hCount) return MSBG_GPU_ERR_ARG;
  if (which != MSBG_GPU_LIST_EXISTING && which != MSBG_GPU_LIST_FINE_COARSE)
    return fail(ctx, MSBG_GPU_ERR_ARG, "get_block_list: list %d", which);
  if (which == MSBG_GPU_LIST_FINE_COARSE && (level < 0 || level >= ctx->nLevels))
    return fail(ctx, MSBG_GPU_ERR_ARG, "get_block_list: level %d", level);
  if (!ctx->layoutValid) return fail(ctx, MSBG_GPU_ERR_STATE, "get_block_list: no block layout");
  return compactBlocks(ctx, which, level, dBids, nullptr, hCount);
}

extern "C" int msbg_gpu_dist_fine_coarse(msbg_gpu_ctx *ctx, int level, int32_t *dState, uint16_t *dData,
                                         int64_t capBlocks, int64_t *hCount) {
  if (!ctx || !dState || !hCount || capBlocks < 0 || (capBlocks > 0 && !dData)) return MSBG_GPU_ERR_ARG;
  if (level < 0 || level >= ctx->nLevels || (ctx->bsx >> level) < 1)
    return fail(ctx, MSBG_GPU_ERR_ARG, "dist_fine_coarse: level %d", level);
  if (!ctx->layoutValid) return fail(ctx, MSBG_GPU_ERR_STATE, "dist_fine_coarse: no block layout");
  const int64_t nB = ctx->nBlocks;
  int32_t *list = nullptr;
  MSBG_CUDA(ctx, cudaMallocAsync(&list, (size_t)nB * 4, ctx->stream));
  int64_t n = 0;
  int rc = compactBlocks(ctx, MSBG_GPU_LIST_FINE_COARSE, level, list, dState, &n);
  if (!rc && n > capBlocks)
    rc = fail(ctx, MSBG_GPU_ERR_CAPACITY, "dist_fine_coarse: %lld blocks exceed the capacity %lld", (long long)n,
              (long long)capBlocks);
  if (!rc) {
    kDistFull<<<gridFor(nB, 256), 256, 0, ctx->stream>>>(ctx->dLevels, ctx->dFlags, ctx->nbx, ctx->nby, ctx->nbz,
                                                         level, dState);
    ctx->launches++;
    if (n > 0) {
      // the reference's transition width (src/msbg.cpp:197-202)
      kDistData<<<(unsigned)n, 256, 0, ctx->stream>>>(list, ctx->dLevels, ctx->nbx, ctx->nby, ctx->nbz, level,
                                                       ctx->bsx >> level, 6, dData);
      ctx->launches++;
    }
    if (cudaGetLastError() != cudaSuccess) rc = fail(ctx, MSBG_GPU_ERR_CUDA, "dist_fine_coarse: launch failed");
  }
  cudaFreeAsync(list, ctx->stream);
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess && !rc) rc = fail(ctx, MSBG_GPU_ERR_CUDA, "dist_fine_coarse");
  if (!rc) *hCount = n;
  return rc;
}
