// Morton order of block lists: MultiresSparseGrid::sortBlockListMorton
// (src/msbg2.cpp:46-58), which sorts a block list by FMA::morton64_encode of the block
// coordinates (src/fastmath.h:290-316: x, y, z bits interleaved, x lowest), e.g. the
// existing-block list of setRefinementMap (src/msbg.cpp:2036-2050), for locality.
//
// No comparison sort: the Morton codes of a grid's blocks are all the integers below
// 8^K (K = bits of the largest block-grid side) that decode to a block inside the grid,
// and distinct blocks have distinct codes.  So the sorted list is the stream compaction,
// in code order, of the listed blocks: mark the listed blocks, flag every code whose
// block is marked, scan the flags, scatter.  O(8^K) work, at most 8x the block count.
#include "internal.cuh"

namespace msbg {

namespace {

__device__ __forceinline__ uint32_t compact3(uint64_t m) {  // every third bit, from bit 0
  m &= 0x1249249249249249ull;
  m = (m ^ (m >> 2)) & 0x10c30c30c30c30c3ull;
  m = (m ^ (m >> 4)) & 0x100f00f00f00f00full;
  m = (m ^ (m >> 8)) & 0x1f0000ff0000ffull;
  m = (m ^ (m >> 16)) & 0x1f00000000ffffull;
  m = (m ^ (m >> 32)) & 0x1fffffull;
  return (uint32_t)m;
}

__global__ void kMortonMark(const int32_t *__restrict__ bids, int64_t n, int64_t nBlocks,
                            int32_t *__restrict__ mark, int *__restrict__ bad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t b = bids[i];
  if (b < 0 || b >= nBlocks) {
    atomicOr(bad, 1);
    return;
  }
  if (atomicAdd(mark + b, 1) != 0) atomicOr(bad, 2);  // listed twice
}

// flags[m] = 1 when code m decodes to a marked block
__global__ void kMortonFlags(const int32_t *__restrict__ mark, int64_t nCodes, int nbx, int nby, int nbz,
                             int32_t *__restrict__ flags) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nCodes) return;
  const uint32_t x = compact3((uint64_t)m), y = compact3((uint64_t)m >> 1), z = compact3((uint64_t)m >> 2);
  int32_t f = 0;
  if (x < (uint32_t)nbx && y < (uint32_t)nby && z < (uint32_t)nbz)
    f = mark[(int64_t)z * nbx * nby + (int64_t)y * nbx + x] != 0;
  flags[m] = f;
}

__global__ void kMortonScatter(const int32_t *__restrict__ flags, const int64_t *__restrict__ pos, int64_t nCodes,
                               int nbx, int nby, int32_t *__restrict__ out) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nCodes || !flags[m]) return;
  const uint32_t x = compact3((uint64_t)m), y = compact3((uint64_t)m >> 1), z = compact3((uint64_t)m >> 2);
  out[pos[m]] = (int32_t)((int64_t)z * nbx * nby + (int64_t)y * nbx + x);
}

}  // namespace

}  // namespace msbg

using namespace msbg;

extern "C" int msbg_gpu_sort_block_list_morton(msbg_gpu_ctx *ctx, int32_t *dBids, int64_t n) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  if (n < 0 || n > ctx->nBlocks || (n > 0 && !dBids))
    return fail(ctx, MSBG_GPU_ERR_ARG, "sort_block_list_morton: bad list (n = %lld)", (long long)n);
  if (n <= 1) return MSBG_GPU_OK;
  int K = 0;
  while ((1 << K) < ctx->nbx || (1 << K) < ctx->nby || (1 << K) < ctx->nbz) K++;
  const int64_t nCodes = (int64_t)1 << (3 * K);
  if (nCodes > ((int64_t)1 << 27) && nCodes > 8 * ctx->nBlocks)
    return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED,
                "sort_block_list_morton: block grid too elongated (%lld codes for %lld blocks)",
                (long long)nCodes, (long long)ctx->nBlocks);
  // scratch, 8-byte aligned pieces: offsets and scan partials per code, marks per block,
  // flags per code, the sorted list, a status word and the total
  const int64_t nPart = scanPartialCount(nCodes);
  auto up8 = [](size_t b) { return (b + 7) & ~(size_t)7; };
  const size_t bPos = (size_t)nCodes * 8, bPart = (size_t)nPart * 8, bMark = up8((size_t)ctx->nBlocks * 4),
               bFlags = up8((size_t)nCodes * 4), bOut = up8((size_t)n * 4);
  char *scratch = nullptr;
  MSBG_CUDA(ctx, cudaMalloc(&scratch, bPos + bPart + bMark + bFlags + bOut + 16));
  int64_t *pos = (int64_t *)scratch;
  int64_t *part = (int64_t *)(scratch + bPos);
  int32_t *mark = (int32_t *)(scratch + bPos + bPart);
  int32_t *flags = (int32_t *)(scratch + bPos + bPart + bMark);
  int32_t *out = (int32_t *)(scratch + bPos + bPart + bMark + bFlags);
  int64_t *total = (int64_t *)(scratch + bPos + bPart + bMark + bFlags + bOut);
  int *bad = (int *)(total + 1);
  int rc = MSBG_GPU_OK;
  int hBad = 0;
  do {
    if (cudaMemsetAsync(mark, 0, bMark, ctx->stream) != cudaSuccess ||
        cudaMemsetAsync(bad, 0, sizeof(int), ctx->stream) != cudaSuccess) {
      rc = fail(ctx, MSBG_GPU_ERR_CUDA, "sort_block_list_morton: memset failed");
      break;
    }
    kMortonMark<<<gridFor(n, 256), 256, 0, ctx->stream>>>(dBids, n, ctx->nBlocks, mark, bad);
    ctx->launches++;
    kMortonFlags<<<gridFor(nCodes, 256), 256, 0, ctx->stream>>>(mark, nCodes, ctx->nbx, ctx->nby, ctx->nbz, flags);
    ctx->launches++;
    rc = exclusiveScanFlagsWith(ctx, flags, nCodes, pos, total, part);
    if (rc) break;
    kMortonScatter<<<gridFor(nCodes, 256), 256, 0, ctx->stream>>>(flags, pos, nCodes, ctx->nbx, ctx->nby, out);
    ctx->launches++;
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(&hBad, bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
      rc = fail(ctx, MSBG_GPU_ERR_CUDA, "sort_block_list_morton: launch failed");
      break;
    }
    if (hBad & 1) { rc = fail(ctx, MSBG_GPU_ERR_ARG, "sort_block_list_morton: block id out of range"); break; }
    if (hBad & 2) { rc = fail(ctx, MSBG_GPU_ERR_ARG, "sort_block_list_morton: a block is listed twice"); break; }
    if (cudaMemcpyAsync(dBids, out, (size_t)n * 4, cudaMemcpyDeviceToDevice, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess)
      rc = fail(ctx, MSBG_GPU_ERR_CUDA, "sort_block_list_morton: copy failed");
  } while (0);
  cudaFree(scratch);
  return rc;
}
