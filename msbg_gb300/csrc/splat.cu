// Particle splat and distance-to-density finalize (channel 0).
//
// Reference: the demo's 8-color lockless splat (src/msbg_demo.cpp:527-636) and
// finalize (src/msbg_demo.cpp:655-680).  The CPU code walks per-block particle
// lists in 8 colors so that threads never write the same block concurrently.
// Here the particles are sorted by the value blocks their splat boxes touch (a
// counting sort: count, scan, scatter), and one CTA per value block takes the
// minimum of its particles' values in shared memory (atomicMin on the float's bit
// pattern: distances are non-negative, so their bit patterns order like the
// floats) and writes the block once.  The minimum is order-independent, so this
// gives the same field as the colored passes.
//
// The minimum is taken in FP32.  For uint16 / FP16 storage the splat runs into an
// FP32 staging slab and the finalize quantizes the minimum to the storage type
// first: rounding is monotonic, so quantize(min) == min(quantize) and the result
// equals the demo's min over quantized values (src/msbg_demo.cpp:624-628).
#include "internal.cuh"

namespace msbg {

// Every voxel of a slab <- v (the demo fills value blocks with 1.0 before splatting).
// Eight voxels per thread and step, stored as 16-byte vectors.
template <typename T>
__global__ void kFill(T *__restrict__ p, int64_t n, float v, double vd) {
  T e;
  if constexpr (sizeof(T) == 8) e = vd; else Store<T>::storeRHA(&e, v);
  T q[8];
#pragma unroll
  for (int k = 0; k < 8; k++) q[k] = e;
  const int64_t n8 = n / 8;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n8; i += (int64_t)gridDim.x * blockDim.x) {
    uint4 *dst = reinterpret_cast<uint4 *>(p + 8 * i);
#pragma unroll
    for (int k = 0; k < (int)(8 * sizeof(T) / 16); k++) dst[k] = reinterpret_cast<const uint4 *>(q)[k];
  }
  for (int64_t i = 8 * n8 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = e;
}

static unsigned gridVec(int64_t n) {  // 8 elements per thread, grid-stride
  const int64_t t = (n / 8 + 255) / 256;
  return (unsigned)(t < 1 ? 1 : t > 152 * 64 ? 152 * 64 : t);
}

int fillChannel(msbg_gpu_ctx *ctx, int chan, double v) {
  Channel &c = ctx->ch[chan];
  const int64_t n = ctx->nActive * ctx->voxPerBlock;
  if (n == 0) return MSBG_GPU_OK;
  switch (c.storage) {
    case MSBG_GPU_F32: MSBG_LAUNCH(ctx, kFill<float>, gridVec(n), 256, 0, (float *)c.d, n, (float)v, v); break;
    case MSBG_GPU_U16: MSBG_LAUNCH(ctx, kFill<uint16_t>, gridVec(n), 256, 0, (uint16_t *)c.d, n, (float)v, v); break;
    case MSBG_GPU_F16: MSBG_LAUNCH(ctx, kFill<__half>, gridVec(n), 256, 0, (__half *)c.d, n, (float)v, v); break;
    default: MSBG_LAUNCH(ctx, kFill<double>, gridVec(n), 256, 0, (double *)c.d, n, (float)v, v); break;
  }
  return MSBG_GPU_OK;
}

struct SplatGeom {
  int sx, sy, sz, nbx, nby, log2bs;
  float domMin[3], domMax[3];
  float rScan, distSqMax, distSqMaxInv;
};

// A particle's splat box (src/msbg_demo.cpp:571-592): voxels [i1, i2] per axis,
// the voxel centres within rScan of the particle, clamped to the grid.
struct SplatBox {
  int ix1, iy1, iz1, ix2, iy2, iz2;
  float x0, y0, z0;  // particle position - 0.5 (voxel centre offsets)
};

__device__ __forceinline__ bool splatBox(const SplatGeom &g, float px, float py, float pz, SplatBox &b) {
  const float r = g.rScan;
  b.ix1 = max((int)ceilf(__fsub_rn(__fsub_rn(px, r), 0.5f)), 0);
  b.iy1 = max((int)ceilf(__fsub_rn(__fsub_rn(py, r), 0.5f)), 0);
  b.iz1 = max((int)ceilf(__fsub_rn(__fsub_rn(pz, r), 0.5f)), 0);
  b.ix2 = min((int)floorf(__fsub_rn(__fadd_rn(px, r), 0.5f)), g.sx - 1);
  b.iy2 = min((int)floorf(__fsub_rn(__fadd_rn(py, r), 0.5f)), g.sy - 1);
  b.iz2 = min((int)floorf(__fsub_rn(__fadd_rn(pz, r), 0.5f)), g.sz - 1);
  b.x0 = __fsub_rn(px, 0.5f); b.y0 = __fsub_rn(py, 0.5f); b.z0 = __fsub_rn(pz, 0.5f);
  return b.ix2 >= b.ix1 && b.iy2 >= b.iy1 && b.iz2 >= b.iz1;
}

// Pass 1, one thread per particle.  Valid particles (the marking loop's domain
// tests, src/msbg_demo.cpp:358-360, and an owning value block: the demo walks the
// particle lists of value blocks only, src/msbg_demo.cpp:541-566) get their abort
// index: the scan position (z, y, x order over the box) of the first in-sphere
// voxel whose block is not a value block (src/msbg_demo.cpp:613-618), or the box
// size.  Voxels from that position on are not written.  Every value block the box
// touches (at most two per axis) counts the particle once.  abortAt = 0 marks a
// particle that writes nothing.
__global__ void __launch_bounds__(256) kSplatCount(const float *__restrict__ pts, int64_t n, SplatGeom g,
                                                   const int32_t *__restrict__ slot, int32_t *__restrict__ abortAt,
                                                   int32_t *__restrict__ cnt,
                                                   unsigned long long *__restrict__ nAborted) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float px = pts[3 * i], py = pts[3 * i + 1], pz = pts[3 * i + 2];
  abortAt[i] = 0;
  if (px < g.domMin[0] || px > g.domMax[0] || py < g.domMin[1] || py > g.domMax[1] ||
      pz < g.domMin[2] || pz > g.domMax[2])
    return;
  const int s = g.log2bs;
  const int64_t nxy = (int64_t)g.nbx * g.nby;
  {
    const int ix = (int)px, iy = (int)py, iz = (int)pz;
    if (ix < 0 || ix >= g.sx || iy < 0 || iy >= g.sy || iz < 0 || iz >= g.sz) return;
    if (slot[(int64_t)(iz >> s) * nxy + (int64_t)(iy >> s) * g.nbx + (ix >> s)] < 0) return;
  }
  SplatBox b;
  if (!splatBox(g, px, py, pz, b)) return;
  const int nx = b.ix2 - b.ix1 + 1, ny = b.iy2 - b.iy1 + 1, nz = b.iz2 - b.iz1 + 1;
  const int total = nx * ny * nz;
  const int bx[2] = {b.ix1 >> s, b.ix2 >> s}, by[2] = {b.iy1 >> s, b.iy2 >> s}, bz[2] = {b.iz1 >> s, b.iz2 >> s};
  int32_t sl[8];
  bool allValue = true;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    sl[k] = slot[(int64_t)bz[k >> 2] * nxy + (int64_t)by[(k >> 1) & 1] * g.nbx + bx[k & 1]];
    allValue = allValue && sl[k] >= 0;
  }
  int abortIdx = total;
  if (!allValue) {
    for (int t = 0; t < total; t++) {
      const int lx = t % nx, rest = t / nx, ly = rest % ny, lz = rest / ny;
      const int ix = b.ix1 + lx, iy = b.iy1 + ly, iz = b.iz1 + lz;
      const float dz = __fsub_rn((float)iz, b.z0), dy = __fsub_rn((float)iy, b.y0), dx = __fsub_rn((float)ix, b.x0);
      const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dz, dz), __fmul_rn(dy, dy)), __fmul_rn(dx, dx));
      if (d2 > g.distSqMax) continue;
      if (slot[(int64_t)(iz >> s) * nxy + (int64_t)(iy >> s) * g.nbx + (ix >> s)] < 0) {
        abortIdx = t;
        break;
      }
    }
    if (abortIdx < total) atomicAdd(nAborted, 1ull);
  }
  abortAt[i] = abortIdx;
  if (abortIdx == 0) return;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    // each distinct touched value block once
    const bool dup = ((k & 1) && bx[1] == bx[0]) || ((k & 2) && by[1] == by[0]) || ((k & 4) && bz[1] == bz[0]);
    if (!dup && sl[k] >= 0) atomicAdd(&cnt[sl[k]], 1);
  }
}

// Pass 2: the particle's index into the list of every value block it touches
// (list of slot s: entries[off[s] .. off[s+1]-1], in no particular order).
__global__ void __launch_bounds__(256) kSplatScatter(const float *__restrict__ pts, int64_t n, SplatGeom g,
                                                     const int32_t *__restrict__ slot,
                                                     const int32_t *__restrict__ abortAt,
                                                     const int64_t *__restrict__ off, int32_t *__restrict__ cursor,
                                                     int32_t *__restrict__ entries) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || abortAt[i] == 0) return;
  const float px = pts[3 * i], py = pts[3 * i + 1], pz = pts[3 * i + 2];
  SplatBox b;
  splatBox(g, px, py, pz, b);
  const int s = g.log2bs;
  const int64_t nxy = (int64_t)g.nbx * g.nby;
  const int bx[2] = {b.ix1 >> s, b.ix2 >> s}, by[2] = {b.iy1 >> s, b.iy2 >> s}, bz[2] = {b.iz1 >> s, b.iz2 >> s};
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const bool dup = ((k & 1) && bx[1] == bx[0]) || ((k & 2) && by[1] == by[0]) || ((k & 4) && bz[1] == bz[0]);
    if (dup) continue;
    const int sl = slot[(int64_t)bz[k >> 2] * nxy + (int64_t)by[(k >> 1) & 1] * g.nbx + bx[k & 1]];
    if (sl >= 0) entries[off[sl] + atomicAdd(&cursor[sl], 1)] = (int32_t)i;
  }
}

// Pass 3, one CTA per value block (slot = blockIdx.x): the minimum of the splat
// values of the block's particles in shared memory, starting from the block's
// current values (init: FP32 channels, where the demo's splat takes the minimum
// with what the channel holds) or from 1.0 (the FP32 staging of other storage
// types, which the demo fills with 1.0 first), then one coalesced write of the
// block.  A warp takes one particle at a time; its
// lanes take the (y, z) rows of the box clipped to the block, skip rows already
// outside the sphere (dz*dz + dy*dy exceeds it, and adding dx*dx >= 0 cannot lower
// a float sum), and keep the voxels before the particle's abort index.
// The block's minima in shared memory use a row stride of BS + 1 words: the lanes
// of a warp take different rows, which then fall into different banks.  NZ CTAs
// share a block, each taking BS/NZ of its z-planes (and clipping the boxes to
// them): for BS = 32 two halves of 68 KB let three CTAs share an SM where a whole
// block's 135 KB allowed one.
template <int BS, int NZ>
constexpr int splatSmemWords() { return BS * (BS / NZ) * (BS + 1); }
// threads per CTA (512, 256, 128 for BS 32, 16, 8), and CTAs per SM to keep the registers
// for: 1536 threads
template <int BS>
constexpr int splatThreads() { return 16 * BS; }
template <int BS>
constexpr int splatMinCtas() { return 1536 / splatThreads<BS>(); }

template <int BS, int NZ>
__global__ void __launch_bounds__(splatThreads<BS>(), splatMinCtas<BS>()) kSplatBlock(const float *__restrict__ pts, SplatGeom g,
                                                   const int32_t *__restrict__ active,
                                                   const int32_t *__restrict__ abortAt,
                                                   const int64_t *__restrict__ off,
                                                   const int32_t *__restrict__ entries, const float *init,
                                                   float *dst) {
  constexpr int VPB = BS * BS * BS, RS = BS + 1, PZ = BS / NZ, VPP = BS * BS * PZ;
  extern __shared__ __align__(16) int smin[];
  const int sl = blockIdx.x / NZ, zp = blockIdx.x % NZ;
  const int bid = active[sl];
  const int X0 = (bid % g.nbx) * BS, Y0 = ((bid / g.nbx) % g.nby) * BS,
            Z0 = (int)(bid / ((int64_t)g.nbx * g.nby)) * BS + zp * PZ;  // this CTA's first plane
  const int one = __float_as_int(1.0f);
  const float *in = init ? init + (int64_t)sl * VPB + zp * VPP : nullptr;
  for (int v = threadIdx.x; v < VPP; v += blockDim.x)
    smin[(v / BS) * RS + v % BS] = in ? __float_as_int(in[v]) : one;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nWarps = blockDim.x >> 5;
  const int64_t e0 = off[sl], e1 = off[sl + 1];
  for (int64_t e = e0 + warp; e < e1; e += nWarps) {
    const int i = entries[e];
    const float px = pts[3 * (int64_t)i], py = pts[3 * (int64_t)i + 1], pz = pts[3 * (int64_t)i + 2];
    const int ab = abortAt[i];
    SplatBox b;
    splatBox(g, px, py, pz, b);
    const int nx = b.ix2 - b.ix1 + 1, ny = b.iy2 - b.iy1 + 1;
    const int cx1 = max(b.ix1, X0), cx2 = min(b.ix2, X0 + BS - 1);
    const int cy1 = max(b.iy1, Y0), cy2 = min(b.iy2, Y0 + BS - 1);
    const int cz1 = max(b.iz1, Z0), cz2 = min(b.iz2, Z0 + PZ - 1);
    const int cny = cy2 - cy1 + 1, cnz = cz2 - cz1 + 1;
    if (cx2 < cx1 || cny <= 0 || cnz <= 0) continue;
    // the lane's rows: row = lane + 32 k, decoded as (row % cny, row / cny) through an
    // approximate reciprocal (row < 34^2 and cny <= 33: the quotient's fraction stays
    // at least 1/(2 cny) away from an integer, so the truncation is exact)
    const float rcny = __frcp_rn((float)cny);
    for (int row = lane; row < cny * cnz; row += 32) {
      const int qz = (int)(((float)row + 0.5f) * rcny);
      const int iy = cy1 + row - qz * cny, iz = cz1 + qz;
      const float dz = __fsub_rn((float)iz, b.z0), dy = __fsub_rn((float)iy, b.y0);
      const float dzy = __fadd_rn(__fmul_rn(dz, dz), __fmul_rn(dy, dy));
      if (dzy > g.distSqMax) continue;
      const int rowScan = ((iz - b.iz1) * ny + (iy - b.iy1)) * nx - b.ix1;  // + ix: the scan index
      int *rowMin = smin + ((iz - Z0) * BS + (iy - Y0)) * RS - X0;
      // the scan index grows with ix along the row, so the abort rule cuts the row at
      // ab - rowScan; x runs as a float (exact for these integers)
      const int xEnd = min(cx2, ab - 1 - rowScan);
      float fx = (float)cx1;
      for (int ix = cx1; ix <= xEnd; ix++, fx += 1.0f) {
        // distSq exactly as the demo forms it: (dz*dz + dy*dy) + dx*dx
        const float dx = __fsub_rn(fx, b.x0);
        const float d2 = __fadd_rn(dzy, __fmul_rn(dx, dx));
        if (d2 > g.distSqMax) continue;
        atomicMin(rowMin + ix, __float_as_int(__fmul_rn(d2, g.distSqMaxInv)));
      }
    }
  }
  __syncthreads();
  float *out = dst + (int64_t)sl * VPB + zp * VPP;
  for (int v = threadIdx.x * 4; v < VPP; v += blockDim.x * 4) {
    const int *row = smin + (v / BS) * RS + v % BS;
    *reinterpret_cast<int4 *>(out + v) = make_int4(row[0], row[1], row[2], row[3]);
  }
}

// The demo's particlesPerBlock (src/msbg_demo.cpp:349-390): the containing block
// of every point that passes the marking loop's domain tests.
__device__ __forceinline__ int64_t ownerBlock(const SplatGeom &g, int nbz, const float *pts, int64_t i) {
  const float px = pts[3 * i], py = pts[3 * i + 1], pz = pts[3 * i + 2];
  if (px < g.domMin[0] || px > g.domMax[0] || py < g.domMin[1] || py > g.domMax[1] || pz < g.domMin[2] ||
      pz > g.domMax[2])
    return -1;
  const int ix = (int)px, iy = (int)py, iz = (int)pz;
  if (ix < 0 || ix >= g.sx || iy < 0 || iy >= g.sy || iz < 0 || iz >= g.sz) return -1;
  const int s = g.log2bs;
  return ((int64_t)(iz >> s) * g.nby + (iy >> s)) * g.nbx + (ix >> s);
}

__global__ void kOwnerCount(const float *__restrict__ pts, int64_t n, SplatGeom g, int nbz, int32_t *__restrict__ cnt) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t b = ownerBlock(g, nbz, pts, i);
  if (b >= 0) atomicAdd(&cnt[b], 1);
}

__global__ void kOwnerScatter(const float *__restrict__ pts, int64_t n, SplatGeom g, int nbz,
                              const int64_t *__restrict__ off, int32_t *__restrict__ cursor,
                              int32_t *__restrict__ index) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t b = ownerBlock(g, nbz, pts, i);
  if (b >= 0) index[off[b] + atomicAdd(&cursor[b], 1)] = (int32_t)i;
}

// distance -> density of one voxel (q: the quantized minimum splat value)
__device__ __forceinline__ float finalizeValue(float d, float rParticle, float nbDist, float distSqMax) {
  float f = 0.0f;
  if (d < 0.999f) {
    d = __fmul_rn(d, distSqMax);
    const float dist = __fsub_rn(__fsqrt_rn(d), rParticle);
    // 1 - MT_LINSTEPF(-rParticle, rParticle + nbDist, dist) (src/mtool.h:400-408);
    // the reference's -ffast-math build divides by the constant span through its
    // rounded reciprocal.
    const float a = -rParticle, b = __fadd_rn(rParticle, nbDist);
    float lin;
    if (dist < a) lin = 0.0f;
    else if (dist >= b) lin = 1.0f;
    else lin = __fmul_rn(__fsub_rn(dist, a), __frcp_rn(__fsub_rn(b, a)));
    f = __fsub_rn(1.0f, lin);
  }
  return f;
}

// Eight voxels per thread and step: two 16-byte reads of the FP32 minimum, one
// 16-byte (2-byte storage) or two (FP32) writes.
template <typename T>
__global__ void kFinalize(const float *__restrict__ splat, T *__restrict__ out, int64_t n, float rParticle,
                          float nbDist, float distSqMax) {
  const int64_t n8 = n / 8;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n8; i += (int64_t)gridDim.x * blockDim.x) {
    const float4 a = reinterpret_cast<const float4 *>(splat)[2 * i], b = reinterpret_cast<const float4 *>(splat)[2 * i + 1];
    const float in[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
    T q[8];
#pragma unroll
    for (int k = 0; k < 8; k++)  // the demo reads back the quantized minimum (renderDensToFloat_)
      Store<T>::storeRHA(&q[k], finalizeValue(Store<T>::quant(in[k]), rParticle, nbDist, distSqMax));
    uint4 *dst = reinterpret_cast<uint4 *>(out + 8 * i);
#pragma unroll
    for (int k = 0; k < (int)(8 * sizeof(T) / 16); k++) dst[k] = reinterpret_cast<const uint4 *>(q)[k];
  }
  for (int64_t i = 8 * n8 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    Store<T>::storeRHA(out + i, finalizeValue(Store<T>::quant(splat[i]), rParticle, nbDist, distSqMax));
}

template <>
__global__ void kFinalize<double>(const float *__restrict__ splat, double *__restrict__ out, int64_t n,
                                  float rParticle, float nbDist, float distSqMax) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = (double)finalizeValue(splat[i], rParticle, nbDist, distSqMax);
}

int splatRun(msbg_gpu_ctx *ctx, const float *dPts, int64_t n, float rParticle, float nbDist) {
  Channel &c = ctx->ch[0];
  const int64_t nAct = ctx->nActive;
  const int64_t nVox = nAct * ctx->voxPerBlock;
  float *dst;
  if (c.storage == MSBG_GPU_F32) {
    dst = (float *)c.d;
  } else {
    int rc = ensureTmpSlab(ctx, (size_t)(nVox > 0 ? nVox : 1) * 4);
    if (rc) return rc;
    dst = (float *)ctx->dTmpSlab;
  }
  MSBG_CUDA(ctx, cudaMemsetAsync(ctx->dCounters + 1, 0, 8, ctx->stream));
  if (nVox == 0) return MSBG_GPU_OK;
  SplatGeom g;
  g.sx = ctx->sx; g.sy = ctx->sy; g.sz = ctx->sz; g.nbx = ctx->nbx; g.nby = ctx->nby;
  g.log2bs = ctx->log2bs;
  for (int k = 0; k < 3; k++) { g.domMin[k] = ctx->domMin[k]; g.domMax[k] = ctx->domMax[k]; }
  g.rScan = rParticle + nbDist;
  g.distSqMax = g.rScan * g.rScan;
  g.distSqMaxInv = 1.0f / g.distSqMax;
  // scratch (stream-ordered): abort indices [n], counts / cursors [nAct], offsets
  // [nAct + 1], list entries [8 n] (a box touches at most 8 blocks)
  const int64_t nn = n > 0 ? n : 1;
  const size_t bAbort = (size_t)nn * 4, bCnt = ((size_t)nAct * 4 + 15) & ~size_t(15),
               bOff = (size_t)(nAct + 1) * 8, bEnt = (size_t)nn * 8 * 4;
  char *scratch = nullptr;
  MSBG_CUDA(ctx, cudaMallocAsync((void **)&scratch, bAbort + 2 * bCnt + bOff + bEnt + 64, ctx->stream));
  int32_t *abortAt = (int32_t *)scratch;
  int32_t *cnt = (int32_t *)(scratch + ((bAbort + 15) & ~size_t(15)));
  int32_t *cursor = (int32_t *)((char *)cnt + bCnt);
  int64_t *off = (int64_t *)((char *)cursor + bCnt);
  int32_t *entries = (int32_t *)((char *)off + ((bOff + 15) & ~size_t(15)));
  int rc = MSBG_GPU_OK;
  auto run = [&]() -> int {
    MSBG_CUDA(ctx, cudaMemsetAsync(cnt, 0, 2 * bCnt, ctx->stream));
    if (n > 0) {
      MSBG_LAUNCH(ctx, kSplatCount, gridFor(n, 256), 256, 0, dPts, n, g, ctx->dSlot, abortAt, cnt,
                  (unsigned long long *)(ctx->dCounters + 1));
    }
    int r = exclusiveScanCounts(ctx, cnt, nAct, off, off + nAct);
    if (r) return r;
    if (n > 0) {
      MSBG_LAUNCH(ctx, kSplatScatter, gridFor(n, 256), 256, 0, dPts, n, g, ctx->dSlot, abortAt, off, cursor,
                  entries);
    }
    const float *init = c.storage == MSBG_GPU_F32 ? dst : nullptr;
    if (ctx->bsx == 32) {
      constexpr int smem = splatSmemWords<32, 2>() * 4;
      static bool attr = false;
      if (!attr) {
        MSBG_CUDA(ctx, cudaFuncSetAttribute(kSplatBlock<32, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        attr = true;
      }
      MSBG_LAUNCH(ctx, (kSplatBlock<32, 2>), (unsigned)(2 * nAct), splatThreads<32>(), smem, dPts, g, ctx->dActive, abortAt, off,
                  entries, init, dst);
    } else if (ctx->bsx == 16) {
      MSBG_LAUNCH(ctx, (kSplatBlock<16, 1>), (unsigned)nAct, splatThreads<16>(), (splatSmemWords<16, 1>() * 4), dPts, g, ctx->dActive,
                  abortAt, off, entries, init, dst);
    } else {
      MSBG_LAUNCH(ctx, (kSplatBlock<8, 1>), (unsigned)nAct, splatThreads<8>(), (splatSmemWords<8, 1>() * 4), dPts, g, ctx->dActive,
                  abortAt, off, entries, init, dst);
    }
    return MSBG_GPU_OK;
  };
  rc = run();
  cudaFreeAsync(scratch, ctx->stream);
  return rc;
}

int splatFinalizeRun(msbg_gpu_ctx *ctx, float rParticle, float nbDist) {
  Channel &c = ctx->ch[0];
  const int64_t n = ctx->nActive * ctx->voxPerBlock;
  if (n == 0) return MSBG_GPU_OK;
  const float rScan = rParticle + nbDist, distSqMax = rScan * rScan;
  const float *src = c.storage == MSBG_GPU_F32 ? (const float *)c.d : (const float *)ctx->dTmpSlab;
  if (c.storage != MSBG_GPU_F32 && ctx->tmpSlabBytes < (size_t)n * 4)
    return fail(ctx, MSBG_GPU_ERR_STATE, "finalize without a splat");
  switch (c.storage) {
    case MSBG_GPU_F32: MSBG_LAUNCH(ctx, kFinalize<float>, gridVec(n), 256, 0, src, (float *)c.d, n, rParticle, nbDist, distSqMax); break;
    case MSBG_GPU_U16: MSBG_LAUNCH(ctx, kFinalize<uint16_t>, gridVec(n), 256, 0, src, (uint16_t *)c.d, n, rParticle, nbDist, distSqMax); break;
    case MSBG_GPU_F16: MSBG_LAUNCH(ctx, kFinalize<__half>, gridVec(n), 256, 0, src, (__half *)c.d, n, rParticle, nbDist, distSqMax); break;
    default: MSBG_LAUNCH(ctx, kFinalize<double>, gridFor(n, 256), 256, 0, src, (double *)c.d, n, rParticle, nbDist, distSqMax); break;
  }
  return MSBG_GPU_OK;
}

int particlesPerBlockRun(msbg_gpu_ctx *ctx, const float *dPts, int64_t n, int64_t *dOff, int32_t *dIndex,
                         int64_t *count) {
  const int64_t nB = ctx->nBlocks;
  SplatGeom g;
  g.sx = ctx->sx; g.sy = ctx->sy; g.sz = ctx->sz; g.nbx = ctx->nbx; g.nby = ctx->nby;
  g.log2bs = ctx->log2bs;
  for (int k = 0; k < 3; k++) { g.domMin[k] = ctx->domMin[k]; g.domMax[k] = ctx->domMax[k]; }
  const size_t bCnt = ((size_t)nB * 4 + 15) & ~size_t(15);
  int32_t *cnt = nullptr;
  MSBG_CUDA(ctx, cudaMallocAsync((void **)&cnt, 2 * bCnt, ctx->stream));
  int32_t *cursor = (int32_t *)((char *)cnt + bCnt);
  auto run = [&]() -> int {
    MSBG_CUDA(ctx, cudaMemsetAsync(cnt, 0, 2 * bCnt, ctx->stream));
    if (n > 0) MSBG_LAUNCH(ctx, kOwnerCount, gridFor(n, 256), 256, 0, dPts, n, g, ctx->nbz, cnt);
    int r = exclusiveScanCounts(ctx, cnt, nB, dOff, dOff + nB);
    if (r) return r;
    if (n > 0) MSBG_LAUNCH(ctx, kOwnerScatter, gridFor(n, 256), 256, 0, dPts, n, g, ctx->nbz, dOff, cursor, dIndex);
    MSBG_CUDA(ctx, cudaMemcpyAsync(count, dOff + nB, 8, cudaMemcpyDeviceToHost, ctx->stream));
    return MSBG_GPU_OK;
  };
  int rc = run();
  cudaFreeAsync(cnt, ctx->stream);
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess && !rc) rc = fail(ctx, MSBG_GPU_ERR_CUDA, "particles_per_block");
  return rc;
}

}  // namespace msbg
