// Particle splat and distance-to-density finalize (channel 0).
//
// Reference: the demo's 8-color lockless splat (src/msbg_demo.cpp:527-636) and
// finalize (src/msbg_demo.cpp:655-680).  The CPU code needs the 8 colors so that
// threads never write the same block concurrently; on the GPU every write is an
// atomicMin on the float's bit pattern (distances are non-negative, so their bit
// patterns order like the floats), which is order-independent: one launch over
// all particles gives the same field as the colored passes.
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

// One warp per particle.  The lanes walk the particle's clipped voxel box in the
// demo's z,y,x scan order (flattened).  Abort rule (src/msbg_demo.cpp:613-618):
// the particle stops at the first in-sphere voxel whose block is not a value
// block; voxels before it in scan order keep their writes.  The box spans at most
// two blocks per axis, so the warp first checks those blocks: if all are value
// blocks nothing can abort (the common case); otherwise it finds the earliest
// aborting scan index with a warp min-reduction and writes only voxels before it.
__global__ void __launch_bounds__(256) kSplat(const float *__restrict__ pts, int64_t n, SplatGeom g,
                                              const int32_t *__restrict__ slot,
                                              float *__restrict__ dst,
                                              unsigned long long *__restrict__ nAborted) {
  const int64_t warpId = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warpId >= n) return;
  const float px = pts[3 * warpId], py = pts[3 * warpId + 1], pz = pts[3 * warpId + 2];
  // domain tests of the marking loop (src/msbg_demo.cpp:358-360)
  if (px < g.domMin[0] || px > g.domMax[0] || py < g.domMin[1] || py > g.domMax[1] ||
      pz < g.domMin[2] || pz > g.domMax[2])
    return;
  const int s = g.log2bs, mask = (1 << s) - 1;
  const int64_t nxy = (int64_t)g.nbx * g.nby;
  {
    const int ix = (int)px, iy = (int)py, iz = (int)pz;
    if (ix < 0 || ix >= g.sx || iy < 0 || iy >= g.sy || iz < 0 || iz >= g.sz) return;
    // the demo walks the particle lists of value blocks only
    // (src/msbg_demo.cpp:541-566): a particle owned by a non-value block is never splatted
    if (slot[(int64_t)(iz >> s) * nxy + (int64_t)(iy >> s) * g.nbx + (ix >> s)] < 0) return;
  }
  const float r = g.rScan;
  const int ix1 = max((int)ceilf(__fsub_rn(__fsub_rn(px, r), 0.5f)), 0);
  const int iy1 = max((int)ceilf(__fsub_rn(__fsub_rn(py, r), 0.5f)), 0);
  const int iz1 = max((int)ceilf(__fsub_rn(__fsub_rn(pz, r), 0.5f)), 0);
  const int ix2 = min((int)floorf(__fsub_rn(__fadd_rn(px, r), 0.5f)), g.sx - 1);
  const int iy2 = min((int)floorf(__fsub_rn(__fadd_rn(py, r), 0.5f)), g.sy - 1);
  const int iz2 = min((int)floorf(__fsub_rn(__fadd_rn(pz, r), 0.5f)), g.sz - 1);
  const int nx = ix2 - ix1 + 1, ny = iy2 - iy1 + 1, nz = iz2 - iz1 + 1;
  if (nx <= 0 || ny <= 0 || nz <= 0) return;
  const float x0 = __fsub_rn(px, 0.5f), y0 = __fsub_rn(py, 0.5f), z0 = __fsub_rn(pz, 0.5f);
  const int64_t vpb = (int64_t)1 << (3 * s);

  // blocks touched by the box (<= 2 per axis)
  bool allValue = true;
  {
    const int bxa = ix1 >> s, bxb = ix2 >> s, bya = iy1 >> s, byb = iy2 >> s, bza = iz1 >> s, bzb = iz2 >> s;
    if (lane < 8) {
      const int bx = (lane & 1) ? bxb : bxa, by = (lane & 2) ? byb : bya, bz = (lane & 4) ? bzb : bza;
      allValue = slot[bz * nxy + (int64_t)by * g.nbx + bx] >= 0;
    }
    allValue = __all_sync(0xffffffffu, allValue);
  }
  const int total = nx * ny * nz;
  int abortAt = total;
  if (!allValue) {
    int first = total;
    for (int t = lane; t < total; t += 32) {
      const int lx = t % nx, rest = t / nx, ly = rest % ny, lz = rest / ny;
      const int ix = ix1 + lx, iy = iy1 + ly, iz = iz1 + lz;
      const float dz = __fsub_rn((float)iz, z0), dy = __fsub_rn((float)iy, y0), dx = __fsub_rn((float)ix, x0);
      const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dz, dz), __fmul_rn(dy, dy)), __fmul_rn(dx, dx));
      if (d2 > g.distSqMax) continue;
      const int64_t b = (int64_t)(iz >> s) * nxy + (int64_t)(iy >> s) * g.nbx + (ix >> s);
      if (slot[b] < 0) { first = t; break; }  // lane-local scan order is increasing
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) first = min(first, __shfl_xor_sync(0xffffffffu, first, o));
    abortAt = first;
    if (lane == 0 && abortAt < total) atomicAdd(nAborted, 1ull);
  }
  if (abortAt == total) {
    // Nothing aborts (every touched block holds data): lanes take whole (y, z) rows of
    // the box, skip the rows outside the sphere (dz*dz + dy*dy already exceeds it, and
    // adding dx*dx >= 0 cannot lower a float sum), and find the row's two possible
    // blocks once.
    const int nRows = ny * nz;
    for (int row = lane; row < nRows; row += 32) {
      const int ly = row % ny, lz = row / ny;
      const int iy = iy1 + ly, iz = iz1 + lz;
      const float dz = __fsub_rn((float)iz, z0), dy = __fsub_rn((float)iy, y0);
      const float dzy = __fadd_rn(__fmul_rn(dz, dz), __fmul_rn(dy, dy));
      if (dzy > g.distSqMax) continue;
      const int64_t rowBlk = (int64_t)(iz >> s) * nxy + (int64_t)(iy >> s) * g.nbx;
      const int bxa = ix1 >> s;
      const int64_t sa = (int64_t)slot[rowBlk + bxa] * vpb, sb = (int64_t)slot[rowBlk + (ix2 >> s)] * vpb;
      const int rowVid = ((iz & mask) << (2 * s)) + ((iy & mask) << s);
      for (int ix = ix1; ix <= ix2; ix++) {
        // distSq exactly as the demo forms it: (dz*dz + dy*dy) + dx*dx
        const float dx = __fsub_rn((float)ix, x0);
        const float d2 = __fadd_rn(dzy, __fmul_rn(dx, dx));
        if (d2 > g.distSqMax) continue;
        const int64_t base = (ix >> s) == bxa ? sa : sb;
        atomicMin((int *)(dst + base + rowVid + (ix & mask)), __float_as_int(__fmul_rn(d2, g.distSqMaxInv)));
      }
    }
    return;
  }
  for (int t = lane; t < abortAt; t += 32) {
    const int lx = t % nx, rest = t / nx, ly = rest % ny, lz = rest / ny;
    const int ix = ix1 + lx, iy = iy1 + ly, iz = iz1 + lz;
    // distSq exactly as the demo forms it: (dz*dz + dy*dy) + dx*dx
    const float dz = __fsub_rn((float)iz, z0), dy = __fsub_rn((float)iy, y0), dx = __fsub_rn((float)ix, x0);
    const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dz, dz), __fmul_rn(dy, dy)), __fmul_rn(dx, dx));
    if (d2 > g.distSqMax) continue;
    const int64_t b = (int64_t)(iz >> s) * nxy + (int64_t)(iy >> s) * g.nbx + (ix >> s);
    const int sl = slot[b];
    if (sl < 0) continue;  // unreachable: an earlier in-sphere voxel would have set abortAt
    const int vid = ((iz & mask) << (2 * s)) + ((iy & mask) << s) + (ix & mask);
    const float q = __fmul_rn(d2, g.distSqMaxInv);
    atomicMin((int *)(dst + (int64_t)sl * vpb + vid), __float_as_int(q));
  }
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

__global__ void kFillF32(float *p, int64_t n, float v) {  // 8 per thread and step
  const int64_t n8 = n / 8;
  const float4 q = make_float4(v, v, v, v);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n8; i += (int64_t)gridDim.x * blockDim.x) {
    reinterpret_cast<float4 *>(p)[2 * i] = q;
    reinterpret_cast<float4 *>(p)[2 * i + 1] = q;
  }
  for (int64_t i = 8 * n8 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = v;
}

int splatRun(msbg_gpu_ctx *ctx, const float *dPts, int64_t n, float rParticle, float nbDist) {
  Channel &c = ctx->ch[0];
  const int64_t nVox = ctx->nActive * ctx->voxPerBlock;
  float *dst;
  if (c.storage == MSBG_GPU_F32) {
    dst = (float *)c.d;  // channel was filled with 1.0 by set_refinement_map
  } else {
    int rc = ensureTmpSlab(ctx, (size_t)(nVox > 0 ? nVox : 1) * 4);
    if (rc) return rc;
    dst = (float *)ctx->dTmpSlab;
    if (nVox) MSBG_LAUNCH(ctx, kFillF32, gridVec(nVox), 256, 0, dst, nVox, 1.0f);
  }
  MSBG_CUDA(ctx, cudaMemsetAsync(ctx->dCounters + 1, 0, 8, ctx->stream));
  if (n == 0 || nVox == 0) return MSBG_GPU_OK;
  SplatGeom g;
  g.sx = ctx->sx; g.sy = ctx->sy; g.sz = ctx->sz; g.nbx = ctx->nbx; g.nby = ctx->nby;
  g.log2bs = ctx->log2bs;
  for (int k = 0; k < 3; k++) { g.domMin[k] = ctx->domMin[k]; g.domMax[k] = ctx->domMax[k]; }
  g.rScan = rParticle + nbDist;
  g.distSqMax = g.rScan * g.rScan;
  g.distSqMaxInv = 1.0f / g.distSqMax;
  const int64_t threads = n * 32;
  MSBG_LAUNCH(ctx, kSplat, gridFor(threads, 256), 256, 0, dPts, n, g, ctx->dSlot, dst,
              (unsigned long long *)(ctx->dCounters + 1));
  return MSBG_GPU_OK;
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

}  // namespace msbg
