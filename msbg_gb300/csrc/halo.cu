// Multi-level channels and the cross-resolution halo fill.
//
// Reference: HaloBlockSet::fillHaloBlock_<T> (src/halo.cpp:266-479) with its
// out-of-block rule getOutOfBlockValue (src/halo.h:270-330), on the per-level
// SparseGrids of a channel (getChannel<T>(msbg, chan, level), src/msbg.h:720).
// The reference fills one block at a time into a per-thread FP32 buffer; here one
// call fills a list of blocks, one CTA per block, into a caller-owned device array.
//
// Level l of a level channel: block edge bs = bsx>>l, domain s = (sx,sy,sz)>>l, the
// block grid of level 0 (src/msbg.cpp:800-812).  Per block a state (payload index,
// constant empty, constant full, or no block) and a payload slab [nData][bs^3].
//
// Position p (level coordinates) of block b's halo box:
//   in the domain, and its block exists at level l   -> that voxel
//   else OPT_BC_NEUMANN                              -> own block at p clamped to it
//   else OPT_BC_COARSE_LEVEL: outside the domain p is clamped to it and read at
//        level l if that block exists; otherwise p/2 at level l+1
//   else                                             -> the level's empty value.
// For p >= 0 inside the domain, the level-(l+1) voxel p/2 lies in the block with the
// same block coordinates as p at level l (bs is even), so both lookups go through one
// 27-entry table of the block's neighbourhood, per level, in shared memory.  The
// reference's clamp of p/2 to the level-(l+1) domain is then a no-op.
//
// Bytes per block: bs^3 S own reads + the halo's neighbour reads, (bs+2h)^3 * 4 written.
#include <math.h>

#include "internal.cuh"

namespace msbg {

constexpr int kMaxLevelChannels = 8;
constexpr int kMaxGridLevels = 8;

struct LevelGrid {
  int32_t *ownState = nullptr;     // [nBlocks], the library's copy
  void *ownPay = nullptr;          // [nData][bs^3], the library's copy
  size_t payCap = 0;               // bytes of ownPay
  const int32_t *state = nullptr;  // what the fill reads: own copies or bound caller arrays
  const void *pay = nullptr;
  float emptyF = 0.0f, fullF = 1.0f;  // constant blocks' values as read back
  bool set = false;
};

struct LevelChannel {
  int storage = -1;
  LevelGrid lv[kMaxGridLevels];
};

struct LevelChannels {
  LevelChannel ch[kMaxLevelChannels];
  unsigned long long *dSkip = nullptr;
};

void levelChannelsFree(LevelChannels *lc) {
  if (!lc) return;
  for (auto &c : lc->ch)
    for (auto &g : c.lv) {
      if (g.ownState) cudaFree(g.ownState);
      if (g.ownPay) cudaFree(g.ownPay);
    }
  if (lc->dSkip) cudaFree(lc->dSkip);
  delete lc;
}

namespace {

struct HaloLevel {
  const int32_t *state;  // null: the level holds no blocks
  const void *pay;
  float emptyF, fullF;
};

struct HaloArgs {
  const int32_t *bids;
  const int32_t *levels;  // layout level of every block
  HaloLevel lv, lo;       // level l and level l+1
  int level, bs, h, hs;
  uint32_t hsMagic;       // ceil(2^32 / hs): i / hs = umulhi(i, hsMagic) for i < hs^3
  int sx, sy, sz;         // level-l domain
  int nbx, nby, nbz;
  int opt;
  float *out;
  unsigned long long *skipped;
};

template <typename T> __device__ __forceinline__ float ldRaw(const T *p);
template <> __device__ __forceinline__ float ldRaw<float>(const float *p) { return __ldg(p); }
template <> __device__ __forceinline__ float ldRaw<uint16_t>(const uint16_t *p) {
  return __fmul_rn((float)__ldg(p), kU16ToF);
}
template <> __device__ __forceinline__ float ldRaw<__half>(const __half *p) { return __half2float(__ldg(p)); }

// Where the value of one box position comes from: a payload element, or a constant.
template <typename T>
struct Src {
  const T *p;  // null: the constant c
  float c;
};

// Source of a block of state st at in-block voxel (x, y, z); st != NONE.
template <typename T>
__device__ __forceinline__ Src<T> blockSrc(const HaloLevel &L, int32_t st, int bs, int x, int y, int z) {
  if (st >= 0) return {(const T *)L.pay + (int64_t)st * bs * bs * bs + ((z * bs + y) * bs + x), 0.0f};
  return {nullptr, st == MSBG_GPU_LBLK_EMPTY ? L.emptyF : L.fullF};
}

__device__ __forceinline__ int nbIndex(int p, int o, int bs) { return p < o ? 0 : (p >= o + bs ? 2 : 1); }

constexpr int kHaloThreads = 256;
constexpr int kHaloUnroll = 8;  // box positions resolved per thread before their loads issue

template <typename T>
__global__ void __launch_bounds__(kHaloThreads) kFillHalo(HaloArgs a) {
  __shared__ int32_t stL[27], stC[27];
  const int bid = a.bids[blockIdx.x];
  const int64_t nxy = (int64_t)a.nbx * a.nby;
  const int64_t nBlocks = nxy * a.nbz;
  if (bid < 0 || bid >= nBlocks || a.levels[bid] != a.level || !a.lv.state ||
      a.lv.state[bid] == MSBG_GPU_LBLK_NONE) {
    if (threadIdx.x == 0) atomicAdd(a.skipped, 1ull);
    return;
  }
  const int bx = (int)(bid % a.nbx), by = (int)((bid / a.nbx) % a.nby), bz = (int)(bid / nxy);
  if (threadIdx.x < 27) {
    const int t = threadIdx.x;
    const int x = bx + t % 3 - 1, y = by + (t / 3) % 3 - 1, z = bz + t / 9 - 1;
    int32_t l = MSBG_GPU_LBLK_NONE, c = MSBG_GPU_LBLK_NONE;
    if (x >= 0 && y >= 0 && z >= 0 && x < a.nbx && y < a.nby && z < a.nbz) {
      const int64_t b = (int64_t)z * nxy + (int64_t)y * a.nbx + x;
      l = a.lv.state[b];
      if (a.lo.state) c = a.lo.state[b];
    }
    stL[t] = l;
    stC[t] = c;
  }
  __syncthreads();
  const int bs = a.bs, h = a.h, hs = a.hs;
  const int ox = bx * bs, oy = by * bs, oz = bz * bs;
  const int per = hs * hs * hs;
  float *dst = a.out + (int64_t)blockIdx.x * per;
  const bool neumann = (a.opt & MSBG_GPU_BC_NEUMANN) != 0;
  const bool coarse = (a.opt & MSBG_GPU_BC_COARSE_LEVEL) != 0;
  const int bsC = bs >> 1;
  auto resolve = [&](int i) -> Src<T> {
    const int q = (int)__umulhi((uint32_t)i, a.hsMagic), hz = (int)__umulhi((uint32_t)q, a.hsMagic);
    const int hx = i - q * hs, hy = q - hz * hs;
    int px = ox + hx - h, py = oy + hy - h, pz = oz + hz - h;
    const bool inRange = px >= 0 && py >= 0 && pz >= 0 && px < a.sx && py < a.sy && pz < a.sz;
    int n = nbIndex(px, ox, bs) + 3 * nbIndex(py, oy, bs) + 9 * nbIndex(pz, oz, bs);
    int32_t st = inRange ? stL[n] : MSBG_GPU_LBLK_NONE;
    if (st != MSBG_GPU_LBLK_NONE) return blockSrc<T>(a.lv, st, bs, px & (bs - 1), py & (bs - 1), pz & (bs - 1));
    if (neumann) {
      const int cx = min(max(px, ox), ox + bs - 1), cy = min(max(py, oy), oy + bs - 1),
                cz = min(max(pz, oz), oz + bs - 1);
      return blockSrc<T>(a.lv, stL[13], bs, cx - ox, cy - oy, cz - oz);
    }
    if (!coarse) return {nullptr, a.lv.emptyF};
    if (!inRange) {
      px = min(max(px, 0), a.sx - 1);
      py = min(max(py, 0), a.sy - 1);
      pz = min(max(pz, 0), a.sz - 1);
      n = nbIndex(px, ox, bs) + 3 * nbIndex(py, oy, bs) + 9 * nbIndex(pz, oz, bs);
      st = stL[n];
      if (st != MSBG_GPU_LBLK_NONE) return blockSrc<T>(a.lv, st, bs, px & (bs - 1), py & (bs - 1), pz & (bs - 1));
    }
    const int32_t sc = stC[n];
    if (sc == MSBG_GPU_LBLK_NONE) return {nullptr, a.lv.emptyF};
    return blockSrc<T>(a.lo, sc, bsC, (px >> 1) & (bsC - 1), (py >> 1) & (bsC - 1), (pz >> 1) & (bsC - 1));
  };
  // kHaloUnroll positions per thread and round: all sources first, then all loads, so
  // that each thread has that many independent reads in flight
  for (int i0 = threadIdx.x; i0 < per; i0 += kHaloThreads * kHaloUnroll) {
    Src<T> src[kHaloUnroll];
#pragma unroll
    for (int u = 0; u < kHaloUnroll; u++) {
      const int i = i0 + u * kHaloThreads;
      src[u] = i < per ? resolve(i) : Src<T>{nullptr, 0.0f};
    }
    float v[kHaloUnroll];
#pragma unroll
    for (int u = 0; u < kHaloUnroll; u++) v[u] = src[u].p ? ldRaw<T>(src[u].p) : src[u].c;
#pragma unroll
    for (int u = 0; u < kHaloUnroll; u++) {
      const int i = i0 + u * kHaloThreads;
      if (i < per) dst[i] = v[u];
    }
  }
}

float quantConst(int storage, float v) {
  switch (storage) {
    case MSBG_GPU_U16: {
      const float q = roundf(v * 65535.0f);
      return (float)(uint16_t)fminf(fmaxf(q, 0.0f), 65535.0f) * kU16ToF;
    }
    case MSBG_GPU_F16: return __half2float(__float2half_rn(v));
    default: return v;
  }
}

LevelChannels *levelChannels(msbg_gpu_ctx *ctx) {
  if (!ctx->levelCh) ctx->levelCh = new LevelChannels();
  return ctx->levelCh;
}

}  // namespace

}  // namespace msbg

using namespace msbg;

extern "C" int msbg_gpu_level_grid_set(msbg_gpu_ctx *ctx, int lchan, int level, int storage,
                                       const int32_t *hState, const void *hPayload, int64_t nData,
                                       float emptyValue, float fullValue) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  if (lchan < 0 || lchan >= kMaxLevelChannels)
    return fail(ctx, MSBG_GPU_ERR_ARG, "level_grid_set: level channel %d out of range", lchan);
  if (level < 0 || level >= ctx->nLevels || level >= kMaxGridLevels || (ctx->bsx >> level) < 1)
    return fail(ctx, MSBG_GPU_ERR_ARG, "level_grid_set: level %d out of range", level);
  if (storage != MSBG_GPU_F32 && storage != MSBG_GPU_F16 && storage != MSBG_GPU_U16)
    return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED, "level_grid_set: storage must be FP32, FP16 or uint16");
  if (!hState || nData < 0 || (nData > 0 && !hPayload))
    return fail(ctx, MSBG_GPU_ERR_ARG, "level_grid_set: null or negative argument");
  for (int64_t b = 0; b < ctx->nBlocks; b++)
    if (hState[b] < MSBG_GPU_LBLK_NONE || hState[b] >= nData)
      return fail(ctx, MSBG_GPU_ERR_ARG, "level_grid_set: block %lld has state %d outside [-3, %lld)",
                  (long long)b, hState[b], (long long)nData);
  LevelChannel &c = levelChannels(ctx)->ch[lchan];
  if (c.storage != storage) {
    for (auto &g : c.lv) g.set = false;
    c.storage = storage;
  }
  LevelGrid &g = c.lv[level];
  g.set = false;
  if (!g.ownState) MSBG_CUDA(ctx, cudaMalloc(&g.ownState, ctx->nBlocks * sizeof(int32_t)));
  const int64_t bs = ctx->bsx >> level;
  const size_t bytes = (size_t)nData * bs * bs * bs * storageBytes(storage);
  if (g.payCap < bytes) {
    MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (g.ownPay) MSBG_CUDA(ctx, cudaFree(g.ownPay));
    g.ownPay = nullptr;
    g.payCap = 0;
    MSBG_CUDA(ctx, cudaMalloc(&g.ownPay, bytes));
    g.payCap = bytes;
  }
  MSBG_CUDA(ctx, cudaMemcpyAsync(g.ownState, hState, ctx->nBlocks * sizeof(int32_t), cudaMemcpyHostToDevice,
                                 ctx->stream));
  if (bytes) MSBG_CUDA(ctx, cudaMemcpyAsync(g.ownPay, hPayload, bytes, cudaMemcpyHostToDevice, ctx->stream));
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // host buffers may go away after the call
  g.state = g.ownState;
  g.pay = g.ownPay;
  g.emptyF = quantConst(storage, emptyValue);
  g.fullF = quantConst(storage, fullValue);
  g.set = true;
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_level_grid_bind(msbg_gpu_ctx *ctx, int lchan, int level, int storage,
                                        const int32_t *dState, const void *dPayload, float emptyValue,
                                        float fullValue) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  if (lchan < 0 || lchan >= kMaxLevelChannels)
    return fail(ctx, MSBG_GPU_ERR_ARG, "level_grid_bind: level channel %d out of range", lchan);
  if (level < 0 || level >= ctx->nLevels || level >= kMaxGridLevels || (ctx->bsx >> level) < 1)
    return fail(ctx, MSBG_GPU_ERR_ARG, "level_grid_bind: level %d out of range", level);
  if (storage != MSBG_GPU_F32 && storage != MSBG_GPU_F16 && storage != MSBG_GPU_U16)
    return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED, "level_grid_bind: storage must be FP32, FP16 or uint16");
  if (!dState) return fail(ctx, MSBG_GPU_ERR_ARG, "level_grid_bind: null state array");
  LevelChannel &c = levelChannels(ctx)->ch[lchan];
  if (c.storage != storage) {
    for (auto &g : c.lv) g.set = false;
    c.storage = storage;
  }
  LevelGrid &g = c.lv[level];
  g.state = dState;
  g.pay = dPayload;
  g.emptyF = quantConst(storage, emptyValue);
  g.fullF = quantConst(storage, fullValue);
  g.set = true;
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_fill_halo_blocks(msbg_gpu_ctx *ctx, int lchan, int level, const int32_t *dBids,
                                         int64_t n, int haloSize, int opt, float *dOut, int64_t *hSkipped) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  if (lchan < 0 || lchan >= kMaxLevelChannels)
    return fail(ctx, MSBG_GPU_ERR_ARG, "fill_halo: level channel %d out of range", lchan);
  if (level < 0 || level >= ctx->nLevels || level >= kMaxGridLevels || (ctx->bsx >> level) < 2)
    return fail(ctx, MSBG_GPU_ERR_ARG, "fill_halo: level %d out of range (block edge must be >= 2)", level);
  const int bs = ctx->bsx >> level;
  if (haloSize < 1 || haloSize > 4 || haloSize > bs)
    return fail(ctx, MSBG_GPU_ERR_ARG, "fill_halo: halo size %d outside [1, min(4, %d)]", haloSize, bs);
  if (opt & ~(MSBG_GPU_BC_NEUMANN | MSBG_GPU_BC_COARSE_LEVEL))
    return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED, "fill_halo: unsupported option bits 0x%x",
                opt & ~(MSBG_GPU_BC_NEUMANN | MSBG_GPU_BC_COARSE_LEVEL));
  if (n < 0 || n > 0x7fffffff || (n > 0 && (!dBids || !dOut)))
    return fail(ctx, MSBG_GPU_ERR_ARG, "fill_halo: bad block list");
  if (!ctx->layoutValid) return fail(ctx, MSBG_GPU_ERR_STATE, "no block layout: call set_refinement_map");
  LevelChannels *lc = levelChannels(ctx);
  LevelChannel &c = lc->ch[lchan];
  if (c.storage < 0 || !c.lv[level].set)
    return fail(ctx, MSBG_GPU_ERR_STATE, "fill_halo: level %d of level channel %d is not set", level, lchan);
  if (!lc->dSkip) MSBG_CUDA(ctx, cudaMalloc(&lc->dSkip, sizeof(unsigned long long)));
  MSBG_CUDA(ctx, cudaMemsetAsync(lc->dSkip, 0, sizeof(unsigned long long), ctx->stream));
  HaloArgs a;
  a.bids = dBids;
  a.levels = ctx->dLevels;
  const LevelGrid &gl = c.lv[level];
  a.lv = {gl.state, gl.pay, gl.emptyF, gl.fullF};
  const bool hasLo = level + 1 < ctx->nLevels && level + 1 < kMaxGridLevels && c.lv[level + 1].set;
  if (hasLo) {
    const LevelGrid &go = c.lv[level + 1];
    a.lo = {go.state, go.pay, go.emptyF, go.fullF};
  } else {
    a.lo = {nullptr, nullptr, 0.0f, 0.0f};
  }
  a.level = level;
  a.bs = bs;
  a.h = haloSize;
  a.hs = bs + 2 * haloSize;
  a.hsMagic = (uint32_t)(((1ull << 32) + a.hs - 1) / a.hs);  // exact for every i < hs^3 <= 40^3
  a.sx = ctx->sx >> level; a.sy = ctx->sy >> level; a.sz = ctx->sz >> level;
  a.nbx = ctx->nbx; a.nby = ctx->nby; a.nbz = ctx->nbz;
  a.opt = opt;
  a.out = dOut;
  a.skipped = lc->dSkip;
  if (n > 0) {
    switch (c.storage) {
      case MSBG_GPU_F32: MSBG_LAUNCH(ctx, kFillHalo<float>, (unsigned)n, kHaloThreads, 0, a); break;
      case MSBG_GPU_F16: MSBG_LAUNCH(ctx, kFillHalo<__half>, (unsigned)n, kHaloThreads, 0, a); break;
      default: MSBG_LAUNCH(ctx, kFillHalo<uint16_t>, (unsigned)n, kHaloThreads, 0, a); break;
    }
  }
  if (hSkipped) {
    unsigned long long s = 0;
    MSBG_CUDA(ctx, cudaMemcpyAsync(&s, lc->dSkip, sizeof(s), cudaMemcpyDeviceToHost, ctx->stream));
    MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *hSkipped = (int64_t)s;
  }
  return MSBG_GPU_OK;
}
