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
  LevelChannel fl[kMaxLevelChannels];  // cell flags (raw uint16) of the solver's halo
  unsigned long long *dSkip = nullptr;
};

void levelChannelsFree(LevelChannels *lc) {
  if (!lc) return;
  for (LevelChannel *set : {lc->ch, lc->fl})
    for (int i = 0; i < kMaxLevelChannels; i++)
      for (auto &g : set[i].lv) {
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
  int level, bs, log2bs, h, hs;
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

// Four consecutive voxels of a row (16- or 8-byte aligned: x is a multiple of 4).
template <typename T> __device__ __forceinline__ void load4(const T *p, float v[4]);
template <> __device__ __forceinline__ void load4<float>(const float *p, float v[4]) {
  const float4 q = __ldg(reinterpret_cast<const float4 *>(p));
  v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
}
template <> __device__ __forceinline__ void load4<__half>(const __half *p, float v[4]) {
  const uint2 q = __ldg(reinterpret_cast<const uint2 *>(p));
  const float2 lo = __half22float2(*reinterpret_cast<const __half2 *>(&q.x));
  const float2 hi = __half22float2(*reinterpret_cast<const __half2 *>(&q.y));
  v[0] = lo.x; v[1] = lo.y; v[2] = hi.x; v[3] = hi.y;
}
template <> __device__ __forceinline__ void load4<uint16_t>(const uint16_t *p, float v[4]) {
  const uint2 q = __ldg(reinterpret_cast<const uint2 *>(p));
  v[0] = __fmul_rn((float)(q.x & 0xffffu), kU16ToF);
  v[1] = __fmul_rn((float)(q.x >> 16), kU16ToF);
  v[2] = __fmul_rn((float)(q.y & 0xffffu), kU16ToF);
  v[3] = __fmul_rn((float)(q.y >> 16), kU16ToF);
}

__device__ __forceinline__ int nbIndex(int p, int o, int bs) { return p < o ? 0 : (p >= o + bs ? 2 : 1); }

constexpr int kHaloThreads = 256;

template <typename T>
__global__ void __launch_bounds__(kHaloThreads, 8) kFillHalo(HaloArgs a) {
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
  auto resolve = [&](int hx, int hy, int hz) -> Src<T> {
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
  auto value = [&](int hx, int hy, int hz) -> float {
    const Src<T> src = resolve(hx, hy, hz);
    return src.p ? ldRaw<T>(src.p) : src.c;
  };
  const int L = a.log2bs;
  if (bs < 4) {  // every position the general way
    for (int i = threadIdx.x; i < per; i += kHaloThreads) {
      const int q = (int)__umulhi((uint32_t)i, a.hsMagic), hz = (int)__umulhi((uint32_t)q, a.hsMagic);
      dst[i] = value(i - q * hs, q - hz * hs, hz);
    }
    return;
  }
  // Plane by plane through a shared double buffer, so that every output plane (hs^2
  // floats, a multiple of 16 bytes at a 16-byte aligned offset) leaves in whole 16-byte
  // stores and no DRAM sector is written in parts.  Interior rows of an interior plane
  // come from the own block, 4 voxels per thread; the rest of the plane resolves per
  // position.
  extern __shared__ __align__(16) float plane[];
  const int hs2 = hs * hs;
  const int32_t own = stL[13];
  const T *blk = own >= 0 ? (const T *)a.lv.pay + (int64_t)own * bs * bs * bs : nullptr;
  const float cOwn = own == MSBG_GPU_LBLK_EMPTY ? a.lv.emptyF : a.lv.fullF;
  const int nShell = 2 * h * hs + 2 * h * bs;  // halo rows, then halo columns of the block rows
  for (int hz = 0; hz < hs; hz++) {
    float *buf = plane + (hz & 1) * hs2;
    const int z = hz - h;
    if (z < 0 || z >= bs) {
      for (int i = threadIdx.x; i < hs2; i += kHaloThreads) {
        const int hy = (int)__umulhi((uint32_t)i, a.hsMagic);
        buf[i] = value(i - hy * hs, hy, hz);
      }
    } else {
      for (int k = threadIdx.x; k < bs * bs / 4; k += kHaloThreads) {
        const int xq = k & ((bs >> 2) - 1), y = k >> (L - 2);
        float v[4];
        if (blk) load4<T>(blk + (z * bs + y) * bs + 4 * xq, v);
        else v[0] = v[1] = v[2] = v[3] = cOwn;
        float *o = buf + (y + h) * hs + h + 4 * xq;
        o[0] = v[0]; o[1] = v[1]; o[2] = v[2]; o[3] = v[3];
      }
      for (int j = threadIdx.x; j < nShell; j += kHaloThreads) {
        int hx, hy;
        if (j < 2 * h * hs) {
          const int r = (int)__umulhi((uint32_t)j, a.hsMagic);
          hx = j - r * hs;
          hy = r < h ? r : r + bs;
        } else {  // 2h halo columns on each of the bs block rows
          const int jj = j - 2 * h * hs, yb = jj / (2 * h), xx = jj - yb * 2 * h;
          hy = h + yb;
          hx = xx < h ? xx : xx + bs;
        }
        buf[hy * hs + hx] = value(hx, hy, hz);
      }
    }
    __syncthreads();
    float4 *o4 = reinterpret_cast<float4 *>(dst + hz * hs2);
    const float4 *b4 = reinterpret_cast<const float4 *>(buf);
    for (int i = threadIdx.x; i < hs2 / 4; i += kHaloThreads) o4[i] = b4[i];
  }
}

// Restriction of halo boxes ((bs+2)^3, halo 1) to (bs/2)^3 coarse values: the 4^3
// Gauss-like weights (1,3,3,1)^3/512 (src/grid.c:30-70) in the reference's summation
// order (per x offset i and row j, S[j][i] = fma(w, f, S[j][i]) over the 4 planes; then
// T[i] = ((S0+S1)+S2)+S3 and (T0+T1)+(T2+T3)), or the 8-child mean.  One CTA per box,
// one thread per coarse cell (strided); blocks the fill skipped are skipped here too.
template <bool SIMPLE>
__global__ void __launch_bounds__(256) kRestrictBoxes(const float *__restrict__ boxes, const int32_t *__restrict__ bids,
                                                      const int32_t *__restrict__ levels,
                                                      const int32_t *__restrict__ state, int level, int bs,
                                                      float *__restrict__ out) {
  const int bid = bids[blockIdx.x];
  if (levels[bid] != level || state[bid] == MSBG_GPU_LBLK_NONE) return;
  const int hs = bs + 2, cb = bs >> 1;
  const float *b = boxes + (int64_t)blockIdx.x * hs * hs * hs;
  float *o = out + (int64_t)blockIdx.x * cb * cb * cb;
  auto at = [&](int x, int y, int z) { return b[((z + 1) * hs + (y + 1)) * hs + (x + 1)]; };
  for (int c = threadIdx.x; c < cb * cb * cb; c += blockDim.x) {
    const int vx = c % cb, vy = (c / cb) % cb, vz = c / (cb * cb);
    const int x0 = 2 * vx, y0 = 2 * vy, z0 = 2 * vz;
    float val;
    if constexpr (SIMPLE) {
      float sum = at(x0, y0, z0);
#pragma unroll
      for (int k = 1; k < 8; k++) sum = __fadd_rn(sum, at(x0 + (k & 1), y0 + ((k >> 1) & 1), z0 + (k >> 2)));
      val = __fmul_rn(sum, 1.0f / 8.0f);
    } else {
      const float k1[4] = {1.f, 3.f, 3.f, 1.f};
      float S[4][4];
#pragma unroll
      for (int j = 0; j < 4; j++)
#pragma unroll
        for (int i = 0; i < 4; i++) S[j][i] = 0.0f;
#pragma unroll
      for (int k = 0; k < 4; k++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
          for (int i = 0; i < 4; i++)
            S[j][i] = __fmaf_rn(k1[k] * k1[j] * k1[i] / 512.f, at(x0 - 1 + i, y0 - 1 + j, z0 - 1 + k), S[j][i]);
      float T[4];
#pragma unroll
      for (int i = 0; i < 4; i++) T[i] = __fadd_rn(__fadd_rn(__fadd_rn(S[0][i], S[1][i]), S[2][i]), S[3][i]);
      val = __fadd_rn(__fadd_rn(T[0], T[1]), __fadd_rn(T[2], T[3]));
    }
    o[(vz * cb + vy) * cb + vx] = val;
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
  if ((uintptr_t)dOut & 15) return fail(ctx, MSBG_GPU_ERR_ARG, "fill_halo: dOut must be 16-byte aligned");
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
  a.log2bs = ctx->log2bs - level;
  a.h = haloSize;
  a.hs = bs + 2 * haloSize;
  a.hsMagic = (uint32_t)(((1ull << 32) + a.hs - 1) / a.hs);  // exact for every i < hs^3 <= 40^3
  a.sx = ctx->sx >> level; a.sy = ctx->sy >> level; a.sz = ctx->sz >> level;
  a.nbx = ctx->nbx; a.nby = ctx->nby; a.nbz = ctx->nbz;
  a.opt = opt;
  a.out = dOut;
  a.skipped = lc->dSkip;
  const size_t smem = 2 * sizeof(float) * (size_t)a.hs * a.hs;  // the plane double buffer (<= 12.8 KB)
  if (n > 0) {
    switch (c.storage) {
      case MSBG_GPU_F32: MSBG_LAUNCH(ctx, kFillHalo<float>, (unsigned)n, kHaloThreads, smem, a); break;
      case MSBG_GPU_F16: MSBG_LAUNCH(ctx, kFillHalo<__half>, (unsigned)n, kHaloThreads, smem, a); break;
      default: MSBG_LAUNCH(ctx, kFillHalo<uint16_t>, (unsigned)n, kHaloThreads, smem, a); break;
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

extern "C" int msbg_gpu_restrict_level_blocks(msbg_gpu_ctx *ctx, int lchan, int level, const int32_t *dBids,
                                              int64_t n, int simpleAverage, float *dOut, int64_t *hSkipped) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  if (level < 0 || level >= ctx->nLevels || level >= kMaxGridLevels || (ctx->bsx >> level) < 2)
    return fail(ctx, MSBG_GPU_ERR_ARG, "restrict_level: level %d out of range (block edge must be >= 2)", level);
  if (n < 0 || n > 0x7fffffff || (n > 0 && (!dBids || !dOut)))
    return fail(ctx, MSBG_GPU_ERR_ARG, "restrict_level: bad block list");
  if (n == 0) {
    if (hSkipped) *hSkipped = 0;
    return MSBG_GPU_OK;
  }
  if (!ctx->levelCh || lchan < 0 || lchan >= kMaxLevelChannels || !ctx->levelCh->ch[lchan].lv[level].set)
    return fail(ctx, MSBG_GPU_ERR_STATE, "restrict_level: level %d of level channel %d is not set", level, lchan);
  const int bs = ctx->bsx >> level, hs = bs + 2, cb = bs / 2;
  const int64_t box = (int64_t)hs * hs * hs, per = (int64_t)cb * cb * cb;
  const int64_t batch = n < 4096 ? n : 4096;
  float *boxes = nullptr;
  MSBG_CUDA(ctx, cudaMalloc(&boxes, (size_t)(batch * box) * sizeof(float)));
  int rc = MSBG_GPU_OK;
  int64_t skipped = 0;
  const int32_t *state = ctx->levelCh->ch[lchan].lv[level].state;
  for (int64_t k0 = 0; k0 < n && !rc; k0 += batch) {
    const int64_t m = n - k0 < batch ? n - k0 : batch;
    int64_t sk = 0;
    rc = msbg_gpu_fill_halo_blocks(ctx, lchan, level, dBids + k0, m, 1, MSBG_GPU_BC_COARSE_LEVEL, boxes,
                                   hSkipped ? &sk : nullptr);
    if (rc) break;
    skipped += sk;
    if (simpleAverage)
      kRestrictBoxes<true><<<(unsigned)m, 256, 0, ctx->stream>>>(boxes, dBids + k0, ctx->dLevels, state, level, bs,
                                                                  dOut + k0 * per);
    else
      kRestrictBoxes<false><<<(unsigned)m, 256, 0, ctx->stream>>>(boxes, dBids + k0, ctx->dLevels, state, level, bs,
                                                                   dOut + k0 * per);
    ctx->launches++;
    if (cudaGetLastError() != cudaSuccess) rc = fail(ctx, MSBG_GPU_ERR_CUDA, "restrict_level: launch failed");
  }
  // the boxes are read by the kernels above: free only after them
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess && !rc) rc = fail(ctx, MSBG_GPU_ERR_CUDA, "restrict_level: sync");
  cudaFree(boxes);
  if (!rc && hSkipped) *hSkipped = skipped;
  return rc;
}

// =====================================================================================
// HaloBlockSet::fillHaloBlock3 (src/halo.cpp:536-738): the solver's halo, at multigrid
// level 0 with halo 1, for blocks of layout level 0.  Per position p of the (bs+2)^3
// box (level-0 coordinates):
//   p in the domain, its block at layout level 0: flags(0, p) & CELL_VOID -> +1e20
//     (SPEC_FLOAT_DIRICHLET, src/msbgcell.h:199-200), & CELL_SOLID -> -1e20
//     (SPEC_FLOAT_NEUMANN), else value(0, p);
//   p in the domain, its block coarser: the same from level 1 at p/2 (getOutOfBlockValue3,
//     src/halo.cpp:536-562); p/2 lies in the block with p's block coordinates;
//   p outside the domain: +1e20 when the face it leaves through is open, else -1e20, the
//     x face deciding before y before z (the 3x3x3 table, src/msbg.cpp:2527-2548).
// Not a hot kernel (the release calls it nowhere): one CTA per block, one position per
// thread and step.
// =====================================================================================
namespace msbg {
namespace {

constexpr uint16_t kCellSolid = 1u << 0, kCellVoid = 1u << 12;  // src/msbg.h:602-614

struct Halo3Level {
  const int32_t *vState, *fState;
  const void *vPay;
  const uint16_t *fPay;
  float vEmpty, vFull;
  uint16_t fEmpty, fFull;
};

template <typename T>
__global__ void __launch_bounds__(256) kFillHalo3(const int32_t *__restrict__ bids, const int32_t *__restrict__ levels,
                                                  Halo3Level L0, Halo3Level L1, int bs, int sx, int sy, int sz,
                                                  int nbx, int nby, int64_t nBlocks, int4 dbcLo, int4 dbcHi,
                                                  float *__restrict__ out, unsigned long long *__restrict__ skipped) {
  const int hs = bs + 2;
  const int64_t per = (int64_t)hs * hs * hs;
  const int b = bids[blockIdx.x];
  if (b < 0 || b >= nBlocks || levels[b] != 0 || L0.vState[b] == MSBG_GPU_LBLK_NONE) {
    if (threadIdx.x == 0) atomicAdd(skipped, 1ull);
    return;
  }
  const int ox = (b % nbx) * bs, oy = ((b / nbx) % nby) * bs, oz = (int)(b / ((int64_t)nbx * nby)) * bs;
  float *dst = out + (int64_t)blockIdx.x * per;
  for (int64_t i = threadIdx.x; i < per; i += blockDim.x) {
    const int hx = (int)(i % hs), hy = (int)((i / hs) % hs), hz = (int)(i / ((int64_t)hs * hs));
    const int px = ox + hx - 1, py = oy + hy - 1, pz = oz + hz - 1;
    int side = -1;
    if (pz < 0) side = 4; else if (pz >= sz) side = 5;
    if (py < 0) side = 2; else if (py >= sy) side = 3;
    if (px < 0) side = 0; else if (px >= sx) side = 1;
    float v;
    if (side >= 0) {
      const int d = side == 0 ? dbcLo.x : side == 1 ? dbcHi.x : side == 2 ? dbcLo.y : side == 3 ? dbcHi.y
                  : side == 4 ? dbcLo.z : dbcHi.z;
      v = d == 0 ? 1e20f : -1e20f;
    } else {
      const int64_t b2 = (int64_t)(px / bs) + (int64_t)(py / bs) * nbx + (int64_t)(pz / bs) * nbx * nby;
      const int l = levels[b2] == 0 ? 0 : 1;
      const Halo3Level &L = l ? L1 : L0;
      const int bl = bs >> l;
      const int64_t vid = ((int64_t)((pz >> l) & (bl - 1)) * bl + ((py >> l) & (bl - 1))) * bl + ((px >> l) & (bl - 1));
      const int32_t fs = L.fState ? L.fState[b2] : MSBG_GPU_LBLK_NONE;
      const uint16_t f = fs >= 0 ? L.fPay[(int64_t)fs * bl * bl * bl + vid]
                       : fs == MSBG_GPU_LBLK_EMPTY ? L.fEmpty : fs == MSBG_GPU_LBLK_FULL ? L.fFull : (uint16_t)0;
      if (f & kCellVoid) {
        v = 1e20f;
      } else if (f & kCellSolid) {
        v = -1e20f;
      } else {
        const int32_t vs = L.vState ? L.vState[b2] : MSBG_GPU_LBLK_NONE;
        v = vs >= 0 ? ldRaw<T>((const T *)L.vPay + (int64_t)vs * bl * bl * bl + vid)
          : vs == MSBG_GPU_LBLK_EMPTY ? L.vEmpty : vs == MSBG_GPU_LBLK_FULL ? L.vFull : 0.0f;
      }
    }
    dst[i] = v;
  }
}

}  // namespace
}  // namespace msbg

extern "C" int msbg_gpu_level_flags_set(msbg_gpu_ctx *ctx, int fchan, int level, const int32_t *hState,
                                        const uint16_t *hFlags, int64_t nData, uint16_t emptyFlags,
                                        uint16_t fullFlags) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  if (fchan < 0 || fchan >= kMaxLevelChannels)
    return fail(ctx, MSBG_GPU_ERR_ARG, "level_flags_set: flags channel %d out of range", fchan);
  if (level < 0 || level >= ctx->nLevels || level >= kMaxGridLevels || (ctx->bsx >> level) < 1)
    return fail(ctx, MSBG_GPU_ERR_ARG, "level_flags_set: level %d out of range", level);
  if (!hState || nData < 0 || (nData > 0 && !hFlags))
    return fail(ctx, MSBG_GPU_ERR_ARG, "level_flags_set: null or negative argument");
  for (int64_t b = 0; b < ctx->nBlocks; b++)
    if (hState[b] < MSBG_GPU_LBLK_NONE || hState[b] >= nData)
      return fail(ctx, MSBG_GPU_ERR_ARG, "level_flags_set: block %lld has state %d outside [-3, %lld)",
                  (long long)b, hState[b], (long long)nData);
  LevelGrid &g = levelChannels(ctx)->fl[fchan].lv[level];
  g.set = false;
  if (!g.ownState) MSBG_CUDA(ctx, cudaMalloc(&g.ownState, ctx->nBlocks * sizeof(int32_t)));
  const int64_t bs = ctx->bsx >> level;
  const size_t bytes = (size_t)nData * bs * bs * bs * sizeof(uint16_t);
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
  if (bytes) MSBG_CUDA(ctx, cudaMemcpyAsync(g.ownPay, hFlags, bytes, cudaMemcpyHostToDevice, ctx->stream));
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  g.state = g.ownState;
  g.pay = g.ownPay;
  g.emptyF = emptyFlags;  // flag values, exact as floats
  g.fullF = fullFlags;
  g.set = true;
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_fill_halo_blocks3(msbg_gpu_ctx *ctx, int lchan, int fchan, int levelMg, const int32_t *dBids,
                                          int64_t n, const int32_t *hDomainBc, float *dOut, int64_t *hSkipped) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  if (levelMg != 0) return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED, "fill_halo_blocks3: levelMg 0 only");
  if (!hDomainBc || n < 0 || n > 0x7fffffff || (n > 0 && (!dBids || !dOut)))
    return fail(ctx, MSBG_GPU_ERR_ARG, "fill_halo_blocks3: bad arguments");
  if (!ctx->layoutValid) return fail(ctx, MSBG_GPU_ERR_STATE, "fill_halo_blocks3: no block layout");
  if (ctx->nLevels < 2) return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED, "fill_halo_blocks3: needs a level 1");
  if (lchan < 0 || lchan >= kMaxLevelChannels || fchan < 0 || fchan >= kMaxLevelChannels || !ctx->levelCh)
    return fail(ctx, MSBG_GPU_ERR_STATE, "fill_halo_blocks3: channels not set");
  const LevelChannel &vc = ctx->levelCh->ch[lchan];
  const LevelChannel &fc = ctx->levelCh->fl[fchan];
  for (int l = 0; l < 2; l++)
    if (!vc.lv[l].set || !fc.lv[l].set)
      return fail(ctx, MSBG_GPU_ERR_STATE, "fill_halo_blocks3: level %d of the values or the flags is not set", l);
  if (n == 0) {
    if (hSkipped) *hSkipped = 0;
    return MSBG_GPU_OK;
  }
  Halo3Level L[2];
  for (int l = 0; l < 2; l++) {
    L[l].vState = vc.lv[l].state;
    L[l].vPay = vc.lv[l].pay;
    L[l].vEmpty = vc.lv[l].emptyF;
    L[l].vFull = vc.lv[l].fullF;
    L[l].fState = fc.lv[l].state;
    L[l].fPay = (const uint16_t *)fc.lv[l].pay;
    L[l].fEmpty = (uint16_t)fc.lv[l].emptyF;
    L[l].fFull = (uint16_t)fc.lv[l].fullF;
  }
  LevelChannels *lc = levelChannels(ctx);
  if (!lc->dSkip) MSBG_CUDA(ctx, cudaMalloc(&lc->dSkip, sizeof(unsigned long long)));
  MSBG_CUDA(ctx, cudaMemsetAsync(lc->dSkip, 0, sizeof(unsigned long long), ctx->stream));
  const int4 lo = make_int4(hDomainBc[0], hDomainBc[2], hDomainBc[4], 0);
  const int4 hi = make_int4(hDomainBc[1], hDomainBc[3], hDomainBc[5], 0);
  switch (vc.storage) {
    case MSBG_GPU_F32:
      MSBG_LAUNCH(ctx, kFillHalo3<float>, (unsigned)n, 256, 0, dBids, ctx->dLevels, L[0], L[1], ctx->bsx, ctx->sx,
                  ctx->sy, ctx->sz, ctx->nbx, ctx->nby, ctx->nBlocks, lo, hi, dOut, lc->dSkip);
      break;
    case MSBG_GPU_F16:
      MSBG_LAUNCH(ctx, kFillHalo3<__half>, (unsigned)n, 256, 0, dBids, ctx->dLevels, L[0], L[1], ctx->bsx, ctx->sx,
                  ctx->sy, ctx->sz, ctx->nbx, ctx->nby, ctx->nBlocks, lo, hi, dOut, lc->dSkip);
      break;
    default:
      MSBG_LAUNCH(ctx, kFillHalo3<uint16_t>, (unsigned)n, 256, 0, dBids, ctx->dLevels, L[0], L[1], ctx->bsx, ctx->sx,
                  ctx->sy, ctx->sz, ctx->nbx, ctx->nby, ctx->nBlocks, lo, hi, dOut, lc->dSkip);
  }
  if (hSkipped) {
    unsigned long long sk = 0;
    MSBG_CUDA(ctx, cudaMemcpyAsync(&sk, lc->dSkip, sizeof(sk), cudaMemcpyDeviceToHost, ctx->stream));
    MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *hSkipped = (int64_t)sk;
  }
  return MSBG_GPU_OK;
}

// ---- the solver operator on a multi-resolution layout --------------------------------
//
// multiplyLaplacianMatrixOpt (src/msbg3.cpp:1756-1912) with IprocessBlockLaplacian's
// MULTIPLY mode (src/msbg3.cpp:418-1335) for the blocks of one layout level l, every block
// a fluid block at its own level of the X level channel, unit face areas, fluid cells.
// Per cell (h = 2^l): F0 = h X; F1..F6 (x-1, x+1, y-1, y+1, z-1, z+1) = h X of the
// neighbour cell in the block or in a face neighbour at level l (zero outside the domain);
// across a face to a coarser block (level l+1) h times the FP32 product 2/3 X of the one
// coarse cell there, to a finer block (level l-1) h times the FP64 sum of the FP32
// products 1/3 X of the four fine cells there (procNeighMixedRes2, src/msbg3.cpp:46-161,
// in its order of the four).  Y = (1/D) F0 - S where D != 0, else 0; S and Y in the order
// the reference's compiled code evaluates them: in its 4- and 8-wide SIMD paths (block edge
// >= 4) S = (F1+F2) + (F3+F4) + (F5+F6) and Y one fused multiply-add, in its 2-wide path
// (edge 2) S left to right and Y a multiply then a subtraction.  One CTA per listed block;
// not a hot kernel (the multigrid works on the level-0 value blocks).
namespace msbg {
namespace {

constexpr float kCoeffCF = (float)(1.0 / (4 * 0.75));            // DPMR_GRAD_COEFF_CF (src/msbg.h:85)
constexpr float kCoeffFC = (float)(1.0 * 2 * (1.0 / (4 * 0.75)));  // h * 2 * DPMR_GRAD_COEFF_CF, h = 1
constexpr int kMrThreads = 256;

struct MrGrid {
  const int32_t *state;  // null: the level is not set
  const float *pay;
  float emptyF, fullF;
};

struct MrArgs {
  const int32_t *bids;
  const int32_t *levels;  // layout level of every block
  MrGrid x[3];            // X at levels l-1 (finer), l, l+1 (coarser)
  MrGrid d, b;            // the diagonal channel and B at level l (b: residual only)
  int level, bs, log2bs;
  int nbx, nby, nbz, nBlocks;
  float h, hr;
  int residual;
  float *out;
  double *dotPart;        // one FP64 partial per listed block, or null
  unsigned long long *skipped;
};

struct MrSrc {
  const float *pay;  // the block's payload, or null: every cell is cval
  float cval;
  int kind;          // 0 same level, 1 coarser, 2 finer, 3 outside the domain (zeros)
};

__device__ __forceinline__ bool mrResolve(const MrGrid &g, int bid, int bsOfLevel, MrSrc &s) {
  if (!g.state) return false;
  const int st = g.state[bid];
  s.pay = nullptr;
  s.cval = 0.0f;
  if (st >= 0) s.pay = g.pay + (int64_t)st * bsOfLevel * bsOfLevel * bsOfLevel;
  else if (st == MSBG_GPU_LBLK_EMPTY) s.cval = g.emptyF;
  else if (st == MSBG_GPU_LBLK_FULL) s.cval = g.fullF;
  else return false;  // no block at that level: the reference has no data to read there
  return true;
}

// Face f (axis f/2, side f%2) of block bid at level a.level: where its neighbour's cells
// come from.  Returns false when the neighbour has no data where it must be read (a level
// not set, no block there, or a level map that is not regular).
__device__ __forceinline__ bool mrFace(const MrArgs &a, int bid, int f, MrSrc &s) {
  const int axis = f >> 1, side = f & 1;
  int c[3] = {bid % a.nbx, (bid / a.nbx) % a.nby, bid / (a.nbx * a.nby)};
  c[axis] += side ? 1 : -1;
  const int nbd[3] = {a.nbx, a.nby, a.nbz};
  s.kind = 3;
  s.pay = nullptr;
  s.cval = 0.0f;
  if (c[axis] < 0 || c[axis] >= nbd[axis]) return true;
  const int bid2 = c[0] + c[1] * a.nbx + c[2] * a.nbx * a.nby;
  const int l2 = a.levels[bid2];
  if (l2 == a.level) { s.kind = 0; return mrResolve(a.x[1], bid2, a.bs, s); }
  if (l2 == a.level + 1) { s.kind = 1; return mrResolve(a.x[2], bid2, a.bs >> 1, s); }
  if (l2 == a.level - 1) { s.kind = 2; return mrResolve(a.x[0], bid2, a.bs << 1, s); }
  return false;
}

// Halo value of face f at in-plane coordinates (u, v) (x faces (y, z), y faces (x, z),
// z faces (x, y)) of a block of edge bs = 2^lb at spacing h.
__device__ __forceinline__ float mrHalo(const MrSrc &s, int f, int u, int v, int bs, int lb, float h) {
  const int axis = f >> 1, side = f & 1;
  if (s.kind == 3) return 0.0f;
  if (s.kind == 0) {
    const int k = side ? 0 : bs - 1;
    const int idx = axis == 0 ? k + (u << lb) + (v << 2 * lb)
                  : axis == 1 ? u + (k << lb) + (v << 2 * lb) : u + (v << lb) + (k << 2 * lb);
    return __fmul_rn(s.pay ? s.pay[idx] : s.cval, h);
  }
  if (s.kind == 1) {
    const int b2 = bs >> 1, l2 = lb - 1, k = side ? 0 : b2 - 1, cu = u >> 1, cv = v >> 1;
    const int idx = axis == 0 ? k + (cu << l2) + (cv << 2 * l2)
                  : axis == 1 ? cu + (k << l2) + (cv << 2 * l2) : cu + (cv << l2) + (k << 2 * l2);
    return __fmul_rn(__fmul_rn(kCoeffFC, s.pay ? s.pay[idx] : s.cval), h);
  }
  const int b2 = bs << 1, l2 = lb + 1, k = side ? 0 : b2 - 1;
  double sum = 0.0;
#pragma unroll
  for (int q = 0; q < 4; q++) {  // (du, dv) = (0,0), (1,0), (0,1), (1,1)
    const int fu = 2 * u + (q & 1), fv = 2 * v + (q >> 1);
    const int idx = axis == 0 ? k + (fu << l2) + (fv << 2 * l2)
                  : axis == 1 ? fu + (k << l2) + (fv << 2 * l2) : fu + (fv << l2) + (k << 2 * l2);
    sum += (double)__fmul_rn(kCoeffCF, s.pay ? s.pay[idx] : s.cval);
  }
  return __double2float_rn(sum * (double)h);
}

__global__ void __launch_bounds__(kMrThreads) kApplyMultires(MrArgs a) {
  __shared__ MrSrc face[6], own, dg, bb;
  __shared__ int bad;
  const int bid = a.bids[blockIdx.x];
  const int bs = a.bs, lb = a.log2bs;
  if (threadIdx.x == 0) {
    bad = bid < 0 || bid >= a.nBlocks || a.levels[bid] != a.level || !mrResolve(a.x[1], bid, bs, own) || !own.pay ||
          !mrResolve(a.d, bid, bs, dg) || (a.residual && !mrResolve(a.b, bid, bs, bb));
  }
  __syncthreads();
  if (threadIdx.x < 6 && !bad) {
    MrSrc s;
    if (!mrFace(a, bid, threadIdx.x, s)) atomicOr(&bad, 1);
    face[threadIdx.x] = s;
  }
  __syncthreads();
  if (bad) {
    if (threadIdx.x == 0) atomicAdd(a.skipped, 1ull);
    return;
  }
  const float h = a.h;
  auto halo = [&](int f, int u, int v) -> float { return mrHalo(face[f], f, u, v, bs, lb, h); };
  const float *X = own.pay;
  const int n = 1 << 3 * lb, m = bs - 1;
  float *out = a.out + (int64_t)blockIdx.x * n;
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += kMrThreads) {
    const int vx = i & m, vy = (i >> lb) & m, vz = i >> 2 * lb;
    const float F0 = __fmul_rn(X[i], h);
    const float F1 = vx > 0 ? __fmul_rn(X[i - 1], h) : halo(0, vy, vz);
    const float F2 = vx < m ? __fmul_rn(X[i + 1], h) : halo(1, vy, vz);
    const float F3 = vy > 0 ? __fmul_rn(X[i - bs], h) : halo(2, vx, vz);
    const float F4 = vy < m ? __fmul_rn(X[i + bs], h) : halo(3, vx, vz);
    const float F5 = vz > 0 ? __fmul_rn(X[i - bs * bs], h) : halo(4, vx, vy);
    const float F6 = vz < m ? __fmul_rn(X[i + bs * bs], h) : halo(5, vx, vy);
    const float D = dg.pay ? dg.pay[i] : dg.cval;
    float Y = 0.0f;
    if (bs >= 4) {
      const float S = __fadd_rn(__fadd_rn(__fadd_rn(F1, F2), __fadd_rn(F3, F4)), __fadd_rn(F5, F6));
      if (D != 0.0f) Y = __fmaf_rn(__fdiv_rn(1.0f, D), F0, -S);
    } else {
      const float S = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(F1, F2), F3), F4), F5), F6);
      if (D != 0.0f) Y = __fsub_rn(__fmul_rn(__fdiv_rn(1.0f, D), F0), S);
    }
    if (a.residual) Y = __fsub_rn(bb.pay ? bb.pay[i] : bb.cval, Y);
    out[i] = Y;
    acc += (double)Y * (double)__fmul_rn(F0, a.hr);
  }
  if (a.dotPart) {
    __shared__ double warpSum[kMrThreads / 32];
#pragma unroll
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) warpSum[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < kMrThreads / 32; w++) t += warpSum[w];
      a.dotPart[blockIdx.x] = t;
    }
  }
}

// Sum of n FP64 partials in a fixed order (one CTA): the same bits on every run.
__global__ void __launch_bounds__(kMrThreads) kSumPartials(const double *__restrict__ part, int64_t n,
                                                          double *__restrict__ total) {
  __shared__ double s[kMrThreads];
  double t = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += kMrThreads) t += part[i];
  s[threadIdx.x] = t;
  __syncthreads();
  for (int w = kMrThreads / 2; w; w >>= 1) {
    if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = s[0];
}

MrGrid mrGrid(LevelChannels *lc, int lchan, int level, int nLevels) {
  MrGrid g{nullptr, nullptr, 0.0f, 0.0f};
  if (lchan < 0 || level < 0 || level >= nLevels || level >= kMaxGridLevels) return g;
  const LevelChannel &c = lc->ch[lchan];
  const LevelGrid &lg = c.lv[level];
  if (c.storage != MSBG_GPU_F32 || !lg.set) return g;
  g.state = lg.state;
  g.pay = static_cast<const float *>(lg.pay);
  g.emptyF = lg.emptyF;
  g.fullF = lg.fullF;
  return g;
}

}  // namespace
}  // namespace msbg

extern "C" int msbg_gpu_multiply_laplacian_levels(msbg_gpu_ctx *ctx, unsigned options, int level, int lchanX,
                                                  int lchanB, int lchanD, const int32_t *dBids, int64_t n,
                                                  float *dOut, double *pDotprod, int64_t *hSkipped) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  const bool residual = (options & MSBG_GPU_OPT_CALC_RESIDUAL) != 0;
  if (options & ~MSBG_GPU_OPT_CALC_RESIDUAL)
    return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED, "multiply_levels: unsupported option bits 0x%x",
                options & ~MSBG_GPU_OPT_CALC_RESIDUAL);
  if (residual && pDotprod)
    return fail(ctx, MSBG_GPU_ERR_ARG, "multiply_levels: no dot product with the residual (as the reference)");
  if (level < 0 || level >= ctx->nLevels || level >= kMaxGridLevels || (ctx->bsx >> level) < 2)
    return fail(ctx, MSBG_GPU_ERR_ARG, "multiply_levels: level %d out of range (block edge must be >= 2)", level);
  for (int lc : {lchanX, lchanD})
    if (lc < 0 || lc >= kMaxLevelChannels)
      return fail(ctx, MSBG_GPU_ERR_ARG, "multiply_levels: level channel %d out of range", lc);
  if (residual && (lchanB < 0 || lchanB >= kMaxLevelChannels))
    return fail(ctx, MSBG_GPU_ERR_ARG, "multiply_levels: level channel %d out of range", lchanB);
  if (n < 0 || n > 0x7fffffff || (n > 0 && (!dBids || !dOut)))
    return fail(ctx, MSBG_GPU_ERR_ARG, "multiply_levels: bad block list");
  if (!ctx->layoutValid) return fail(ctx, MSBG_GPU_ERR_STATE, "no block layout: call set_refinement_map");
  LevelChannels *lc = levelChannels(ctx);
  MrArgs a;
  a.x[0] = mrGrid(lc, lchanX, level - 1, ctx->nLevels);
  a.x[1] = mrGrid(lc, lchanX, level, ctx->nLevels);
  a.x[2] = mrGrid(lc, lchanX, level + 1, ctx->nLevels);
  a.d = mrGrid(lc, lchanD, level, ctx->nLevels);
  a.b = residual ? mrGrid(lc, lchanB, level, ctx->nLevels) : MrGrid{nullptr, nullptr, 0.0f, 0.0f};
  if (!a.x[1].state || !a.d.state || (residual && !a.b.state))
    return fail(ctx, MSBG_GPU_ERR_STATE,
                "multiply_levels: level %d of an operand's level channel is not set as FP32", level);
  if (n == 0) {
    if (pDotprod) *pDotprod = 0.0;
    if (hSkipped) *hSkipped = 0;
    return MSBG_GPU_OK;
  }
  if (!lc->dSkip) MSBG_CUDA(ctx, cudaMalloc(&lc->dSkip, sizeof(unsigned long long)));
  MSBG_CUDA(ctx, cudaMemsetAsync(lc->dSkip, 0, sizeof(unsigned long long), ctx->stream));
  double *scratch = nullptr;  // partials [n], then the total
  if (pDotprod) MSBG_CUDA(ctx, cudaMallocAsync((void **)&scratch, (size_t)(n + 1) * sizeof(double), ctx->stream));
  a.bids = dBids;
  a.levels = ctx->dLevels;
  a.level = level;
  a.bs = ctx->bsx >> level;
  a.log2bs = ctx->log2bs - level;
  a.nbx = ctx->nbx; a.nby = ctx->nby; a.nbz = ctx->nbz;
  a.nBlocks = (int)ctx->nBlocks;
  a.h = (float)(1 << level);
  a.hr = 1.0f / a.h;
  a.residual = residual;
  a.out = dOut;
  a.dotPart = scratch;
  a.skipped = lc->dSkip;
  int rc = MSBG_GPU_OK;
  kApplyMultires<<<(unsigned)n, kMrThreads, 0, ctx->stream>>>(a);
  ctx->launches++;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && scratch) {
    kSumPartials<<<1, kMrThreads, 0, ctx->stream>>>(scratch, n, scratch + n);
    ctx->launches++;
    e = cudaGetLastError();
  }
  double dot = 0.0;
  unsigned long long sk = 0;
  if (e == cudaSuccess && scratch) e = cudaMemcpyAsync(&dot, scratch + n, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess && hSkipped)
    e = cudaMemcpyAsync(&sk, lc->dSkip, sizeof(sk), cudaMemcpyDeviceToHost, ctx->stream);
  if (scratch) cudaFreeAsync(scratch, ctx->stream);
  if (e == cudaSuccess && (pDotprod || hSkipped)) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) rc = cudaFail(ctx, e, "multiply_levels");
  if (rc == MSBG_GPU_OK) {
    if (pDotprod) *pDotprod = dot;
    if (hSkipped) *hSkipped = (int64_t)sk;
  }
  return rc;
}

// ---- the reference's block smoother on a multi-resolution layout ---------------------
//
// relaxBlockList (src/msbg3.cpp:2170-2239) with IprocessBlockLaplacian's RELAX mode
// (src/msbg3.cpp:1108-1398): one launch per layout level and block parity; a CTA takes a
// listed block of that level and parity, stages it and its halo (the operator's, above) in
// shared memory as h X, and runs blockIter block-local iterations in place: groups of the
// reference's SIMD width (8 cells along x, or the block edge below 8) in z, y, x order,
// backward on alternate iterations, as wavefronts of groups that share no face; the last
// iteration, from the buffer, writes X = Y / h.  Per cell Y = omega (B + S) D +
// (1 - omega) F0 in the order the reference's compiled code evaluates it (its 4- and 8-wide
// paths: S = (F1+F2) + (F3+F4) + (F5+F6), Y = fma(1 - omega, F0, (omega D)(S + B); its
// 2-wide path: source order).
namespace msbg {
namespace {

template <int BS> constexpr int log2Edge() { return BS == 32 ? 5 : BS == 16 ? 4 : BS == 8 ? 3 : BS == 4 ? 2 : 1; }

template <int BS>
__global__ void __launch_bounds__(kMrThreads) kRelaxMultires(MrArgs a, int parity, float omega, int blockIter,
                                                             int reverse, int countOutOfRange) {
  constexpr int HS = BS + 2, HS2 = HS * HS, VPB = BS * BS * BS, LB = log2Edge<BS>();
  constexpr int GW = BS >= 8 ? 8 : BS, G = BS / GW, T = G + 2 * BS - 2;
  extern __shared__ float hb[];
  __shared__ MrSrc face[6], own, dg, bb;
  __shared__ int state;  // 0 relax, 1 another launch's block, 2 skipped
  const int bid = a.bids[blockIdx.x];
  if (threadIdx.x == 0) {
    int st = 0;
    if (bid < 0 || bid >= a.nBlocks) {
      st = countOutOfRange ? 2 : 1;
    } else {
      const int par = (bid % a.nbx + (bid / a.nbx) % a.nby + bid / (a.nbx * a.nby)) & 1;
      if (par != parity || a.levels[bid] != a.level) st = 1;
      else if (!mrResolve(a.x[1], bid, BS, own) || !own.pay || !mrResolve(a.d, bid, BS, dg) ||
               !mrResolve(a.b, bid, BS, bb))
        st = 2;
    }
    state = st;
  }
  __syncthreads();
  if (threadIdx.x < 6 && state == 0) {
    MrSrc s;
    if (!mrFace(a, bid, threadIdx.x, s)) atomicMax(&state, 2);
    face[threadIdx.x] = s;
  }
  __syncthreads();
  if (state) {
    if (state == 2 && threadIdx.x == 0) atomicAdd(a.skipped, 1ull);
    return;
  }
  const float h = a.h;
  float *X = const_cast<float *>(own.pay);  // relaxed in place: no other CTA of this launch reads it
  for (int v = threadIdx.x; v < VPB; v += kMrThreads) {
    const int i = v & (BS - 1), j = (v >> LB) & (BS - 1), k = v >> 2 * LB;
    hb[(k + 1) * HS2 + (j + 1) * HS + i + 1] = __fmul_rn(X[v], h);
  }
  for (int v = threadIdx.x; v < 6 * BS * BS; v += kMrThreads) {
    const int f = v / (BS * BS), p = v % (BS * BS), u = p & (BS - 1), w = p >> LB;
    const int axis = f >> 1, side = f & 1, e = side ? BS + 1 : 0;
    const int idx = axis == 0 ? (w + 1) * HS2 + (u + 1) * HS + e
                  : axis == 1 ? (w + 1) * HS2 + e * HS + u + 1 : e * HS2 + (w + 1) * HS + u + 1;
    hb[idx] = mrHalo(face[f], f, u, w, BS, LB, h);
  }
  __syncthreads();
  const float om1 = __fsub_rn(1.0f, omega);
  auto group = [&](int gi, int j, int k, float *y) {
#pragma unroll
    for (int l = 0; l < GW; l++) {
      const int i = gi * GW + l, c = (k * BS + j) * BS + i;
      const float *p = hb + (k + 1) * HS2 + (j + 1) * HS + i + 1;
      const float F0 = p[0], F1 = p[-1], F2 = p[1], F3 = p[-HS], F4 = p[HS], F5 = p[-HS2], F6 = p[HS2];
      const float B = bb.pay ? bb.pay[c] : bb.cval, D = dg.pay ? dg.pay[c] : dg.cval;
      if constexpr (BS >= 4) {
        const float t = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(F1, F2), __fadd_rn(F3, F4)), __fadd_rn(F5, F6)), B);
        y[l] = __fmaf_rn(om1, F0, __fmul_rn(__fmul_rn(omega, D), t));
      } else {
        const float t = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(F1, F2), F3), F4), F5), F6), B);
        y[l] = __fadd_rn(__fmul_rn(__fmul_rn(omega, t), D), __fmul_rn(om1, F0));
      }
    }
  };
  for (int it = 0; it < blockIter - 1; it++) {
    const bool backward = (it & 1) == reverse;
    for (int t = 0; t < T; t++) {
      for (int q = threadIdx.x; q < BS * BS; q += kMrThreads) {
        const int j0 = q % BS, k0 = q / BS, g0 = t - j0 - k0;
        if (g0 < 0 || g0 >= G) continue;
        const int gi = backward ? G - 1 - g0 : g0, j = backward ? BS - 1 - j0 : j0, k = backward ? BS - 1 - k0 : k0;
        float y[GW];
        group(gi, j, k, y);
        float *o = hb + (k + 1) * HS2 + (j + 1) * HS + gi * GW + 1;
#pragma unroll
        for (int l = 0; l < GW; l++) o[l] = y[l];
      }
      __syncthreads();
    }
  }
  if (blockIter >= 1) {  // the last iteration: every group from the buffer, into X
    const float hr = a.hr;
    for (int q = threadIdx.x; q < G * BS * BS; q += kMrThreads) {
      const int gi = q % G, j = (q / G) % BS, k = q / (G * BS);
      float y[GW];
      group(gi, j, k, y);
      float *o = X + (k * BS + j) * BS + gi * GW;
#pragma unroll
      for (int l = 0; l < GW; l++) o[l] = __fmul_rn(y[l], hr);
    }
  }
}

template <int BS>
int launchRelaxMultires(msbg_gpu_ctx *ctx, const MrArgs &a, unsigned n, int parity, float omega, int blockIter,
                        int reverse, int countOutOfRange) {
  constexpr int smem = (BS + 2) * (BS + 2) * (BS + 2) * (int)sizeof(float);
  static bool attr = false;
  if (!attr) {
    MSBG_CUDA(ctx, cudaFuncSetAttribute(kRelaxMultires<BS>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    attr = true;
  }
  MSBG_LAUNCH(ctx, kRelaxMultires<BS>, n, kMrThreads, smem, a, parity, omega, blockIter, reverse, countOutOfRange);
  return MSBG_GPU_OK;
}

}  // namespace
}  // namespace msbg

extern "C" int msbg_gpu_relax_levels(msbg_gpu_ctx *ctx, int reverseOrder, int lchanX, int lchanB, int lchanD,
                                     const int32_t *dBids, int64_t n, int64_t *hSkipped) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  for (int lc : {lchanX, lchanB, lchanD})
    if (lc < 0 || lc >= kMaxLevelChannels)
      return fail(ctx, MSBG_GPU_ERR_ARG, "relax_levels: level channel %d out of range", lc);
  if (n < 0 || n > 0x7fffffff || (n > 0 && !dBids)) return fail(ctx, MSBG_GPU_ERR_ARG, "relax_levels: bad block list");
  if (!ctx->layoutValid) return fail(ctx, MSBG_GPU_ERR_STATE, "no block layout: call set_refinement_map");
  if (ctx->bsx > 32) return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED, "relax_levels: block edge above 32");
  LevelChannels *lc = levelChannels(ctx);
  if (!lc->dSkip) MSBG_CUDA(ctx, cudaMalloc(&lc->dSkip, sizeof(unsigned long long)));
  MSBG_CUDA(ctx, cudaMemsetAsync(lc->dSkip, 0, sizeof(unsigned long long), ctx->stream));
  bool first = true;
  for (int pass = 0; pass < 2 && n > 0; pass++) {
    // blocks of parity (bx+by+bz)&1 = 1 first, 0 first in the reverse order
    const int parity = (pass == 0) == !reverseOrder ? 1 : 0;
    for (int level = 0; level < ctx->nLevels && level < kMaxGridLevels; level++) {
      const int bs = ctx->bsx >> level;
      if (bs < 2) break;
      MrArgs a;
      a.x[0] = mrGrid(lc, lchanX, level - 1, ctx->nLevels);
      a.x[1] = mrGrid(lc, lchanX, level, ctx->nLevels);
      a.x[2] = mrGrid(lc, lchanX, level + 1, ctx->nLevels);
      a.d = mrGrid(lc, lchanD, level, ctx->nLevels);
      a.b = mrGrid(lc, lchanB, level, ctx->nLevels);
      a.bids = dBids;
      a.levels = ctx->dLevels;
      a.level = level;
      a.bs = bs;
      a.log2bs = ctx->log2bs - level;
      a.nbx = ctx->nbx; a.nby = ctx->nby; a.nbz = ctx->nbz;
      a.nBlocks = (int)ctx->nBlocks;
      a.h = (float)(1 << level);
      a.hr = 1.0f / a.h;
      a.residual = 0;
      a.out = nullptr;
      a.dotPart = nullptr;
      a.skipped = lc->dSkip;
      const int cnt = first ? 1 : 0;
      first = false;
      int rc;
      switch (bs) {
        case 32: rc = launchRelaxMultires<32>(ctx, a, (unsigned)n, parity, ctx->relaxOmega, ctx->relaxBlockIter, reverseOrder ? 1 : 0, cnt); break;
        case 16: rc = launchRelaxMultires<16>(ctx, a, (unsigned)n, parity, ctx->relaxOmega, ctx->relaxBlockIter, reverseOrder ? 1 : 0, cnt); break;
        case 8: rc = launchRelaxMultires<8>(ctx, a, (unsigned)n, parity, ctx->relaxOmega, ctx->relaxBlockIter, reverseOrder ? 1 : 0, cnt); break;
        case 4: rc = launchRelaxMultires<4>(ctx, a, (unsigned)n, parity, ctx->relaxOmega, ctx->relaxBlockIter, reverseOrder ? 1 : 0, cnt); break;
        default: rc = launchRelaxMultires<2>(ctx, a, (unsigned)n, parity, ctx->relaxOmega, ctx->relaxBlockIter, reverseOrder ? 1 : 0, cnt); break;
      }
      if (rc) return rc;
    }
  }
  if (hSkipped) {
    unsigned long long sk = 0;
    MSBG_CUDA(ctx, cudaMemcpyAsync(&sk, lc->dSkip, sizeof(sk), cudaMemcpyDeviceToHost, ctx->stream));
    MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *hSkipped = (int64_t)sk;
  }
  return MSBG_GPU_OK;
}
