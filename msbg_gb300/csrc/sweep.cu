// Stencil sweeps of applyChannelPdeFast<T> (src/msbg4.cpp:60-957) with the
// OPT_BC_NEUMANN halo of fillHaloBlock_ (src/halo.cpp:266-479).
//
// Schedule (src/msbg4.cpp:384-462): numIter rounded up to even; per iteration
// 8 color passes (in place), 2 red-black passes (in place) or one ping-pong pass.
// Within a pass the blocks are independent: a block of the pass's color only
// reads blocks of other colors (same-color blocks are never 26-neighbours), and
// its own voxels are read before they are written.
//
// The in-place schedules of FP32/FP16/uint16 channels run the streaming kernel
// of sweep_color.cu; this file's gather kernel serves the ping-pong schedule and
// FP64 channels.
//
// Gather kernel: one CTA per block of the pass.  The CTA marches through the block in
// z with a ring of three halo'd planes ((bs+2)^2 values each, compute type) in
// shared memory: plane z+1 is gathered (own block, neighbour blocks, the
// constant empty value for non-value blocks, Neumann clamp outside the domain),
// then plane z is computed from planes z-1..z+1 and stored in place.  A plane of
// the own block is always in shared memory before the store that overwrites it.
#include "internal.cuh"
#include "sweep_common.cuh"

namespace msbg {

struct SweepGeom {
  int sx, sy, sz, nbx, nby;
  double emptyValue;
  SweepParams p;
};

template <typename T, typename R>
__device__ __forceinline__ R loadAs(const T *p) {
  return (R)Store<T>::load(p);
}

template <typename T, typename R>
__device__ __forceinline__ void storeSweep(T *p, R v) {
  if constexpr (sizeof(T) == 8) {
    *p = v;
  } else {
    Store<T>::storeRNE(p, (float)v);
  }
}

template <typename T, typename R, int BS, bool EXACT>
__global__ void __launch_bounds__(256) kSweep(const int32_t *__restrict__ bids, const int32_t *__restrict__ slot,
                                              const T *__restrict__ src, T *__restrict__ dst, SweepGeom g) {
  constexpr int HS = BS + 2, HS2 = HS * HS;
  constexpr int LOG = BS == 8 ? 3 : BS == 16 ? 4 : 5;
  constexpr int64_t VPB = (int64_t)BS * BS * BS;
  constexpr int NT = BS * BS < 256 ? BS * BS : 256;
  __shared__ R ring[3][HS2];

  const int tid = threadIdx.x;
  const int bid = bids[blockIdx.x];
  const int64_t nxy = (int64_t)g.nbx * g.nby;
  const int bz = (int)(bid / nxy), by = (int)((bid / g.nbx) % g.nby), bx = (int)(bid % g.nbx);
  const int x0 = bx * BS, y0 = by * BS, z0 = bz * BS;
  const int64_t own = (int64_t)slot[bid] * VPB;
  const R empty = (R)g.emptyValue;

  auto loadPlane = [&](int z, R *pl) {
    const int zg = z0 + z;
    for (int e = tid; e < HS2; e += NT) {
      const int hx = e % HS, hy = e / HS;
      int x = x0 + hx - 1, y = y0 + hy - 1, zz = zg;
      R v;
      if (x >= 0 && x < g.sx && y >= 0 && y < g.sy && zz >= 0 && zz < g.sz) {
        const int sl = slot[(int64_t)(zz >> LOG) * nxy + (int64_t)(y >> LOG) * g.nbx + (x >> LOG)];
        const int vid = ((zz & (BS - 1)) << (2 * LOG)) + ((y & (BS - 1)) << LOG) + (x & (BS - 1));
        v = sl < 0 ? empty : loadAs<T, R>(src + (int64_t)sl * VPB + vid);
      } else {  // OPT_BC_NEUMANN: nearest voxel of the block itself
        x = min(max(x, x0), x0 + BS - 1) - x0;
        y = min(max(y, y0), y0 + BS - 1) - y0;
        zz = min(max(zz, z0), z0 + BS - 1) - z0;
        v = loadAs<T, R>(src + own + ((zz * BS + y) * BS + x));
      }
      pl[e] = v;
    }
  };

  loadPlane(-1, ring[0]);
  loadPlane(0, ring[1]);
  for (int z = 0; z < BS; z++) {
    loadPlane(z + 1, ring[(z + 2) % 3]);
    __syncthreads();
    const R *pm = ring[z % 3], *pc = ring[(z + 1) % 3], *pp = ring[(z + 2) % 3];
    for (int e = tid; e < BS * BS; e += NT) {
      const int x = e % BS, y = e / BS;
      const int c = (y + 1) * HS + (x + 1);
      auto F = [&](int dx, int dy, int dz) -> R {
        const R *pl = dz < 0 ? pm : dz > 0 ? pp : pc;
        return pl[c + dy * HS + dx];
      };
      R out = g.p.kind == K_MCF ? mcfExact<R>(F, (R)g.p.dt) : stencil7<R>(F, g.p);
      if (g.p.constr01) {
        out = out > (R)0 ? out : (R)0;
        out = out < (R)1 ? out : (R)1;
      }
      storeSweep<T, R>(dst + own + ((int64_t)z * BS + y) * BS + x, out);
    }
    __syncthreads();
  }
}

template <typename T, typename R, int BS, bool EXACT>
static int launchSweep(msbg_gpu_ctx *ctx, const int32_t *dBids, int n, const T *src, T *dst,
                       const SweepGeom &g) {
  if (n <= 0) return MSBG_GPU_OK;
  constexpr int NT = BS * BS < 256 ? BS * BS : 256;
  MSBG_LAUNCH(ctx, (kSweep<T, R, BS, EXACT>), (unsigned)n, NT, 0, dBids, ctx->dSlot, src, dst, g);
  return MSBG_GPU_OK;
}

template <typename T, typename R, bool EXACT>
static int launchSweepBS(msbg_gpu_ctx *ctx, const int32_t *dBids, int n, const T *src, T *dst,
                         const SweepGeom &g) {
  switch (ctx->bsx) {
    case 8: return launchSweep<T, R, 8, EXACT>(ctx, dBids, n, src, dst, g);
    case 16: return launchSweep<T, R, 16, EXACT>(ctx, dBids, n, src, dst, g);
    default: return launchSweep<T, R, 32, EXACT>(ctx, dBids, n, src, dst, g);
  }
}

static int launchTyped(msbg_gpu_ctx *ctx, int storage, bool exact, const int32_t *dBids, int n,
                       const void *src, void *dst, const SweepGeom &g) {
  switch (storage) {
    case MSBG_GPU_F32:
      return exact ? launchSweepBS<float, float, true>(ctx, dBids, n, (const float *)src, (float *)dst, g)
                   : launchSweepBS<float, float, false>(ctx, dBids, n, (const float *)src, (float *)dst, g);
    case MSBG_GPU_U16:
      return exact ? launchSweepBS<uint16_t, float, true>(ctx, dBids, n, (const uint16_t *)src, (uint16_t *)dst, g)
                   : launchSweepBS<uint16_t, float, false>(ctx, dBids, n, (const uint16_t *)src, (uint16_t *)dst, g);
    case MSBG_GPU_F16:
      return exact ? launchSweepBS<__half, float, true>(ctx, dBids, n, (const __half *)src, (__half *)dst, g)
                   : launchSweepBS<__half, float, false>(ctx, dBids, n, (const __half *)src, (__half *)dst, g);
    default:
      return launchSweepBS<double, double, true>(ctx, dBids, n, (const double *)src, (double *)dst, g);
  }
}

// Listed blocks of the colour lists: flag[i] = the block at dColorBids[i] is listed.
__global__ void kMarkList(const int32_t *__restrict__ list, int64_t n, int64_t nBlocks, int32_t *__restrict__ mark,
                          int32_t *__restrict__ bad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int b = list[i];
  if (b < 0 || b >= nBlocks) atomicAdd(bad, 1);
  else mark[b] = 1;
}
__global__ void kListedFlags(const int32_t *__restrict__ bids, int64_t n, const int32_t *__restrict__ mark,
                             int32_t *__restrict__ flag) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flag[i] = mark[bids[i]];
}
__global__ void kListedScatter(const int32_t *__restrict__ bids, const int32_t *__restrict__ flag,
                               const int64_t *__restrict__ off, int64_t n, int32_t *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && flag[i]) out[off[i]] = bids[i];
}
// new colour starts: the scan offset at each old colour start, and the total
__global__ void kListedStarts(const int64_t *__restrict__ off, const int64_t *__restrict__ total, int64_t n,
                              const int *__restrict__ starts, int64_t *__restrict__ out) {
  const int c = threadIdx.x;
  if (c < 8) out[c] = starts[c] < n ? off[starts[c]] : *total;
  if (c == 8) out[8] = *total;
}

// The colour lists restricted to the listed blocks (stable, so each colour keeps its
// ascending order): into ctx->dListBids with starts cs[0..8].
static int listedColourLists(msbg_gpu_ctx *ctx, const int32_t *dList, int64_t nList, int cs[9]) {
  const int64_t nB = ctx->nBlocks, nAct = ctx->nActive;
  if (!ctx->dListMark) MSBG_CUDA(ctx, cudaMalloc(&ctx->dListMark, (size_t)nB * 4));
  if (!ctx->dListBids) MSBG_CUDA(ctx, cudaMalloc(&ctx->dListBids, (size_t)nB * 4));
  int rc = ensureTmpSlab(ctx, (size_t)(nAct + 1) * 12 + 256);
  if (rc) return rc;
  int32_t *flag = (int32_t *)ctx->dTmpSlab;
  int64_t *off = (int64_t *)((char *)ctx->dTmpSlab + (((size_t)(nAct + 1) * 4 + 15) & ~size_t(15)));
  int64_t *aux = off + nAct + 1;  // [0]: total, [1..9]: starts, [10]: bad ids (as int32)
  int *dStarts = (int *)(aux + 12);
  MSBG_CUDA(ctx, cudaMemsetAsync(ctx->dListMark, 0, (size_t)nB * 4, ctx->stream));
  MSBG_CUDA(ctx, cudaMemsetAsync(aux, 0, 12 * 8, ctx->stream));
  if (nList > 0)
    MSBG_LAUNCH(ctx, kMarkList, gridFor(nList, 256), 256, 0, dList, nList, nB, ctx->dListMark, (int32_t *)(aux + 10));
  MSBG_CUDA(ctx, cudaMemcpyAsync(dStarts, ctx->colorStart, 9 * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  if (nAct > 0) {
    MSBG_LAUNCH(ctx, kListedFlags, gridFor(nAct, 256), 256, 0, ctx->dColorBids, nAct, ctx->dListMark, flag);
    if ((rc = exclusiveScanFlags(ctx, flag, nAct, off, aux))) return rc;
    MSBG_LAUNCH(ctx, kListedScatter, gridFor(nAct, 256), 256, 0, ctx->dColorBids, flag, off, nAct, ctx->dListBids);
    MSBG_LAUNCH(ctx, kListedStarts, 1, 32, 0, off, aux, nAct, dStarts, aux + 1);
  }
  int64_t h[11] = {};
  if ((rc = readSmall(ctx, h, aux, 11 * 8))) return rc;
  if ((int32_t)h[10]) return fail(ctx, MSBG_GPU_ERR_ARG, "block list holds ids outside the block grid");
  for (int c = 0; c <= 8; c++) cs[c] = nAct > 0 ? (int)h[1 + c] : 0;
  return MSBG_GPU_OK;
}

int pdeRun(msbg_gpu_ctx *ctx, int chan, int laplTyp, int constr01, int numIter, float dt, float anisAlpha,
           int variant, const int32_t *dList, int64_t nList) {
  bool color8 = false, redBlack = false;
  int kind = laplTyp;
  if (kind < 0) {  // src/msbg4.cpp:100-114
    kind = -kind;
    if (kind & MSBG_GPU_OPT_8_COLOR_SCHEME) {
      kind &= ~MSBG_GPU_OPT_8_COLOR_SCHEME;
      color8 = true;
    } else {
      redBlack = true;
    }
  }
  if (!(kind == K_MCF || kind == K_JACOBI || kind == K_PM_JACOBI || kind == K_PM || kind == K_DIFF ||
        kind == K_LAPL))
    return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED, "laplTyp %d not implemented", laplTyp);
  if ((kind == K_PM || kind == K_PM_JACOBI) && !(anisAlpha > 0))
    return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED, "Perona-Malik needs anisDiffAlpha > 0");
  if (variant != MSBG_GPU_SWEEP_EXACT && variant != MSBG_GPU_SWEEP_FAST)
    return fail(ctx, MSBG_GPU_ERR_ARG, "variant %d", variant);
  Channel &c = ctx->ch[chan];
  const bool exact = variant == MSBG_GPU_SWEEP_EXACT;
  SweepGeom g;
  g.sx = ctx->sx; g.sy = ctx->sy; g.sz = ctx->sz; g.nbx = ctx->nbx; g.nby = ctx->nby;
  g.emptyValue = 0.0;
  g.p.kind = kind;
  g.p.constr01 = constr01 ? 1 : 0;
  g.p.dt = dt;
  g.p.anisAlpha = anisAlpha;
  const int nIter0 = numIter;
  int nIter = numIter;
  if (nIter % 2 == 1) nIter++;  // src/msbg4.cpp:150-152
  const int32_t *cb = ctx->dColorBids;
  const int *cs = ctx->colorStart;
  int listStarts[9];
  if (dList) {
    const int rc = listedColourLists(ctx, dList, nList, listStarts);
    if (rc) return rc;
    cb = ctx->dListBids;
    cs = listStarts;
  }
  if ((color8 || redBlack) && c.storage != MSBG_GPU_F64) {
    // streaming kernel with the x-face cache (sweep_color.cu)
    const int rc = colorSweepRun(ctx, c, exact, color8, nIter, g.p, cb, cs);
    if (rc < 0) return rc;
    if (rc == 0) {
      // the streaming kernel's bounded shared-memory waits report through dStatus
      int st = 0;
      if (const int r = readSmall(ctx, &st, ctx->dStatus, sizeof(int))) return r;
      if (st) {
        MSBG_CUDA(ctx, cudaMemsetAsync(ctx->dStatus, 0, sizeof(int), ctx->stream));
        return fail(ctx, MSBG_GPU_ERR_TIMEOUT, "a sweep CTA gave up waiting for its tile (status %d)", st);
      }
      return MSBG_GPU_OK;
    }
  }
  if (color8 || redBlack) {
    // red-black pass 0 processes parity-1 blocks, pass 1 parity-0 (src/msbg4.cpp:447-454);
    // parity = popcount(color) & 1
    static const int rbOrder[2][4] = {{1, 2, 4, 7}, {0, 3, 5, 6}};
    for (int it = 0; it < nIter; it++) {
      if (color8) {
        for (int col = 0; col < 8; col++) {
          int rc = launchTyped(ctx, c.storage, exact, cb + cs[col], cs[col + 1] - cs[col], c.d, c.d, g);
          if (rc) return rc;
        }
      } else {
        for (int pass = 0; pass < 2; pass++)
          for (int k = 0; k < 4; k++) {
            const int col = rbOrder[pass][k];
            int rc = launchTyped(ctx, c.storage, exact, cb + cs[col], cs[col + 1] - cs[col], c.d, c.d, g);
            if (rc) return rc;
          }
      }
    }
    return MSBG_GPU_OK;
  }
  // ping-pong through the temp slab over the whole block set, or over the listed value
  // blocks with both buffers holding the unlisted blocks' values
  const size_t bytes = (size_t)ctx->nActive * ctx->voxPerBlock * storageBytes(c.storage);
  const int32_t *pbids = dList ? cb : ctx->dActive;
  const int pn = dList ? cs[8] : (int)ctx->nActive;
  void *tmp = nullptr;
  if (dList) {  // the colour-list scratch above lives in the temp slab: a slab of its own
    if (bytes) MSBG_CUDA(ctx, cudaMallocAsync(&tmp, bytes, ctx->stream));
    if (bytes) MSBG_CUDA(ctx, cudaMemcpyAsync(tmp, c.d, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
  } else {
    int rc = ensureTmpSlab(ctx, bytes ? bytes : 1);
    if (rc) return rc;
    tmp = ctx->dTmpSlab;
  }
  void *bufs[2] = {c.d, tmp};
  int cur = 0, rc = MSBG_GPU_OK;
  for (int it = 0; it < nIter && !rc; it++) {
    const bool copyOnly = it == nIter - 1 && (nIter0 % 2) == 1;
    if (copyOnly) {
      if (bytes && cudaMemcpyAsync(bufs[cur ^ 1], bufs[cur], bytes, cudaMemcpyDeviceToDevice, ctx->stream) != cudaSuccess)
        rc = fail(ctx, MSBG_GPU_ERR_CUDA, "ping-pong copy failed");
    } else {
      rc = launchTyped(ctx, c.storage, exact, pbids, pn, bufs[cur], bufs[cur ^ 1], g);
    }
    cur ^= 1;
  }
  if (dList && tmp) cudaFreeAsync(tmp, ctx->stream);
  return rc;
}

}  // namespace msbg
