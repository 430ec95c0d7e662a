// Stencil sweeps of applyChannelPdeFast<T> (src/msbg4.cpp:60-957) with the
// OPT_BC_NEUMANN halo of fillHaloBlock_ (src/halo.cpp:266-479).
//
// Schedule (src/msbg4.cpp:384-462): numIter rounded up to even; per iteration
// 8 color passes (in place), 2 red-black passes (in place) or one ping-pong pass.
// Within a pass the blocks are independent: a block of the pass's color only
// reads blocks of other colors (same-color blocks are never 26-neighbours), and
// its own voxels are read before they are written.
//
// Kernel: one CTA per block of the pass.  The CTA marches through the block in
// z with a ring of three halo'd planes ((bs+2)^2 values each, compute type) in
// shared memory: plane z+1 is gathered (own block, neighbour blocks, the
// constant empty value for non-value blocks, Neumann clamp outside the domain),
// then plane z is computed from planes z-1..z+1 and stored in place.  A plane of
// the own block is always in shared memory before the store that overwrites it.
#include "internal.cuh"

namespace msbg {

enum { K_MCF = 4, K_JACOBI = 17, K_PM_JACOBI = 15, K_PM = 14, K_DIFF = 3, K_LAPL = 1 };

struct SweepGeom {
  int sx, sy, sz, nbx, nby;
  double emptyValue;
  int kind, constr01;
  float dt, anisAlpha;
};

// Correctly rounded scalar ops; no contraction, so results follow the written
// expression order exactly (the reference's and the CPU restatement's).
template <typename R> struct Op;
template <> struct Op<float> {
  static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
  static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
  static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
  static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
  static __device__ __forceinline__ float sqrt_(float a) { return __fsqrt_rn(a); }
};
template <> struct Op<double> {
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
  static __device__ __forceinline__ double sqrt_(double a) { return __dsqrt_rn(a); }
};

// Mean curvature flow update, laplTyp 4 (src/msbg4.cpp:559-637), in the
// reference's expression order.  P(dx,dy,dz) reads the halo'd planes.
template <typename R, typename P>
__device__ __forceinline__ R mcfExact(const P &F, R dt) {
  using O = Op<R>;
  const R h = (R)0.5, two = (R)2;
  const R f0 = F(0, 0, 0), f1 = F(-1, 0, 0), f2 = F(1, 0, 0), f3 = F(0, -1, 0), f4 = F(0, 1, 0),
          f5 = F(0, 0, -1), f6 = F(0, 0, 1);
  const R fx = O::mul(h, O::sub(f2, f1)), fy = O::mul(h, O::sub(f4, f3)), fz = O::mul(h, O::sub(f6, f5));
  const R f02 = O::mul(two, f0);
  const R fxx = O::sub(O::add(f1, f2), f02), fyy = O::sub(O::add(f3, f4), f02),
          fzz = O::sub(O::add(f5, f6), f02);
  const R fy_r = O::mul(O::sub(F(1, 1, 0), F(1, -1, 0)), h);
  const R fy_l = O::mul(O::sub(F(-1, 1, 0), F(-1, -1, 0)), h);
  const R fz_r = O::mul(O::sub(F(1, 0, 1), F(1, 0, -1)), h);
  const R fz_l = O::mul(O::sub(F(-1, 0, 1), F(-1, 0, -1)), h);
  const R fz_u = O::mul(O::sub(F(0, 1, 1), F(0, 1, -1)), h);
  const R fz_d = O::mul(O::sub(F(0, -1, 1), F(0, -1, -1)), h);
  const R fyx = O::mul(O::sub(fy_r, fy_l), h), fzx = O::mul(O::sub(fz_r, fz_l), h),
          fzy = O::mul(O::sub(fz_u, fz_d), h);
  const R xx = O::mul(fx, fx), yy = O::mul(fy, fy), zz = O::mul(fz, fz);
  R H = O::add(O::add(O::mul(O::add(yy, zz), fxx), O::mul(O::add(xx, zz), fyy)), O::mul(O::add(xx, yy), fzz));
  const R cross = O::add(O::add(O::mul(O::mul(fx, fy), fyx), O::mul(O::mul(fx, fz), fzx)),
                         O::mul(O::mul(fy, fz), fzy));
  H = O::sub(H, O::mul(two, cross));
  const R g2 = O::add(O::add(xx, yy), zz);
  H = g2 > (R)1e-7f ? O::div(H, g2) : (R)0;
  R D = O::mul(dt, H);
  D = D < (R)-0.1f ? (R)-0.1f : D;
  D = D > (R)0.1f ? (R)0.1f : D;
  return O::add(f0, D);
}

// Same PDE, re-associated for fused multiply-adds (float only).  Uses unscaled
// central differences g = 2*f_x and G = 4*f_xy:
//   H |grad|^2 = |g|^2 lap/4 - (gx^2 fxx + gy^2 fyy + gz^2 fzz)/4 - (gx gy Gyx + ...)/8
// with |grad|^2 = |g|^2/4.
template <typename P>
__device__ __forceinline__ float mcfFast(const P &F, float dt) {
  const float f0 = F(0, 0, 0), f1 = F(-1, 0, 0), f2 = F(1, 0, 0), f3 = F(0, -1, 0), f4 = F(0, 1, 0),
              f5 = F(0, 0, -1), f6 = F(0, 0, 1);
  const float gx = f2 - f1, gy = f4 - f3, gz = f6 - f5;
  const float fxx = fmaf(-2.0f, f0, f1 + f2), fyy = fmaf(-2.0f, f0, f3 + f4),
              fzz = fmaf(-2.0f, f0, f5 + f6);
  const float Gyx = (F(1, 1, 0) - F(1, -1, 0)) - (F(-1, 1, 0) - F(-1, -1, 0));
  const float Gzx = (F(1, 0, 1) - F(1, 0, -1)) - (F(-1, 0, 1) - F(-1, 0, -1));
  const float Gzy = (F(0, 1, 1) - F(0, 1, -1)) - (F(0, -1, 1) - F(0, -1, -1));
  const float xx = gx * gx, yy = gy * gy, zz = gz * gz;
  const float g2 = xx + yy + zz;  // 4 |grad f|^2
  const float lap = fxx + fyy + fzz;
  const float s = fmaf(xx, fxx, fmaf(yy, fyy, zz * fzz));
  const float n1 = fmaf(g2, lap, -s);                         // 4 * (first part)
  const float n2 = fmaf(gx, fmaf(gy, Gyx, gz * Gzx), gy * gz * Gzy);  // 16 * cross
  // H = (n1/4 - n2/8) / (g2/4) = (n1 - n2/2) / g2
  const float Hn = fmaf(-0.5f, n2, n1);
  float H = g2 > 4e-7f ? __fdividef(Hn, g2) : 0.0f;
  float D = fminf(fmaxf(dt * H, -0.1f), 0.1f);
  return f0 + D;
}

// 7-point kernels (src/msbg4.cpp:681-805).
template <typename R, typename P>
__device__ __forceinline__ R stencil7(const P &F, const SweepGeom &g) {
  using O = Op<R>;
  const R dt = (R)g.dt;
  const R phi = F(0, 0, 0);
  const R F1 = F(-1, 0, 0), F2 = F(1, 0, 0), F3 = F(0, -1, 0), F4 = F(0, 1, 0), F5 = F(0, 0, -1),
          F6 = F(0, 0, 1);
  switch (g.kind) {
    case K_JACOBI: {
      const R s6 = O::add(O::add(O::add(O::add(O::add(F1, F2), F3), F4), F5), F6);
      return O::div(O::add(phi, O::mul(dt, s6)), O::add((R)1, O::mul(dt, (R)6)));
    }
    case K_DIFF: {
      const R s6 = O::add(O::add(O::add(O::add(O::add(F1, F2), F3), F4), F5), F6);
      const R S = O::mul((R)1 / (R)6, s6);
      return O::add(phi, O::mul(dt, O::sub(S, phi)));
    }
    case K_LAPL: {
      const R s6 = O::add(O::add(O::add(O::add(O::add(F1, F2), F3), F4), F5), F6);
      const R L = O::sub(s6, O::mul((R)6, phi));
      const R GX = O::mul((R)0.5, O::sub(F2, F1)), GY = O::mul((R)0.5, O::sub(F4, F3)),
              GZ = O::mul((R)0.5, O::sub(F6, F5));
      const R G = O::sqrt_(O::add(O::add(O::mul(GX, GX), O::mul(GY, GY)), O::mul(GZ, GZ)));
      return O::add(phi, O::mul(O::mul(dt, L), G));
    }
    default: {  // K_PM_JACOBI / K_PM, anisAlpha > 0 (src/msbg4.cpp:738-790)
      const R a = (R)g.anisAlpha;
      const R fn[6] = {F1, F2, F3, F4, F5, F6};
      R sum = 0, wsum = 0, dsum = 0;
#pragma unroll
      for (int k = 0; k < 6; k++) {
        const R gk = O::sub(fn[k], phi);
        const R ag = gk < (R)0 ? -gk : gk;
        const R t = O::div(ag, a);
        const R Gk = O::div((R)1, O::add((R)1, O::mul(t, t)));
        sum = O::add(sum, O::mul(Gk, fn[k]));
        wsum = O::add(wsum, Gk);
        dsum = O::add(dsum, O::mul(Gk, gk));
      }
      if (g.kind == K_PM_JACOBI) return O::div(O::add(phi, O::mul(dt, sum)), O::add((R)1, O::mul(dt, wsum)));
      return O::add(phi, O::mul(dt, dsum));
    }
  }
}

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
      R out;
      if (g.kind == K_MCF) {
        if constexpr (EXACT || sizeof(R) == 8) out = mcfExact<R>(F, (R)g.dt);
        else out = mcfFast(F, g.dt);
      } else {
        out = stencil7<R>(F, g);
      }
      if (g.constr01) {
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

int pdeRun(msbg_gpu_ctx *ctx, int chan, int laplTyp, int constr01, int numIter, float dt, float anisAlpha,
           int variant) {
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
  g.kind = kind;
  g.constr01 = constr01 ? 1 : 0;
  g.dt = dt;
  g.anisAlpha = anisAlpha;
  const int nIter0 = numIter;
  int nIter = numIter;
  if (nIter % 2 == 1) nIter++;  // src/msbg4.cpp:150-152
  const int32_t *cb = ctx->dColorBids;
  const int *cs = ctx->colorStart;
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
  // ping-pong through the temp slab; the active list is the whole block set
  const size_t bytes = (size_t)ctx->nActive * ctx->voxPerBlock * storageBytes(c.storage);
  int rc = ensureTmpSlab(ctx, bytes ? bytes : 1);
  if (rc) return rc;
  void *bufs[2] = {c.d, ctx->dTmpSlab};
  int cur = 0;
  for (int it = 0; it < nIter; it++) {
    const bool copyOnly = it == nIter - 1 && (nIter0 % 2) == 1;
    if (copyOnly) {
      if (bytes) MSBG_CUDA(ctx, cudaMemcpyAsync(bufs[cur ^ 1], bufs[cur], bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    } else {
      rc = launchTyped(ctx, c.storage, exact, ctx->dActive, (int)ctx->nActive, bufs[cur], bufs[cur ^ 1], g);
      if (rc) return rc;
    }
    cur ^= 1;
  }
  return MSBG_GPU_OK;
}

}  // namespace msbg
