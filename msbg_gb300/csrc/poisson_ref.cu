// The reference's solver calls with their block lists, and the reference's own block
// smoother.
//
// Every solver call of MultiresSparseGrid takes a `std::vector<int> *blockList` (NULL:
// all blocks): multiplyLaplacianMatrixOpt (src/msbg3.cpp:1756-1912), relax through its
// member list _blocksRelax (src/msbg3.cpp:2244-2369), dotProdChannel_
// (src/msbg.cpp:4524-4646), AXPBYChannel[Combined] (src/msbg.cpp:4651-4872).  Here a
// list is a device array of block ids; listed blocks without payload are skipped, as the
// reference skips BLK_NO_FLUID blocks.  Calls without a list take the solver's
// whole-level kernels (poisson.cu, poisson_blk.cu); calls with one run the per-block
// kernels below, one CTA per listed block.
//
// The block smoother is relax() as the reference runs it: red-black over blocks by
// (bx+by+bz)&1 (relaxBlockList, src/msbg3.cpp:2170-2239), each block with its
// face-neighbour halo taken at its start and _mgSmBlockIter block-local iterations
// in place (IprocessBlockLaplacian, src/msbg3.cpp:1108-1332): cells in groups of the
// reference's SIMD width along x (8 for block edges 8 and 16, src/msbg3.cpp:1688-1745;
// 8 here for edge 32 too, which the reference does not handle), a group updated from
// values read before its store,
//   S = fma(F6,W6, ... fma(F1,W1, 0)),   Y = omega (B + S) / d + (1 - omega) F0,
// iteration i sweeping the groups backward when (i&1) equals the reverse flag, the last
// iteration storing to X instead of the block buffer (so it is a Jacobi step).  A
// sequential sweep is a wavefront here: group (g, y, z) of a forward sweep depends on
// (g-1, y, z), (g, y-1, z) and (g, y, z-1), so all groups with g+y+z = t update together
// in step t, and the values each group reads are exactly those the sequential order
// gives it.
#include "poisson.cuh"

namespace msbg {

namespace {

constexpr int kListThreads = 256;

// device bids -> slots; value blocks appended to the parity lists (order within a
// parity does not matter: such blocks share no face); err[0] counts bad ids
__global__ void kListSlots(const int32_t *__restrict__ bids, int64_t n, const int32_t *__restrict__ slot,
                           int64_t nBlocks, int nbx, int nby, int32_t *__restrict__ all, int32_t *__restrict__ par0,
                           int32_t *__restrict__ par1, int32_t *__restrict__ cnt) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int bid = bids[i];
  if (bid < 0 || bid >= nBlocks) {
    atomicAdd(&cnt[3], 1);
    all[i] = -1;
    return;
  }
  const int s = slot[bid];
  all[i] = s;
  if (s < 0) return;
  const int bx = bid % nbx, by = (bid / nbx) % nby, bz = (int)(bid / ((int64_t)nbx * nby));
  if ((bx + by + bz) & 1)
    par1[atomicAdd(&cnt[1], 1)] = s;
  else
    par0[atomicAdd(&cnt[0], 1)] = s;
}

__device__ __forceinline__ double ctaSumD(double v) {
  __shared__ double ws[kListThreads / 32];
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) ws[w] = v;
  __syncthreads();
  v = 0.0;
#pragma unroll
  for (int k = 0; k < kListThreads / 32; k++) v += ws[k];
  __syncthreads();
  return v;
}

// (A x)_c = d x_c - sum_f c_f x_nb(f) for the cells of the listed blocks (x = 0 outside
// the value blocks); residual: y = b - A x; part[k] = sum over block k of y*x (FP64).
// The reference keeps 1/d in CH_DIAGONAL and multiplies x by the reciprocal of that, in one
// fused multiply-add with the face sum (its compiled form); so does this kernel, from d:
// 1/(1/d) in FP32, which makes it equal the reference's operator bit for bit.
__global__ void __launch_bounds__(kListThreads) kApplyList(const int32_t *__restrict__ slots, BlkGeom g,
                                                           const float *__restrict__ x, const float *__restrict__ b,
                                                           const float *__restrict__ cx, const float *__restrict__ cy,
                                                           const float *__restrict__ cz, const float *__restrict__ d,
                                                           float *__restrict__ y, int residual,
                                                           double *__restrict__ part) {
  const int s = slots[blockIdx.x];
  if (s < 0) {
    if (part && threadIdx.x == 0) part[blockIdx.x] = 0.0;
    return;
  }
  const int bs = g.bs, lg = g.log2bs;
  const int64_t vpb = (int64_t)1 << (3 * lg), base = (int64_t)s * vpb;
  const int32_t *nb = g.nbr + (int64_t)s * 6;
  double acc = 0.0;
  for (int64_t v = threadIdx.x; v < vpb; v += blockDim.x) {
    const int i = (int)(v & (bs - 1)), j = (int)((v >> lg) & (bs - 1)), k = (int)(v >> (2 * lg));
    const int64_t c = base + v;
    auto at = [&](int dir, int64_t inner, int64_t across) -> float {
      // dir: 0 -x, 1 +x, 2 -y, 3 +y, 4 -z, 5 +z
      if (inner >= 0) return x[inner];
      const int t = nb[dir];
      return t < 0 ? 0.0f : x[(int64_t)t * vpb + across];
    };
    const int64_t sy = bs, sz = (int64_t)bs * bs;
    const float xm = at(0, i > 0 ? c - 1 : -1, v + (bs - 1));
    const float xp = at(1, i < bs - 1 ? c + 1 : -1, v - (bs - 1));
    const float ym = at(2, j > 0 ? c - sy : -1, v + (bs - 1) * sy);
    const float yp = at(3, j < bs - 1 ? c + sy : -1, v - (bs - 1) * sy);
    const float zm = at(4, k > 0 ? c - sz : -1, v + (bs - 1) * sz);
    const float zp = at(5, k < bs - 1 ? c + sz : -1, v - (bs - 1) * sz);
    auto up = [&](const float *cc, int dir, int64_t inner, int64_t across) -> float {
      if (inner >= 0) return cc[inner];
      const int t = nb[dir];
      return t < 0 ? 0.0f : cc[(int64_t)t * vpb + across];
    };
    const float cxp = up(cx, 1, i < bs - 1 ? c + 1 : -1, v - (bs - 1));
    const float cyp = up(cy, 3, j < bs - 1 ? c + sy : -1, v - (bs - 1) * sy);
    const float czp = up(cz, 5, k < bs - 1 ? c + sz : -1, v - (bs - 1) * sz);
    float s6 = cx[c] * xm;
    s6 = fmaf(cxp, xp, s6);
    s6 = fmaf(cy[c], ym, s6);
    s6 = fmaf(cyp, yp, s6);
    s6 = fmaf(cz[c], zm, s6);
    s6 = fmaf(czp, zp, s6);
    const float xc = x[c];
    float r = fmaf(__fdiv_rn(1.0f, __frcp_rn(d[c])), xc, -s6);
    if (residual) r = b[c] - r;
    y[c] = r;
    acc += (double)r * (double)xc;
  }
  if (part) {
    acc = ctaSumD(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = acc;
  }
}

__global__ void __launch_bounds__(kListThreads) kDotList(const int32_t *__restrict__ slots, int64_t vpb,
                                                         const float *__restrict__ a, const float *__restrict__ b,
                                                         double *__restrict__ part) {
  const int s = slots[blockIdx.x];
  double acc = 0.0;
  if (s >= 0) {
    const int64_t base = (int64_t)s * vpb;
    for (int64_t v = threadIdx.x; v < vpb; v += blockDim.x) acc += (double)a[base + v] * (double)b[base + v];
  }
  acc = ctaSumD(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

__global__ void __launch_bounds__(kListThreads) kSumList(const double *__restrict__ part, int64_t n,
                                                         double *__restrict__ out) {
  double acc = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) acc += part[i];
  acc = ctaSumD(acc);
  if (threadIdx.x == 0) *out = acc;
}

// AXPBYChannel (src/msbg.cpp:4773-4872): Y = a X + b Y; AXPBYChannelCombined
// (src/msbg.cpp:4651-4768): X += a P, P = Q + b P; FP64 arithmetic, FP32 storage.
__global__ void __launch_bounds__(kListThreads) kAxpbyList(const int32_t *__restrict__ slots, int64_t vpb, double a,
                                                           const float *__restrict__ x, double b,
                                                           float *__restrict__ y) {
  const int s = slots[blockIdx.x];
  if (s < 0) return;
  const int64_t base = (int64_t)s * vpb;
  for (int64_t v = threadIdx.x; v < vpb; v += blockDim.x)
    y[base + v] = (float)(a * (double)x[base + v] + b * (double)y[base + v]);
}

__global__ void __launch_bounds__(kListThreads) kAxpbyCombinedList(const int32_t *__restrict__ slots, int64_t vpb,
                                                                   double a, double b, const float *__restrict__ q,
                                                                   float *__restrict__ x, float *__restrict__ p) {
  const int s = slots[blockIdx.x];
  if (s < 0) return;
  const int64_t base = (int64_t)s * vpb;
  for (int64_t v = threadIdx.x; v < vpb; v += blockDim.x) {
    const double pi = p[base + v];
    x[base + v] = (float)((double)x[base + v] + a * pi);
    p[base + v] = (float)((double)q[base + v] + b * pi);
  }
}

// The reference's block smoother on the blocks of one parity (slots[]).  hb holds
// the block and its six face layers, (BS+2)^3 floats, x fastest.
template <int BS>
__global__ void __launch_bounds__(kListThreads) kRelaxRef(const int32_t *__restrict__ slots, BlkGeom g,
                                                          float *__restrict__ x, const float *__restrict__ b,
                                                          const float *__restrict__ cx, const float *__restrict__ cy,
                                                          const float *__restrict__ cz, const float *__restrict__ d,
                                                          float omega, int blockIter, int reverse) {
  constexpr int HS = BS + 2, HS2 = HS * HS, VPB = BS * BS * BS;
  constexpr int GW = BS >= 8 ? 8 : BS;  // the reference's SIMD width for this block edge
  constexpr int G = BS / GW;            // groups per row
  constexpr int T = G + 2 * BS - 2;     // wavefront steps of one sweep
  extern __shared__ float hb[];
  const int s = slots[blockIdx.x];
  const int64_t base = (int64_t)s * VPB;
  const int32_t *nb = g.nbr + (int64_t)s * 6;
  const int tid = threadIdx.x;
  for (int v = tid; v < VPB; v += blockDim.x) {
    const int i = v % BS, j = (v / BS) % BS, k = v / (BS * BS);
    hb[(k + 1) * HS2 + (j + 1) * HS + (i + 1)] = x[base + v];
  }
  // face layers: the adjacent layer of the neighbour block, 0 without one
  for (int v = tid; v < 6 * BS * BS; v += blockDim.x) {
    const int f = v / (BS * BS), p = v % (BS * BS), u = p % BS, w = p / BS;
    const int t = nb[f];
    const int axis = f >> 1, hi = f & 1;
    int si, sj, sk, hi_, hj, hk;  // source cell in the neighbour, destination in hb
    if (axis == 0) { si = hi ? 0 : BS - 1; sj = u; sk = w; hi_ = hi ? BS + 1 : 0; hj = u + 1; hk = w + 1; }
    else if (axis == 1) { si = u; sj = hi ? 0 : BS - 1; sk = w; hi_ = u + 1; hj = hi ? BS + 1 : 0; hk = w + 1; }
    else { si = u; sj = w; sk = hi ? 0 : BS - 1; hi_ = u + 1; hj = w + 1; hk = hi ? BS + 1 : 0; }
    hb[hk * HS2 + hj * HS + hi_] = t < 0 ? 0.0f : x[(int64_t)t * VPB + (sk * BS + sj) * BS + si];
  }
  __syncthreads();
  const float oneMinusOmega = 1.0f - omega;
  // one group: GW cells from (g*GW, j, k); results to y[]
  auto group = [&](int gi, int j, int k, float *y) {
#pragma unroll
    for (int l = 0; l < GW; l++) {
      const int i = gi * GW + l;
      const int v = (k * BS + j) * BS + i;
      const int64_t c = base + v;
      const float *p = hb + (k + 1) * HS2 + (j + 1) * HS + (i + 1);
      const float F0 = p[0], F1 = p[-1], F2 = p[1], F3 = p[-HS], F4 = p[HS], F5 = p[-HS2], F6 = p[HS2];
      const float W1 = cx[c], W3 = cy[c], W5 = cz[c];
      const float W2 = i < BS - 1 ? cx[c + 1] : (nb[1] < 0 ? 0.0f : cx[(int64_t)nb[1] * VPB + v - (BS - 1)]);
      const float W4 = j < BS - 1 ? cy[c + BS] : (nb[3] < 0 ? 0.0f : cy[(int64_t)nb[3] * VPB + v - (BS - 1) * BS]);
      const float W6 = k < BS - 1 ? cz[c + BS * BS]
                                  : (nb[5] < 0 ? 0.0f : cz[(int64_t)nb[5] * VPB + v - (BS - 1) * BS * BS]);
      float S = 0.0f;
      S = __fmaf_rn(F1, W1, S);
      S = __fmaf_rn(F2, W2, S);
      S = __fmaf_rn(F3, W3, S);
      S = __fmaf_rn(F4, W4, S);
      S = __fmaf_rn(F5, W5, S);
      S = __fmaf_rn(F6, W6, S);
      // omega (B + S) D + (1 - omega) F0 as the reference's compiled 8-wide path forms it
      const float dinv = __frcp_rn(d[c]);
      const float t = __fadd_rn(S, b[c]);
      y[l] = __fmaf_rn(oneMinusOmega, F0, __fmul_rn(__fmul_rn(omega, dinv), t));
    }
  };
  for (int it = 0; it < blockIter - 1; it++) {
    const bool backward = (it & 1) == reverse;
    for (int t = 0; t < T; t++) {
      for (int q = tid; q < BS * BS; q += blockDim.x) {
        const int j0 = q % BS, k0 = q / BS;
        const int g0 = t - j0 - k0;
        if (g0 < 0 || g0 >= G) continue;
        const int gi = backward ? G - 1 - g0 : g0, j = backward ? BS - 1 - j0 : j0,
                  k = backward ? BS - 1 - k0 : k0;
        float y[GW];
        group(gi, j, k, y);
        float *p = hb + (k + 1) * HS2 + (j + 1) * HS + gi * GW + 1;
#pragma unroll
        for (int l = 0; l < GW; l++) p[l] = y[l];
      }
      __syncthreads();
    }
  }
  if (blockIter >= 1) {  // the last iteration: every group from the buffer, into x
    for (int q = tid; q < G * BS * BS; q += blockDim.x) {
      const int gi = q % G, j = (q / G) % BS, k = q / (G * BS);
      float y[GW];
      group(gi, j, k, y);
      float *o = x + base + (k * BS + j) * BS + gi * GW;
#pragma unroll
      for (int l = 0; l < GW; l++) o[l] = y[l];
    }
  }
}

template <int BS>
int launchRelaxRef(msbg_gpu_ctx *ctx, const int32_t *slots, int64_t n, BlkGeom g, float *x, const float *b,
                   const PrecSet &P, float omega, int blockIter, int reverse) {
  if (n <= 0) return MSBG_GPU_OK;
  constexpr size_t smem = sizeof(float) * (BS + 2) * (BS + 2) * (BS + 2);
  static bool attr = false;
  if (!attr) {
    MSBG_CUDA(ctx, cudaFuncSetAttribute(kRelaxRef<BS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = true;
  }
  MSBG_LAUNCH(ctx, kRelaxRef<BS>, (unsigned)n, kListThreads, smem, slots, g, x, b, (const float *)P.cx[0],
              (const float *)P.cy[0], (const float *)P.cz[0], (const float *)P.d[0], omega, blockIter, reverse);
  return MSBG_GPU_OK;
}

}  // namespace

int listSlots(msbg_gpu_ctx *ctx, PoissonState *ps, const int32_t *dBids, int64_t n, SlotLists *out) {
  const int64_t nAct = ps->levels[0].nAct;
  const int64_t need = 3 * (n > nAct ? n : nAct) + 8;
  if (ps->listCap < need) {
    if (ps->dListBuf) cudaFree(ps->dListBuf);
    if (ps->dListPart) cudaFree(ps->dListPart);
    ps->dListBuf = nullptr;
    ps->dListPart = nullptr;
    ps->listCap = 0;
    MSBG_CUDA(ctx, cudaMalloc(&ps->dListBuf, (size_t)need * 4));
    MSBG_CUDA(ctx, cudaMalloc(&ps->dListPart, (size_t)need * 8));
    ps->listCap = need;
  }
  const int64_t m = n > nAct ? n : nAct;
  int32_t *all = ps->dListBuf, *par0 = all + m, *par1 = par0 + m, *cnt = par1 + m;
  MSBG_CUDA(ctx, cudaMemsetAsync(cnt, 0, 16, ctx->stream));
  if (n > 0)
    MSBG_LAUNCH(ctx, kListSlots, gridFor(n, 256), 256, 0, dBids, n, ctx->dSlot, ctx->nBlocks, ctx->nbx, ctx->nby, all,
                par0, par1, cnt);
  int32_t h[4] = {0, 0, 0, 0};
  MSBG_CUDA(ctx, cudaMemcpyAsync(h, cnt, 16, cudaMemcpyDeviceToHost, ctx->stream));
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (h[3]) return fail(ctx, MSBG_GPU_ERR_ARG, "block list holds %d ids outside the block grid", h[3]);
  out->all = all;
  out->nAll = n;
  out->par[0] = par0;
  out->par[1] = par1;
  out->nPar[0] = h[0];
  out->nPar[1] = h[1];
  return MSBG_GPU_OK;
}

int applyList(msbg_gpu_ctx *ctx, PoissonState *ps, const SlotLists &L, const float *x, const float *b, float *y,
              int residual, double *dDot) {
  if (L.nAll <= 0) {
    if (dDot) MSBG_CUDA(ctx, cudaMemsetAsync(dDot, 0, 8, ctx->stream));
    return MSBG_GPU_OK;
  }
  const PrecSet &P = ps->f32;
  const BlkGeom g = blkOf(ps, ps->levels[0]);
  MSBG_LAUNCH(ctx, kApplyList, (unsigned)L.nAll, kListThreads, 0, L.all, g, x, b, (const float *)P.cx[0],
              (const float *)P.cy[0], (const float *)P.cz[0], (const float *)P.d[0], y, residual,
              dDot ? ps->dListPart : nullptr);
  if (dDot) MSBG_LAUNCH(ctx, kSumList, 1, kListThreads, 0, ps->dListPart, L.nAll, dDot);
  return MSBG_GPU_OK;
}

int dotList(msbg_gpu_ctx *ctx, PoissonState *ps, const SlotLists &L, const float *a, const float *b, double *dOut) {
  if (L.nAll <= 0) {
    MSBG_CUDA(ctx, cudaMemsetAsync(dOut, 0, 8, ctx->stream));
    return MSBG_GPU_OK;
  }
  MSBG_LAUNCH(ctx, kDotList, (unsigned)L.nAll, kListThreads, 0, L.all, ctx->voxPerBlock, a, b, ps->dListPart);
  MSBG_LAUNCH(ctx, kSumList, 1, kListThreads, 0, ps->dListPart, L.nAll, dOut);
  return MSBG_GPU_OK;
}

int axpbyList(msbg_gpu_ctx *ctx, const SlotLists &L, double a, const float *x, double b, float *y) {
  if (L.nAll > 0) MSBG_LAUNCH(ctx, kAxpbyList, (unsigned)L.nAll, kListThreads, 0, L.all, ctx->voxPerBlock, a, x, b, y);
  return MSBG_GPU_OK;
}

int axpbyCombinedList(msbg_gpu_ctx *ctx, const SlotLists &L, double a, double b, const float *q, float *x,
                      float *p) {
  if (L.nAll > 0)
    MSBG_LAUNCH(ctx, kAxpbyCombinedList, (unsigned)L.nAll, kListThreads, 0, L.all, ctx->voxPerBlock, a, b, q, x, p);
  return MSBG_GPU_OK;
}

int relaxReference(msbg_gpu_ctx *ctx, PoissonState *ps, const SlotLists *L, float *x, const float *b, int passes,
                   int reverse, int blockIter, float omega) {
  const MgLevel &L0 = ps->levels[0];
  const BlkGeom g = blkOf(ps, L0);
  // parity lists: the caller's, or level 0's parity-ordered slot list (even first)
  const int32_t *par[2];
  int64_t nPar[2];
  if (L) {
    par[0] = L->par[0]; par[1] = L->par[1];
    nPar[0] = L->nPar[0]; nPar[1] = L->nPar[1];
  } else {
    par[0] = ps->dParList; par[1] = ps->dParList + ps->nEven;
    nPar[0] = ps->nEven; nPar[1] = L0.nAct - ps->nEven;
  }
  for (int pass = 0; pass < passes; pass++)
    for (int rb = 0; rb < 2; rb++) {
      // relaxBlockList skips blocks whose parity equals the half-pass index: parity 1
      // first, parity 0 first with the reverse order
      const int parity = reverse ? rb : 1 - rb;
      int rc;
      switch (L0.bs) {
        case 8: rc = launchRelaxRef<8>(ctx, par[parity], nPar[parity], g, x, b, ps->f32, omega, blockIter, reverse); break;
        case 16: rc = launchRelaxRef<16>(ctx, par[parity], nPar[parity], g, x, b, ps->f32, omega, blockIter, reverse); break;
        case 32: rc = launchRelaxRef<32>(ctx, par[parity], nPar[parity], g, x, b, ps->f32, omega, blockIter, reverse); break;
        default: return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED, "block smoother for block edge %d", L0.bs);
      }
      if (rc) return rc;
    }
  return MSBG_GPU_OK;
}

}  // namespace msbg

// ---- the operator at a dense multigrid level --------------------------------------------
//
// ImultiplyLaplacianMatrixProcessSliceDenseLevel (src/msbg3.cpp:166-403), the operator of
// multiplyLaplacianMatrixOpt at levelMg >= nLevels, on one dense level's arrays (x fastest;
// X and the face areas are 0 outside the box, and its cells are void there).  The reference
// walks each row in groups of 4 cells from x = 0: a group without a fluid cell is skipped,
// a group with a solid or partially solid cell weighs every cell's neighbours by the face
// areas.  Per fluid cell Y = h (X / D - S), S = (F1+F2) + ((F3+F4) + (F5+F6)) (the
// reference's compiled form of h (1/D) X - h sum F), 0 for other cells of a processed
// group; the residual B - Y.  One thread per cell.
namespace msbg {
namespace {

constexpr unsigned kCellSolid = 1u << 0, kCellPartialSolid = 1u << 6, kCellVoid = 1u << 12;

__global__ void __launch_bounds__(256) kApplyDense(int sx, int sy, int sz, float h, int residual,
                                                   const uint16_t *__restrict__ fl, const float *__restrict__ x,
                                                   const float *__restrict__ b, const float *__restrict__ d,
                                                   const float *__restrict__ ax, const float *__restrict__ ay,
                                                   const float *__restrict__ az, float *__restrict__ y) {
  const int64_t sxy = (int64_t)sx * sy, n = sxy * sz;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t row = i / sx;
  const int xx = (int)(i - row * sx), yy = (int)(row % sy), zz = (int)(row / sy);
  bool active = false, weighted = false;
  for (int k = 0, g0 = xx & ~3; k < 4 && g0 + k < sx; k++) {
    const unsigned f = fl[row * sx + g0 + k];
    active |= (f & (kCellSolid | kCellVoid)) == 0;
    weighted |= (f & (kCellSolid | kCellPartialSolid)) != 0;
  }
  if (!active) return;  // the reference skips the group and leaves its outputs as they are
  float Y = 0.0f;
  if ((fl[i] & (kCellSolid | kCellVoid)) == 0) {
    float F1 = xx > 0 ? x[i - 1] : 0.0f, F2 = xx < sx - 1 ? x[i + 1] : 0.0f;
    float F3 = yy > 0 ? x[i - sx] : 0.0f, F4 = yy < sy - 1 ? x[i + sx] : 0.0f;
    float F5 = zz > 0 ? x[i - sxy] : 0.0f, F6 = zz < sz - 1 ? x[i + sxy] : 0.0f;
    if (weighted) {
      F1 = __fmul_rn(F1, ax[i]);
      F2 = __fmul_rn(F2, xx < sx - 1 ? ax[i + 1] : 0.0f);
      F3 = __fmul_rn(F3, ay[i]);
      F4 = __fmul_rn(F4, yy < sy - 1 ? ay[i + sx] : 0.0f);
      F5 = __fmul_rn(F5, az[i]);
      F6 = __fmul_rn(F6, zz < sz - 1 ? az[i + sxy] : 0.0f);
    }
    const float S = __fadd_rn(__fadd_rn(F1, F2), __fadd_rn(__fadd_rn(F3, F4), __fadd_rn(F5, F6)));
    Y = __fmul_rn(__fsub_rn(__fdiv_rn(x[i], d[i]), S), h);
  }
  if (residual) Y = __fsub_rn(b[i], Y);
  y[i] = Y;
}

// One omega-Jacobi iteration of the dense-level smoother (src/msbg3.cpp:1917-2165, without
// the block Gauss-Seidel and scheduled-omega switches, as the release builds it): src -> dst,
// the operator's groups and weights; fluid cells Y = fma(1 - omega, F0, (B + h S)(D omega/h)),
// the reference's compiled form, other cells of a processed group 0, skipped groups untouched.
__global__ void __launch_bounds__(256) kRelaxDense(int sx, int sy, int sz, float h, float omega,
                                                   const uint16_t *__restrict__ fl, const float *__restrict__ x,
                                                   const float *__restrict__ b, const float *__restrict__ d,
                                                   const float *__restrict__ ax, const float *__restrict__ ay,
                                                   const float *__restrict__ az, float *__restrict__ y) {
  const int64_t sxy = (int64_t)sx * sy, n = sxy * sz;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t row = i / sx;
  const int xx = (int)(i - row * sx), yy = (int)(row % sy), zz = (int)(row / sy);
  bool active = false, weighted = false;
  for (int k = 0, g0 = xx & ~3; k < 4 && g0 + k < sx; k++) {
    const unsigned f = fl[row * sx + g0 + k];
    active |= (f & (kCellSolid | kCellVoid)) == 0;
    weighted |= (f & (kCellSolid | kCellPartialSolid)) != 0;
  }
  if (!active) return;
  float Y = 0.0f;
  if ((fl[i] & (kCellSolid | kCellVoid)) == 0) {
    float F1 = xx > 0 ? x[i - 1] : 0.0f, F2 = xx < sx - 1 ? x[i + 1] : 0.0f;
    float F3 = yy > 0 ? x[i - sx] : 0.0f, F4 = yy < sy - 1 ? x[i + sx] : 0.0f;
    float F5 = zz > 0 ? x[i - sxy] : 0.0f, F6 = zz < sz - 1 ? x[i + sxy] : 0.0f;
    if (weighted) {
      F1 = __fmul_rn(F1, ax[i]);
      F2 = __fmul_rn(F2, xx < sx - 1 ? ax[i + 1] : 0.0f);
      F3 = __fmul_rn(F3, ay[i]);
      F4 = __fmul_rn(F4, yy < sy - 1 ? ay[i + sx] : 0.0f);
      F5 = __fmul_rn(F5, az[i]);
      F6 = __fmul_rn(F6, zz < sz - 1 ? az[i + sxy] : 0.0f);
    }
    const float S = __fmul_rn(__fadd_rn(__fadd_rn(F1, F2), __fadd_rn(__fadd_rn(F3, F4), __fadd_rn(F5, F6))), h);
    const float t = __fadd_rn(b[i], S);
    const float dho = __fmul_rn(d[i], __fdiv_rn(omega, h));
    Y = __fmaf_rn(__fsub_rn(1.0f, omega), x[i], __fmul_rn(t, dho));
  }
  y[i] = Y;
}

}  // namespace
}  // namespace msbg

extern "C" int msbg_gpu_relax_dense(msbg_gpu_ctx *ctx, int levelMg, int sx, int sy, int sz, int nIter,
                                    const uint16_t *dFlags, float *dX, const float *dB, const float *dDiag,
                                    const float *dAreaX, const float *dAreaY, const float *dAreaZ, float *dTmp) {
  using namespace msbg;
  if (!ctx) return MSBG_GPU_ERR_ARG;
  if (levelMg < 0 || levelMg > 30) return fail(ctx, MSBG_GPU_ERR_ARG, "relax_dense: levelMg %d out of range", levelMg);
  if (sx <= 0 || sy <= 0 || sz <= 0 || nIter < 0) return fail(ctx, MSBG_GPU_ERR_ARG, "relax_dense: bad sizes");
  if (!dFlags || !dX || !dB || !dDiag || !dAreaX || !dAreaY || !dAreaZ || !dTmp || dTmp == dX)
    return fail(ctx, MSBG_GPU_ERR_ARG, "relax_dense: null or aliased array");
  const int64_t n = (int64_t)sx * sy * sz;
  const float h = (float)(1 << levelMg);
  float *src = dX, *dst = dTmp;
  for (int it = 0; it < nIter; it++) {
    MSBG_LAUNCH(ctx, kRelaxDense, (unsigned)((n + 255) / 256), 256, 0, sx, sy, sz, h, ctx->relaxOmega, dFlags, src, dB,
                dDiag, dAreaX, dAreaY, dAreaZ, dst);
    float *t = src;
    src = dst;
    dst = t;
  }
  // after an odd count the result is in the temporary array: the whole array goes to X
  if (src != dX) MSBG_CUDA(ctx, cudaMemcpyAsync(dX, src, (size_t)n * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_multiply_laplacian_dense(msbg_gpu_ctx *ctx, unsigned options, int levelMg, int sx, int sy,
                                                 int sz, const uint16_t *dFlags, const float *dX, const float *dB,
                                                 const float *dDiag, const float *dAreaX, const float *dAreaY,
                                                 const float *dAreaZ, float *dY) {
  using namespace msbg;
  if (!ctx) return MSBG_GPU_ERR_ARG;
  const bool residual = (options & MSBG_GPU_OPT_CALC_RESIDUAL) != 0;
  if (options & ~(unsigned)MSBG_GPU_OPT_CALC_RESIDUAL)
    return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED, "multiply_dense: options 0x%x", options);
  if (levelMg < 0 || levelMg > 30) return fail(ctx, MSBG_GPU_ERR_ARG, "multiply_dense: levelMg %d out of range", levelMg);
  if (sx <= 0 || sy <= 0 || sz <= 0) return fail(ctx, MSBG_GPU_ERR_ARG, "multiply_dense: empty box");
  if (!dFlags || !dX || !dDiag || !dAreaX || !dAreaY || !dAreaZ || !dY || (residual && !dB))
    return fail(ctx, MSBG_GPU_ERR_ARG, "multiply_dense: null array");
  const int64_t n = (int64_t)sx * sy * sz;
  MSBG_LAUNCH(ctx, kApplyDense, (unsigned)((n + 255) / 256), 256, 0, sx, sy, sz, (float)(1 << levelMg),
              residual ? 1 : 0, dFlags, dX, dB, dDiag, dAreaX, dAreaY, dAreaZ, dY);
  return MSBG_GPU_OK;
}
