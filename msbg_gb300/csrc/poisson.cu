// Sparse Poisson solve on the value blocks: 7-point variable-coefficient operator,
// geometric multigrid V-cycle preconditioner, preconditioned CG with FP64 dots.
//
// Reference building blocks (the release has no driver that calls them):
//   operator multiply / residual  Y = (1/D) F0 - sum w F    src/msbg3.cpp:1281-1296
//   smoother                       relax / relaxBlockList    src/msbg3.cpp:2170-2369
//   restriction                    downsampleFloatChannelNew src/msbg4.cpp:1035-1379
//   prolongation                   constant (MG_CONST_PROLONGATION) src/msbgcell.h:99-101
//   dot product (FP64 accumulate)  dotProdChannel_           src/msbg.cpp:4524-4646
//   X += aP, P = Q + bP            AXPBYChannelCombined      src/msbg.cpp:4651-4768
//   Y = aX + bY                    AXPBYChannel              src/msbg.cpp:4773-4872
//   dense coarse MG levels         src/msbg.cpp:854-998, src/msbg3.cpp:1917-2165
//
// Operator.  For every active cell i with face coefficients c_f:
//   (A x)_i = d_i x_i - sum_{faces f} c_f x_nb(f),   x = 0 outside the active cells
// Coefficients are stored per cell as its three lower faces (cx, cy, cz) and the
// diagonal d (which also carries the faces to inactive neighbours, Dirichlet 0);
// the upper face of a cell is the lower face of the neighbour above.
//
// Hierarchy.  Level 0 is the value-block payload (block edge bs).  Each coarser
// level halves the block edge on the same block set until one cell per block,
// then aggregates 2x2x2 blocks of that block grid per level (the dense coarse
// levels).  Every level is a "block-sparse grid": block grid, slot map, active
// list, cells [nAct][bs^3].  Transfers are piecewise constant: restriction sums
// the 8 children (R = P^T), prolongation injects; the coarse operator is
// P^T A P / 2 (the rediscretized coefficient of a coarse face is half the sum of
// its four fine faces), which keeps the V-cycle symmetric for CG.  Smoothing is
// red-black Gauss-Seidel on cells (parity of x+y+z), pre-smoothing red first and
// post-smoothing black first; the coarsest level (<= 4096 cells) is relaxed by one
// CTA for many sweeps.
#include <math.h>
#include <string.h>

#include <vector>

#include "internal.cuh"
#include "poisson.cuh"

namespace msbg {

// ---------------------------------------------------------------------------------
// cell addressing on a level
// ---------------------------------------------------------------------------------
__device__ __forceinline__ void cellOf(const LvGeom &g, int64_t c, int &gx, int &gy, int &gz) {
  const int s = (int)(c >> (3 * g.log2bs));
  const int v = (int)(c & ((1 << (3 * g.log2bs)) - 1));
  const int m = g.bs - 1;
  const int lx = v & m, ly = (v >> g.log2bs) & m, lz = v >> (2 * g.log2bs);
  const int bid = g.active[s];
  const int bx = bid % g.nbx, by = (bid / g.nbx) % g.nby, bz = bid / (g.nbx * g.nby);
  gx = (bx << g.log2bs) + lx;
  gy = (by << g.log2bs) + ly;
  gz = (bz << g.log2bs) + lz;
}

// linear index of cell (gx,gy,gz) on the level, or -1 when outside / inactive
__device__ __forceinline__ int64_t cellIdx(const LvGeom &g, int gx, int gy, int gz) {
  if (gx < 0 || gy < 0 || gz < 0) return -1;
  const int bx = gx >> g.log2bs, by = gy >> g.log2bs, bz = gz >> g.log2bs;
  if (bx >= g.nbx || by >= g.nby || bz >= g.nbz) return -1;
  const int s = g.slot[((int64_t)bz * g.nby + by) * g.nbx + bx];
  if (s < 0) return -1;
  const int m = g.bs - 1;
  return ((int64_t)s << (3 * g.log2bs)) + ((((gz & m) << g.log2bs) + (gy & m)) << g.log2bs) + (gx & m);
}

template <typename R>
__device__ __forceinline__ R nbVal(const LvGeom &g, const float *x, int gx, int gy, int gz) {
  const int64_t j = cellIdx(g, gx, gy, gz);
  return j < 0 ? (R)0 : (R)x[j];
}

// A x at cell c (coords gx,gy,gz), compute type R
template <typename R>
__device__ __forceinline__ R applyAt(const LvGeom &g, const float *__restrict__ x, const float *__restrict__ cx,
                                     const float *__restrict__ cy, const float *__restrict__ cz,
                                     const float *__restrict__ d, int64_t c, int gx, int gy, int gz) {
  R s = (R)d[c] * (R)x[c];
  {
    const int64_t j = cellIdx(g, gx - 1, gy, gz);
    if (j >= 0) s -= (R)cx[c] * (R)x[j];
    const int64_t k = cellIdx(g, gx + 1, gy, gz);
    if (k >= 0) s -= (R)cx[k] * (R)x[k];
  }
  {
    const int64_t j = cellIdx(g, gx, gy - 1, gz);
    if (j >= 0) s -= (R)cy[c] * (R)x[j];
    const int64_t k = cellIdx(g, gx, gy + 1, gz);
    if (k >= 0) s -= (R)cy[k] * (R)x[k];
  }
  {
    const int64_t j = cellIdx(g, gx, gy, gz - 1);
    if (j >= 0) s -= (R)cz[c] * (R)x[j];
    const int64_t k = cellIdx(g, gx, gy, gz + 1);
    if (k >= 0) s -= (R)cz[k] * (R)x[k];
  }
  return s;
}

// ---------------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------------
// mode 0: y = A x; mode 1: y = b - A x.  Grid-stride over the level's cells.
__global__ void kApply(LvGeom g, const float *__restrict__ x, const float *__restrict__ b,
                       const float *__restrict__ cx, const float *__restrict__ cy,
                       const float *__restrict__ cz, const float *__restrict__ d, float *__restrict__ y,
                       int mode) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < g.nCell;
       c += (int64_t)gridDim.x * blockDim.x) {
    int gx, gy, gz;
    cellOf(g, c, gx, gy, gz);
    const float ax = applyAt<float>(g, x, cx, cy, cz, d, c, gx, gy, gz);
    y[c] = mode ? b[c] - ax : ax;
  }
}

// Red-black Gauss-Seidel half sweep: cells with (gx+gy+gz)&1 == color get
// x = (b + sum c x_nb) / d.
__global__ void kRBGS(LvGeom g, float *__restrict__ x, const float *__restrict__ b,
                      const float *__restrict__ cx, const float *__restrict__ cy,
                      const float *__restrict__ cz, const float *__restrict__ d, int color) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < g.nCell;
       c += (int64_t)gridDim.x * blockDim.x) {
    int gx, gy, gz;
    cellOf(g, c, gx, gy, gz);
    if (((gx + gy + gz) & 1) != color) continue;
    float s = b[c];
    int64_t j;
    if ((j = cellIdx(g, gx - 1, gy, gz)) >= 0) s += cx[c] * x[j];
    if ((j = cellIdx(g, gx + 1, gy, gz)) >= 0) s += cx[j] * x[j];
    if ((j = cellIdx(g, gx, gy - 1, gz)) >= 0) s += cy[c] * x[j];
    if ((j = cellIdx(g, gx, gy + 1, gz)) >= 0) s += cy[j] * x[j];
    if ((j = cellIdx(g, gx, gy, gz - 1)) >= 0) s += cz[c] * x[j];
    if ((j = cellIdx(g, gx, gy, gz + 1)) >= 0) s += cz[j] * x[j];
    x[c] = s / d[c];
  }
}

// Coarsest level: nIter red-black sweeps by one CTA (cells <= blockDim * k).
__global__ void kCoarsestGS(LvGeom g, float *__restrict__ x, const float *__restrict__ b,
                            const float *__restrict__ cx, const float *__restrict__ cy,
                            const float *__restrict__ cz, const float *__restrict__ d, int nIter) {
  for (int64_t c = threadIdx.x; c < g.nCell; c += blockDim.x) x[c] = 0.0f;
  __syncthreads();
  for (int it = 0; it < nIter; it++) {
    for (int color = 0; color < 2; color++) {
      for (int64_t c = threadIdx.x; c < g.nCell; c += blockDim.x) {
        int gx, gy, gz;
        cellOf(g, c, gx, gy, gz);
        if (((gx + gy + gz) & 1) != color) continue;
        float s = b[c];
        int64_t j;
        if ((j = cellIdx(g, gx - 1, gy, gz)) >= 0) s += cx[c] * x[j];
        if ((j = cellIdx(g, gx + 1, gy, gz)) >= 0) s += cx[j] * x[j];
        if ((j = cellIdx(g, gx, gy - 1, gz)) >= 0) s += cy[c] * x[j];
        if ((j = cellIdx(g, gx, gy + 1, gz)) >= 0) s += cy[j] * x[j];
        if ((j = cellIdx(g, gx, gy, gz - 1)) >= 0) s += cz[c] * x[j];
        if ((j = cellIdx(g, gx, gy, gz + 1)) >= 0) s += cz[j] * x[j];
        x[c] = s / d[c];
      }
      __syncthreads();
    }
  }
}

// b_C = R r_F (sum of the active children); x_C = 0.
__global__ void kRestrictSum(LvGeom gf, LvGeom gc, const float *__restrict__ rf, float *__restrict__ bc,
                             float *__restrict__ xc) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < gc.nCell;
       c += (int64_t)gridDim.x * blockDim.x) {
    int gx, gy, gz;
    cellOf(gc, c, gx, gy, gz);
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const int64_t j = cellIdx(gf, 2 * gx + (k & 1), 2 * gy + ((k >> 1) & 1), 2 * gz + (k >> 2));
      if (j >= 0) s += rf[j];
    }
    bc[c] = s;
    xc[c] = 0.0f;
  }
}

// x_F += P x_C (constant injection of the parent's value)
__global__ void kProlongAdd(LvGeom gf, LvGeom gc, const float *__restrict__ xc, float *__restrict__ xf) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < gf.nCell;
       c += (int64_t)gridDim.x * blockDim.x) {
    int gx, gy, gz;
    cellOf(gf, c, gx, gy, gz);
    const int64_t p = cellIdx(gc, gx >> 1, gy >> 1, gz >> 1);
    if (p >= 0) xf[c] += xc[p];
  }
}

// Coarse operator P^T A P / 2 from the fine level's coefficients.
__global__ void kCoarseCoeffs(LvGeom gf, LvGeom gc, const float *__restrict__ fcx,
                              const float *__restrict__ fcy, const float *__restrict__ fcz,
                              const float *__restrict__ fd, float *__restrict__ ccx, float *__restrict__ ccy,
                              float *__restrict__ ccz, float *__restrict__ cd) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < gc.nCell;
       c += (int64_t)gridDim.x * blockDim.x) {
    int gx, gy, gz;
    cellOf(gc, c, gx, gy, gz);
    int64_t ch[8];
#pragma unroll
    for (int k = 0; k < 8; k++)
      ch[k] = cellIdx(gf, 2 * gx + (k & 1), 2 * gy + ((k >> 1) & 1), 2 * gz + (k >> 2));
    double dsum = 0.0, lx = 0.0, ly = 0.0, lz = 0.0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
      if (ch[k] < 0) continue;
      const int ix = k & 1, iy = (k >> 1) & 1, iz = k >> 2;
      const int fx = 2 * gx + ix, fy = 2 * gy + iy, fz = 2 * gz + iz;
      dsum += fd[ch[k]];
      // lower faces: external when the child sits on the coarse cell's lower side,
      // internal otherwise (coupling to the sibling below)
      if (ix == 0) { if (cellIdx(gf, fx - 1, fy, fz) >= 0) lx += fcx[ch[k]]; }
      else if (ch[k - 1] >= 0) dsum -= 2.0 * fcx[ch[k]];
      if (iy == 0) { if (cellIdx(gf, fx, fy - 1, fz) >= 0) ly += fcy[ch[k]]; }
      else if (ch[k - 2] >= 0) dsum -= 2.0 * fcy[ch[k]];
      if (iz == 0) { if (cellIdx(gf, fx, fy, fz - 1) >= 0) lz += fcz[ch[k]]; }
      else if (ch[k - 4] >= 0) dsum -= 2.0 * fcz[ch[k]];
    }
    ccx[c] = (float)(0.5 * lx);
    ccy[c] = (float)(0.5 * ly);
    ccz[c] = (float)(0.5 * lz);
    cd[c] = (float)(0.5 * dsum);
  }
}

// ---- reductions ----------------------------------------------------------------------
constexpr int kRedThreads = 256;

__device__ __forceinline__ double blockSum(double v) {
  __shared__ double ws[kRedThreads / 32];
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) ws[w] = v;
  __syncthreads();
  v = threadIdx.x < kRedThreads / 32 ? ws[threadIdx.x] : 0.0;
  if (w == 0) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  }
  __syncthreads();
  return v;
}

// partial[blockIdx] = sum a*b (FP64 accumulation of FP32 products)
__global__ void kDotPartial(const float *__restrict__ a, const float *__restrict__ b, int64_t n,
                            double *__restrict__ partial) {
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s += (double)a[i] * (double)b[i];
  s = blockSum(s);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

__global__ void kSumPartials(const double *__restrict__ partial, int n, double *__restrict__ out) {
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += partial[i];
  s = blockSum(s);
  if (threadIdx.x == 0) *out = s;
}

// true residual in FP64: partial[block] = {sum (b - A x)^2, sum b^2}
__global__ void kResidualNorm64(LvGeom g, const float *__restrict__ x, const float *__restrict__ b,
                                const float *__restrict__ cx, const float *__restrict__ cy,
                                const float *__restrict__ cz, const float *__restrict__ d,
                                double *__restrict__ partial) {
  double rr = 0.0, bb = 0.0;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < g.nCell;
       c += (int64_t)gridDim.x * blockDim.x) {
    int gx, gy, gz;
    cellOf(g, c, gx, gy, gz);
    const double r = (double)b[c] - applyAt<double>(g, x, cx, cy, cz, d, c, gx, gy, gz);
    rr += r * r;
    bb += (double)b[c] * (double)b[c];
  }
  rr = blockSum(rr);
  bb = blockSum(bb);
  if (threadIdx.x == 0) {
    partial[2 * blockIdx.x] = rr;
    partial[2 * blockIdx.x + 1] = bb;
  }
}

__global__ void kSumPartials2(const double *__restrict__ partial, int n, double *__restrict__ out) {
  double s0 = 0.0, s1 = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    s0 += partial[2 * i];
    s1 += partial[2 * i + 1];
  }
  s0 = blockSum(s0);
  s1 = blockSum(s1);
  if (threadIdx.x == 0) { out[0] = s0; out[1] = s1; }
}

// CG updates with the scalars read from device memory (no host round trip):
// alpha = sc[0] / sc[1]; x += alpha p; r -= alpha q
__global__ void kCgUpdateXR(const double *__restrict__ sc, const float *__restrict__ p, const float *__restrict__ q,
                            float *__restrict__ x, float *__restrict__ r, int64_t n) {
  const double alpha = sc[1] != 0.0 ? sc[0] / sc[1] : 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] = (float)((double)x[i] + alpha * (double)p[i]);
    r[i] = (float)((double)r[i] - alpha * (double)q[i]);
  }
}
// beta = sc[2] / sc[0]; p = z + beta p
__global__ void kCgUpdateP(const double *__restrict__ sc, const float *__restrict__ z, float *__restrict__ p, int64_t n) {
  const double beta = sc[0] != 0.0 ? sc[2] / sc[0] : 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = (float)((double)z[i] + beta * (double)p[i]);
}
__global__ void kCopy(const float *__restrict__ a, float *__restrict__ b, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) b[i] = a[i];
}
// AXPBYChannelCombined: X += aP; P = Q + bP (FP64 arithmetic, src/msbg.cpp:4651-4768)
__global__ void kAxpbyCombined(double a, double b, const float *__restrict__ q, float *__restrict__ x,
                               float *__restrict__ p, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double pi = p[i];
    x[i] = (float)((double)x[i] + a * pi);
    p[i] = (float)((double)q[i] + b * pi);
  }
}
// AXPBYChannel: Y = aX + bY (src/msbg.cpp:4773-4872)
__global__ void kAxpby(double a, const float *__restrict__ x, double b, float *__restrict__ y, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = (float)(a * (double)x[i] + b * (double)y[i]);
}
__global__ void kZero(float *p, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = 0.0f;
}

// Coarse level blocks: parent of every fine active block (block grid halved).
__global__ void kMarkParents(const int32_t *__restrict__ activeF, int64_t nAct, int nbxF, int nbyF, int nbxC,
                             int nbyC, int32_t *__restrict__ markC) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nAct) return;
  const int bid = activeF[i];
  const int bx = bid % nbxF, by = (bid / nbxF) % nbyF, bz = bid / (nbxF * nbyF);
  markC[((int64_t)(bz >> 1) * nbyC + (by >> 1)) * nbxC + (bx >> 1)] = 1;
}
__global__ void kSlotsFromMarks(const int32_t *__restrict__ mark, const int64_t *__restrict__ off, int64_t n,
                                int32_t *__restrict__ slot, int32_t *__restrict__ active) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (mark[i]) {
    slot[i] = (int32_t)off[i];
    active[off[i]] = (int32_t)i;
  } else {
    slot[i] = -1;
  }
}

// ---- procedural workload fields --------------------------------------------------
__device__ __forceinline__ uint32_t hash32(uint32_t x) {
  // integer finalizer (xorshift-multiply), also used by the CPU restatement
  x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
  return x;
}
__device__ __forceinline__ float faceCoeff(uint32_t seed, int axis, int gx, int gy, int gz) {
  uint32_t h = hash32(seed ^ hash32((uint32_t)axis + 0x9e3779b9U * 3u));
  h = hash32(h ^ (uint32_t)gx);
  h = hash32(h ^ (uint32_t)gy * 0x85ebca6bU);
  h = hash32(h ^ (uint32_t)gz * 0xc2b2ae35U);
  return 0.5f + 1.5f * (float)(h >> 8) * (1.0f / 16777216.0f);
}
// cx, cy, cz (lower faces) and d (all six faces) of level 0 from the seeded field
__global__ void kProceduralCoeffs(LvGeom g, uint32_t seed, float *__restrict__ cx, float *__restrict__ cy,
                                  float *__restrict__ cz, float *__restrict__ d) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < g.nCell;
       c += (int64_t)gridDim.x * blockDim.x) {
    int gx, gy, gz;
    cellOf(g, c, gx, gy, gz);
    const float lx = faceCoeff(seed, 0, gx, gy, gz), ly = faceCoeff(seed, 1, gx, gy, gz),
                lz = faceCoeff(seed, 2, gx, gy, gz);
    const float ux = faceCoeff(seed, 0, gx + 1, gy, gz), uy = faceCoeff(seed, 1, gx, gy + 1, gz),
                uz = faceCoeff(seed, 2, gx, gy, gz + 1);
    cx[c] = lx; cy[c] = ly; cz[c] = lz;
    d[c] = ((lx + ux) + (ly + uy)) + (lz + uz);
  }
}

}  // namespace msbg

using namespace msbg;

// =====================================================================================
// host side
// =====================================================================================
namespace {

unsigned gridCells(int64_t n) {
  int64_t g = (n + 255) / 256;
  if (g > 152 * 16) g = 152 * 16;
  if (g < 1) g = 1;
  return (unsigned)g;
}

void freeLevel(MgLevel &L) {
  for (float **p : {&L.x, &L.b, &L.r, &L.cx, &L.cy, &L.cz, &L.d})
    if (*p) { cudaFree(*p); *p = nullptr; }
  if (L.ownsIndex) {
    if (L.slot) cudaFree(L.slot);
    if (L.active) cudaFree(L.active);
  }
  L.slot = nullptr;
  L.active = nullptr;
}

}  // namespace

namespace msbg {

void poissonFree(PoissonState *ps) {
  if (!ps) return;
  for (auto &L : ps->levels) freeLevel(L);
  for (float **p : {&ps->r, &ps->p, &ps->z, &ps->s})
    if (*p) cudaFree(*p);
  if (ps->dPartial) cudaFree(ps->dPartial);
  if (ps->dScal) cudaFree(ps->dScal);
  if (ps->hScal) cudaFreeHost(ps->hScal);
  delete ps;
}

static int allocF(msbg_gpu_ctx *ctx, float **p, int64_t n) {
  MSBG_CUDA(ctx, cudaMalloc((void **)p, (size_t)(n > 0 ? n : 1) * sizeof(float)));
  return MSBG_GPU_OK;
}

// Builds the level hierarchy over the context's current layout.
static int buildHierarchy(msbg_gpu_ctx *ctx, PoissonState *ps) {
  int rc;
  MgLevel L0{};
  L0.bs = ctx->bsx; L0.log2bs = ctx->log2bs;
  L0.nbx = ctx->nbx; L0.nby = ctx->nby; L0.nbz = ctx->nbz;
  L0.nAct = ctx->nActive; L0.nCell = ctx->nActive * ctx->voxPerBlock;
  L0.slot = ctx->dSlot; L0.active = ctx->dActive; L0.ownsIndex = false;
  ps->levels.push_back(L0);
  // block edge halves on the same blocks
  while (ps->levels.back().bs > 1) {
    MgLevel f = ps->levels.back(), c{};
    c = f;
    c.bs = f.bs / 2; c.log2bs = f.log2bs - 1;
    c.nCell = c.nAct << (3 * c.log2bs);
    c.x = c.b = c.r = c.cx = c.cy = c.cz = c.d = nullptr;
    c.ownsIndex = false;
    ps->levels.push_back(c);
  }
  // then aggregate blocks of the block grid
  while (true) {
    const MgLevel &f = ps->levels.back();
    if (f.nCell <= ps->coarsestCells || (f.nbx <= 2 && f.nby <= 2 && f.nbz <= 2)) break;
    MgLevel c{};
    c.bs = 1; c.log2bs = 0;
    c.nbx = (f.nbx + 1) / 2; c.nby = (f.nby + 1) / 2; c.nbz = (f.nbz + 1) / 2;
    const int64_t nB = (int64_t)c.nbx * c.nby * c.nbz;
    MSBG_CUDA(ctx, cudaMalloc(&c.slot, (size_t)nB * 4));
    MSBG_CUDA(ctx, cudaMalloc(&c.active, (size_t)nB * 4));
    c.ownsIndex = true;
    rc = ensureTmpSlab(ctx, (size_t)nB * 12 + 16);
    if (rc) return rc;
    int32_t *mark = (int32_t *)ctx->dTmpSlab;
    int64_t *off = (int64_t *)((char *)ctx->dTmpSlab + (((size_t)nB * 4 + 15) & ~size_t(15)));
    MSBG_CUDA(ctx, cudaMemsetAsync(mark, 0, (size_t)nB * 4, ctx->stream));
    MSBG_LAUNCH(ctx, kMarkParents, gridFor(f.nAct, 256), 256, 0, f.active, f.nAct, f.nbx, f.nby, c.nbx, c.nby, mark);
    rc = exclusiveScanFlags(ctx, mark, nB, off, ctx->dCounters + 5);
    if (rc) return rc;
    MSBG_LAUNCH(ctx, kSlotsFromMarks, gridFor(nB, 256), 256, 0, mark, off, nB, c.slot, c.active);
    int64_t cnt = 0;
    MSBG_CUDA(ctx, cudaMemcpyAsync(&cnt, ctx->dCounters + 5, 8, cudaMemcpyDeviceToHost, ctx->stream));
    MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    c.nAct = cnt;
    c.nCell = cnt;
    ps->levels.push_back(c);
  }
  // storage: levels >= 1 own x, b, r and coefficients; level 0 coefficients too
  for (size_t l = 0; l < ps->levels.size(); l++) {
    MgLevel &L = ps->levels[l];
    for (float **p : {&L.cx, &L.cy, &L.cz, &L.d}) if ((rc = allocF(ctx, p, L.nCell))) return rc;
    if (l > 0) for (float **p : {&L.x, &L.b, &L.r}) if ((rc = allocF(ctx, p, L.nCell))) return rc;
  }
  const int64_t n0 = ps->levels[0].nCell;
  for (float **p : {&ps->r, &ps->p, &ps->z, &ps->s}) if ((rc = allocF(ctx, p, n0))) return rc;
  ps->nPartial = 152 * 16;
  MSBG_CUDA(ctx, cudaMalloc(&ps->dPartial, (size_t)ps->nPartial * 2 * sizeof(double)));
  MSBG_CUDA(ctx, cudaMalloc(&ps->dScal, 16 * sizeof(double)));
  MSBG_CUDA(ctx, cudaMallocHost((void **)&ps->hScal, 16 * sizeof(double)));
  return MSBG_GPU_OK;
}

LvGeom geomOf(const MgLevel &L) {
  LvGeom g;
  g.bs = L.bs; g.log2bs = L.log2bs; g.nbx = L.nbx; g.nby = L.nby; g.nbz = L.nbz;
  g.nCell = L.nCell; g.slot = L.slot; g.active = L.active;
  return g;
}

// coarse operators of all levels from level 0's coefficients
static int buildCoarseOps(msbg_gpu_ctx *ctx, PoissonState *ps) {
  for (size_t l = 1; l < ps->levels.size(); l++) {
    MgLevel &F = ps->levels[l - 1], &C = ps->levels[l];
    MSBG_LAUNCH(ctx, kCoarseCoeffs, gridCells(C.nCell), 256, 0, geomOf(F), geomOf(C), F.cx, F.cy, F.cz, F.d,
                C.cx, C.cy, C.cz, C.d);
  }
  return MSBG_GPU_OK;
}

static int smooth(msbg_gpu_ctx *ctx, const MgLevel &L, float *x, const float *b, int nSweeps, bool redFirst) {
  const LvGeom g = geomOf(L);
  for (int s = 0; s < nSweeps; s++)
    for (int k = 0; k < 2; k++) {
      const int color = redFirst ? k : 1 - k;
      MSBG_LAUNCH(ctx, kRBGS, gridCells(L.nCell), 256, 0, g, x, b, L.cx, L.cy, L.cz, L.d, color);
    }
  return MSBG_GPU_OK;
}

// One V-cycle: x = M^{-1} b on level l (x starts at zero).
static int vcycle(msbg_gpu_ctx *ctx, PoissonState *ps, size_t l, float *x, const float *b, float *r) {
  MgLevel &L = ps->levels[l];
  const LvGeom g = geomOf(L);
  int rc;
  if (l + 1 == ps->levels.size()) {
    MSBG_LAUNCH(ctx, kCoarsestGS, 1, 1024, 0, g, x, b, L.cx, L.cy, L.cz, L.d, ps->coarsestIter);
    return MSBG_GPU_OK;
  }
  MSBG_LAUNCH(ctx, kZero, gridCells(L.nCell), 256, 0, x, L.nCell);
  if ((rc = smooth(ctx, L, x, b, ps->preSweeps, true))) return rc;
  MSBG_LAUNCH(ctx, kApply, gridCells(L.nCell), 256, 0, g, x, b, L.cx, L.cy, L.cz, L.d, r, 1);
  MgLevel &C = ps->levels[l + 1];
  MSBG_LAUNCH(ctx, kRestrictSum, gridCells(C.nCell), 256, 0, g, geomOf(C), r, C.b, C.x);
  if ((rc = vcycle(ctx, ps, l + 1, C.x, C.b, C.r))) return rc;
  MSBG_LAUNCH(ctx, kProlongAdd, gridCells(L.nCell), 256, 0, g, geomOf(C), C.x, x);
  return smooth(ctx, L, x, b, ps->postSweeps, false);
}

static int dotDev(msbg_gpu_ctx *ctx, PoissonState *ps, const float *a, const float *b, int64_t n, double *dOut) {
  MSBG_LAUNCH(ctx, kDotPartial, (unsigned)ps->nPartial, kRedThreads, 0, a, b, n, ps->dPartial);
  MSBG_LAUNCH(ctx, kSumPartials, 1, kRedThreads, 0, ps->dPartial, ps->nPartial, dOut);
  return MSBG_GPU_OK;
}

static int trueResidual(msbg_gpu_ctx *ctx, PoissonState *ps, const float *x, const float *b, double *rr,
                        double *bb) {
  const MgLevel &L = ps->levels[0];
  MSBG_LAUNCH(ctx, kResidualNorm64, (unsigned)ps->nPartial, kRedThreads, 0, geomOf(L), x, b, L.cx, L.cy, L.cz,
              L.d, ps->dPartial);
  MSBG_LAUNCH(ctx, kSumPartials2, 1, kRedThreads, 0, ps->dPartial, ps->nPartial, ps->dScal + 8);
  MSBG_CUDA(ctx, cudaMemcpyAsync(ps->hScal + 8, ps->dScal + 8, 16, cudaMemcpyDeviceToHost, ctx->stream));
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  *rr = ps->hScal[8];
  *bb = ps->hScal[9];
  return MSBG_GPU_OK;
}

int poissonEnsure(msbg_gpu_ctx *ctx) {
  if (ctx->poisson && ctx->poisson->layoutStamp == ctx->layoutStamp) return MSBG_GPU_OK;
  if (ctx->poisson) { poissonFree(ctx->poisson); ctx->poisson = nullptr; }
  PoissonState *ps = new PoissonState();
  ctx->poisson = ps;
  ps->layoutStamp = ctx->layoutStamp;
  return buildHierarchy(ctx, ps);
}

}  // namespace msbg

// ---- ABI --------------------------------------------------------------------------------
static int needLayoutP(msbg_gpu_ctx *ctx) {
  if (!ctx->layoutValid) return fail(ctx, MSBG_GPU_ERR_STATE, "no block layout: call set_refinement_map");
  return poissonEnsure(ctx);
}

static int chanF32(msbg_gpu_ctx *ctx, int chan, float **p) {
  if (chan < 0 || chan >= kMaxChannels || !ctx->ch[chan].exists)
    return fail(ctx, MSBG_GPU_ERR_ARG, "channel %d does not exist", chan);
  if (ctx->ch[chan].storage != MSBG_GPU_F32)
    return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED, "channel %d is not FP32", chan);
  *p = (float *)ctx->ch[chan].d;
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_poisson_set_coefficients(msbg_gpu_ctx *ctx, int chanCx, int chanCy, int chanCz,
                                                 int chanDiag) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  int rc = needLayoutP(ctx);
  if (rc) return rc;
  PoissonState *ps = ctx->poisson;
  MgLevel &L = ps->levels[0];
  float *src[4];
  const int ch[4] = {chanCx, chanCy, chanCz, chanDiag};
  for (int k = 0; k < 4; k++) if ((rc = chanF32(ctx, ch[k], &src[k]))) return rc;
  float *dst[4] = {L.cx, L.cy, L.cz, L.d};
  for (int k = 0; k < 4; k++)
    MSBG_CUDA(ctx, cudaMemcpyAsync(dst[k], src[k], (size_t)L.nCell * 4, cudaMemcpyDeviceToDevice, ctx->stream));
  ps->coeffsValid = true;
  return buildCoarseOps(ctx, ps);
}

extern "C" int msbg_gpu_poisson_procedural_coefficients(msbg_gpu_ctx *ctx, uint32_t seed, int chanCx, int chanCy,
                                                       int chanCz, int chanDiag) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  int rc = needLayoutP(ctx);
  if (rc) return rc;
  PoissonState *ps = ctx->poisson;
  MgLevel &L = ps->levels[0];
  MSBG_LAUNCH(ctx, kProceduralCoeffs, gridCells(L.nCell), 256, 0, geomOf(L), seed, L.cx, L.cy, L.cz, L.d);
  ps->coeffsValid = true;
  const int ch[4] = {chanCx, chanCy, chanCz, chanDiag};
  float *dst[4] = {L.cx, L.cy, L.cz, L.d};
  for (int k = 0; k < 4; k++) {
    if (ch[k] < 0) continue;
    float *p;
    if ((rc = chanF32(ctx, ch[k], &p))) return rc;
    MSBG_CUDA(ctx, cudaMemcpyAsync(p, dst[k], (size_t)L.nCell * 4, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  return buildCoarseOps(ctx, ps);
}

static int needCoeffs(msbg_gpu_ctx *ctx) {
  int rc = needLayoutP(ctx);
  if (rc) return rc;
  if (!ctx->poisson->coeffsValid) return fail(ctx, MSBG_GPU_ERR_STATE, "no Poisson coefficients set");
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_multiply_laplacian(msbg_gpu_ctx *ctx, int chanX, int chanB, int chanDstY, int calcResidual) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  int rc = needCoeffs(ctx);
  if (rc) return rc;
  float *x, *b = nullptr, *y;
  if ((rc = chanF32(ctx, chanX, &x)) || (rc = chanF32(ctx, chanDstY, &y))) return rc;
  if (calcResidual && (rc = chanF32(ctx, chanB, &b))) return rc;
  const MgLevel &L = ctx->poisson->levels[0];
  MSBG_LAUNCH(ctx, kApply, gridCells(L.nCell), 256, 0, geomOf(L), x, b, L.cx, L.cy, L.cz, L.d, y, calcResidual ? 1 : 0);
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_relax(msbg_gpu_ctx *ctx, int chanX, int chanB, int nIter, int reverseOrder) {
  if (!ctx || nIter < 0) return MSBG_GPU_ERR_ARG;
  int rc = needCoeffs(ctx);
  if (rc) return rc;
  float *x, *b;
  if ((rc = chanF32(ctx, chanX, &x)) || (rc = chanF32(ctx, chanB, &b))) return rc;
  return smooth(ctx, ctx->poisson->levels[0], x, b, nIter, !reverseOrder);
}

extern "C" int msbg_gpu_vcycle(msbg_gpu_ctx *ctx, int chanX, int chanB) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  int rc = needCoeffs(ctx);
  if (rc) return rc;
  float *x, *b;
  if ((rc = chanF32(ctx, chanX, &x)) || (rc = chanF32(ctx, chanB, &b))) return rc;
  return vcycle(ctx, ctx->poisson, 0, x, b, ctx->poisson->s);
}

extern "C" int msbg_gpu_dot(msbg_gpu_ctx *ctx, int chanA, int chanB, double *out) {
  if (!ctx || !out) return MSBG_GPU_ERR_ARG;
  int rc = needLayoutP(ctx);
  if (rc) return rc;
  float *a, *b;
  if ((rc = chanF32(ctx, chanA, &a)) || (rc = chanF32(ctx, chanB, &b))) return rc;
  PoissonState *ps = ctx->poisson;
  if ((rc = dotDev(ctx, ps, a, b, ps->levels[0].nCell, ps->dScal + 12))) return rc;
  MSBG_CUDA(ctx, cudaMemcpyAsync(ps->hScal + 12, ps->dScal + 12, 8, cudaMemcpyDeviceToHost, ctx->stream));
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  *out = ps->hScal[12];
  if (!isfinite(*out)) return fail(ctx, MSBG_GPU_ERR_NONFINITE, "dot product is not finite");  // src/msbg.cpp:4635
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_axpby(msbg_gpu_ctx *ctx, double a, int chanX, double b, int chanY) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  int rc = needLayoutP(ctx);
  if (rc) return rc;
  float *x, *y;
  if ((rc = chanF32(ctx, chanX, &x)) || (rc = chanF32(ctx, chanY, &y))) return rc;
  const int64_t n = ctx->poisson->levels[0].nCell;
  MSBG_LAUNCH(ctx, kAxpby, gridCells(n), 256, 0, a, x, b, y, n);
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_axpby_combined(msbg_gpu_ctx *ctx, double a, double b, int chanQ, int chanX, int chanP) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  int rc = needLayoutP(ctx);
  if (rc) return rc;
  float *q, *x, *p;
  if ((rc = chanF32(ctx, chanQ, &q)) || (rc = chanF32(ctx, chanX, &x)) || (rc = chanF32(ctx, chanP, &p))) return rc;
  const int64_t n = ctx->poisson->levels[0].nCell;
  MSBG_LAUNCH(ctx, kAxpbyCombined, gridCells(n), 256, 0, a, b, q, x, p, n);
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_mgpcg_solve(msbg_gpu_ctx *ctx, int chanX, int chanB, double tol, int maxIter,
                                    int *itersOut, double *relResOut) {
  if (!ctx || maxIter < 0 || !(tol > 0)) return MSBG_GPU_ERR_ARG;
  int rc = needCoeffs(ctx);
  if (rc) return rc;
  float *x, *b;
  if ((rc = chanF32(ctx, chanX, &x)) || (rc = chanF32(ctx, chanB, &b))) return rc;
  PoissonState *ps = ctx->poisson;
  const MgLevel &L = ps->levels[0];
  const LvGeom g = geomOf(L);
  const int64_t n = L.nCell;
  double *sc = ps->dScal;  // [0] rz, [1] pq, [2] rz_new, [3] rr
  // r = b - A x; z = M r; p = z; rz = <r,z>
  MSBG_LAUNCH(ctx, kApply, gridCells(n), 256, 0, g, x, b, L.cx, L.cy, L.cz, L.d, ps->r, 1);
  double rr0, bb;
  if ((rc = trueResidual(ctx, ps, x, b, &rr0, &bb))) return rc;
  const double bnorm = sqrt(bb);
  double rel = bnorm > 0 ? sqrt(rr0) / bnorm : 0.0;
  int it = 0;
  if (bnorm > 0 && rel > tol) {
    if ((rc = vcycle(ctx, ps, 0, ps->z, ps->r, ps->s))) return rc;
    MSBG_LAUNCH(ctx, kCopy, gridCells(n), 256, 0, ps->z, ps->p, n);
    if ((rc = dotDev(ctx, ps, ps->r, ps->z, n, sc + 0))) return rc;
    double prevRel = rel;
    int growth = 0;
    for (it = 1; it <= maxIter; it++) {
      MSBG_LAUNCH(ctx, kApply, gridCells(n), 256, 0, g, ps->p, nullptr, L.cx, L.cy, L.cz, L.d, ps->s, 0);
      if ((rc = dotDev(ctx, ps, ps->p, ps->s, n, sc + 1))) return rc;
      MSBG_LAUNCH(ctx, kCgUpdateXR, gridCells(n), 256, 0, sc, ps->p, ps->s, x, ps->r, n);
      if ((rc = dotDev(ctx, ps, ps->r, ps->r, n, sc + 3))) return rc;
      MSBG_CUDA(ctx, cudaMemcpyAsync(ps->hScal + 3, sc + 3, 8, cudaMemcpyDeviceToHost, ctx->stream));
      MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      rel = sqrt(ps->hScal[3]) / bnorm;
      if (!isfinite(rel)) return fail(ctx, MSBG_GPU_ERR_DIVERGED, "residual is not finite at iteration %d", it);
      growth = rel > prevRel ? growth + 1 : 0;
      if (growth >= 8) return fail(ctx, MSBG_GPU_ERR_DIVERGED, "residual grew for 8 iterations (%g)", rel);
      prevRel = rel;
      if (rel <= tol) {
        // confirm with the FP64 true residual; continue if the recurrence drifted
        double rr;
        if ((rc = trueResidual(ctx, ps, x, b, &rr, &bb))) return rc;
        rel = sqrt(rr) / bnorm;
        if (rel <= tol) break;
        MSBG_LAUNCH(ctx, kApply, gridCells(n), 256, 0, g, x, b, L.cx, L.cy, L.cz, L.d, ps->r, 1);
      }
      if ((rc = vcycle(ctx, ps, 0, ps->z, ps->r, ps->s))) return rc;
      if ((rc = dotDev(ctx, ps, ps->r, ps->z, n, sc + 2))) return rc;
      MSBG_LAUNCH(ctx, kCgUpdateP, gridCells(n), 256, 0, sc, ps->z, ps->p, n);
      MSBG_CUDA(ctx, cudaMemcpyAsync(sc + 0, sc + 2, 8, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    if (it > maxIter) it = maxIter;
  }
  if (itersOut) *itersOut = it;
  if (relResOut) *relResOut = rel;
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_mg_info(msbg_gpu_ctx *ctx, int *nLevels, int64_t *cellsPerLevel, int cap) {
  if (!ctx || !nLevels) return MSBG_GPU_ERR_ARG;
  int rc = needLayoutP(ctx);
  if (rc) return rc;
  *nLevels = (int)ctx->poisson->levels.size();
  for (int l = 0; l < *nLevels && l < cap && cellsPerLevel; l++) cellsPerLevel[l] = ctx->poisson->levels[l].nCell;
  return MSBG_GPU_OK;
}
