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
// post-smoothing black first; the coarsest level (<= 512 cells) is relaxed by one
// CTA for many sweeps.
//
// Precision.  Every kernel is templated on the storage type (FP32, or FP16 for the
// mixed-precision solve); arithmetic is FP32, dot products and norms FP64.  The
// mixed solve is FP32 iterative refinement: the outer residual b - A x uses the
// FP32 operator, each correction comes from an FP16-storage MG-PCG on the scaled
// residual to a loose inner tolerance.
#include <math.h>
#include <string.h>

#include <vector>

#include "internal.cuh"
#include "poisson.cuh"

namespace msbg {

// ---------------------------------------------------------------------------------
// cell addressing on a level
// ---------------------------------------------------------------------------------
struct Cell {
  int gx, gy, gz;  // global cell coordinates on the level
  int lx, ly, lz;  // inside the block
};

__device__ __forceinline__ Cell cellOf(const LvGeom &g, int64_t c) {
  const int s = (int)(c >> (3 * g.log2bs));
  const int v = (int)(c & ((1 << (3 * g.log2bs)) - 1));
  const int m = g.bs - 1;
  Cell q;
  q.lx = v & m; q.ly = (v >> g.log2bs) & m; q.lz = v >> (2 * g.log2bs);
  const int bid = g.active[s];
  const int bx = bid % g.nbx, by = (bid / g.nbx) % g.nby, bz = bid / (g.nbx * g.nby);
  q.gx = (bx << g.log2bs) + q.lx;
  q.gy = (by << g.log2bs) + q.ly;
  q.gz = (bz << g.log2bs) + q.lz;
  return q;
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

// The six neighbour indices of cell c: inside the block by offset, across a block
// face through the slot map (-1: outside / inactive).
struct Nb6 {
  int64_t xm, xp, ym, yp, zm, zp;
};
__device__ __forceinline__ Nb6 neighbours(const LvGeom &g, int64_t c, const Cell &q) {
  Nb6 n;
  const int e = g.bs - 1;
  const int64_t sy = (int64_t)g.bs, sz = (int64_t)g.bs * g.bs;
  n.xm = q.lx > 0 ? c - 1 : cellIdx(g, q.gx - 1, q.gy, q.gz);
  n.xp = q.lx < e ? c + 1 : cellIdx(g, q.gx + 1, q.gy, q.gz);
  n.ym = q.ly > 0 ? c - sy : cellIdx(g, q.gx, q.gy - 1, q.gz);
  n.yp = q.ly < e ? c + sy : cellIdx(g, q.gx, q.gy + 1, q.gz);
  n.zm = q.lz > 0 ? c - sz : cellIdx(g, q.gx, q.gy, q.gz - 1);
  n.zp = q.lz < e ? c + sz : cellIdx(g, q.gx, q.gy, q.gz + 1);
  return n;
}

// (A x)_c in compute type R
template <typename R, typename V, typename Cf>
__device__ __forceinline__ R applyAt(const V *__restrict__ x, const Cf *__restrict__ cx, const Cf *__restrict__ cy,
                                     const Cf *__restrict__ cz, const Cf *__restrict__ d, int64_t c, const Nb6 &n) {
  R s = (R)ldv(d + c) * (R)ldv(x + c);
  if (n.xm >= 0) s -= (R)ldv(cx + c) * (R)ldv(x + n.xm);
  if (n.xp >= 0) s -= (R)ldv(cx + n.xp) * (R)ldv(x + n.xp);
  if (n.ym >= 0) s -= (R)ldv(cy + c) * (R)ldv(x + n.ym);
  if (n.yp >= 0) s -= (R)ldv(cy + n.yp) * (R)ldv(x + n.yp);
  if (n.zm >= 0) s -= (R)ldv(cz + c) * (R)ldv(x + n.zm);
  if (n.zp >= 0) s -= (R)ldv(cz + n.zp) * (R)ldv(x + n.zp);
  return s;
}

#define GRID_STRIDE(c, n) \
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < (n); c += (int64_t)gridDim.x * blockDim.x)

// ---------------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------------
// mode 0: y = A x; mode 1: y = b - A x
template <typename V, typename Cf>
__global__ void kApply(LvGeom g, const V *__restrict__ x, const V *__restrict__ b, const Cf *__restrict__ cx,
                       const Cf *__restrict__ cy, const Cf *__restrict__ cz, const Cf *__restrict__ d,
                       V *__restrict__ y, int mode) {
  GRID_STRIDE(c, g.nCell) {
    const Cell q = cellOf(g, c);
    const float ax = applyAt<float>(x, cx, cy, cz, d, c, neighbours(g, c, q));
    stv(y + c, mode ? ldv(b + c) - ax : ax);
  }
}

// Red-black Gauss-Seidel half sweep: cells with (gx+gy+gz)&1 == color get
// x = (b + sum c x_nb) / d.
template <typename V, typename Cf>
__device__ __forceinline__ void rbgsCell(const LvGeom &g, V *__restrict__ x, const V *__restrict__ b,
                                         const Cf *__restrict__ cx, const Cf *__restrict__ cy,
                                         const Cf *__restrict__ cz, const Cf *__restrict__ d, int64_t c,
                                         int color) {
  const Cell q = cellOf(g, c);
  if (((q.gx + q.gy + q.gz) & 1) != color) return;
  const Nb6 n = neighbours(g, c, q);
  float s = ldv(b + c);
  if (n.xm >= 0) s += ldv(cx + c) * ldv(x + n.xm);
  if (n.xp >= 0) s += ldv(cx + n.xp) * ldv(x + n.xp);
  if (n.ym >= 0) s += ldv(cy + c) * ldv(x + n.ym);
  if (n.yp >= 0) s += ldv(cy + n.yp) * ldv(x + n.yp);
  if (n.zm >= 0) s += ldv(cz + c) * ldv(x + n.zm);
  if (n.zp >= 0) s += ldv(cz + n.zp) * ldv(x + n.zp);
  stv(x + c, s / ldv(d + c));
}

template <typename V, typename Cf>
__global__ void kRBGS(LvGeom g, V *__restrict__ x, const V *__restrict__ b, const Cf *__restrict__ cx,
                      const Cf *__restrict__ cy, const Cf *__restrict__ cz, const Cf *__restrict__ d, int color) {
  GRID_STRIDE(c, g.nCell) rbgsCell(g, x, b, cx, cy, cz, d, c, color);
}

// Coarsest level: nIter red-black sweeps by one CTA from x = 0.
template <typename V, typename Cf>
__global__ void kCoarsestGS(LvGeom g, V *__restrict__ x, const V *__restrict__ b, const Cf *__restrict__ cx,
                            const Cf *__restrict__ cy, const Cf *__restrict__ cz, const Cf *__restrict__ d,
                            int nIter) {
  for (int64_t c = threadIdx.x; c < g.nCell; c += blockDim.x) stv(x + c, 0.0f);
  __syncthreads();
  for (int it = 0; it < nIter; it++)
    for (int color = 0; color < 2; color++) {
      for (int64_t c = threadIdx.x; c < g.nCell; c += blockDim.x) rbgsCell(g, x, b, cx, cy, cz, d, c, color);
      __syncthreads();
    }
}

// b_C = R r_F (sum of the active children); x_C = 0.
template <typename V>
__global__ void kRestrictSum(LvGeom gf, LvGeom gc, const V *__restrict__ rf, V *__restrict__ bc, V *__restrict__ xc) {
  GRID_STRIDE(c, gc.nCell) {
    const Cell q = cellOf(gc, c);
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const int64_t j = cellIdx(gf, 2 * q.gx + (k & 1), 2 * q.gy + ((k >> 1) & 1), 2 * q.gz + (k >> 2));
      if (j >= 0) s += ldv(rf + j);
    }
    stv(bc + c, s);
    stv(xc + c, 0.0f);
  }
}

// x_F += P x_C (constant injection of the parent's value)
template <typename V>
__global__ void kProlongAdd(LvGeom gf, LvGeom gc, const V *__restrict__ xc, V *__restrict__ xf) {
  GRID_STRIDE(c, gf.nCell) {
    const Cell q = cellOf(gf, c);
    const int64_t p = cellIdx(gc, q.gx >> 1, q.gy >> 1, q.gz >> 1);
    if (p >= 0) stv(xf + c, ldv(xf + c) + ldv(xc + p));
  }
}

// Coarse operator P^T A P / 2 from the fine level's coefficients (FP32).
__global__ void kCoarseCoeffs(LvGeom gf, LvGeom gc, const float *__restrict__ fcx, const float *__restrict__ fcy,
                              const float *__restrict__ fcz, const float *__restrict__ fd, float *__restrict__ ccx,
                              float *__restrict__ ccy, float *__restrict__ ccz, float *__restrict__ cd) {
  GRID_STRIDE(c, gc.nCell) {
    const Cell q = cellOf(gc, c);
    int64_t ch[8];
#pragma unroll
    for (int k = 0; k < 8; k++)
      ch[k] = cellIdx(gf, 2 * q.gx + (k & 1), 2 * q.gy + ((k >> 1) & 1), 2 * q.gz + (k >> 2));
    double dsum = 0.0, lx = 0.0, ly = 0.0, lz = 0.0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
      if (ch[k] < 0) continue;
      const int ix = k & 1, iy = (k >> 1) & 1, iz = k >> 2;
      const int fx = 2 * q.gx + ix, fy = 2 * q.gy + iy, fz = 2 * q.gz + iz;
      dsum += fd[ch[k]];
      // a child's lower face is external on the coarse cell's lower side, internal
      // (coupling to the sibling below) otherwise
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

__global__ void kToHalf(const float *__restrict__ a, __half *__restrict__ b, int64_t n) {
  GRID_STRIDE(i, n) b[i] = __float2half_rn(a[i]);
}

// ---- reductions ----------------------------------------------------------------------
// partial[blockIdx] = sum a*b (FP64 accumulation)
template <typename V>
__global__ void kDotPartial(const V *__restrict__ a, const V *__restrict__ b, int64_t n, double *__restrict__ partial) {
  double s = 0.0;
  GRID_STRIDE(i, n) s += (double)ldv(a + i) * (double)ldv(b + i);
  s = blockSum(s);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

__global__ void kSumPartials(const double *__restrict__ partial, int n, double *__restrict__ out) {
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += partial[i];
  s = blockSum(s);
  if (threadIdx.x == 0) *out = s;
}

// true residual in FP64 (FP32 operator data): partial[block] = {sum (b - A x)^2, sum b^2}
__global__ void kResidualNorm64(LvGeom g, const float *__restrict__ x, const float *__restrict__ b,
                                const float *__restrict__ cx, const float *__restrict__ cy,
                                const float *__restrict__ cz, const float *__restrict__ d,
                                double *__restrict__ partial) {
  double rr = 0.0, bb = 0.0;
  GRID_STRIDE(c, g.nCell) {
    const Cell q = cellOf(g, c);
    const double r = (double)b[c] - applyAt<double>(x, cx, cy, cz, d, c, neighbours(g, c, q));
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
// alpha = sc[0] / sc[1]; x += alpha p; r -= alpha q; partial[block] = sum r^2 (new r)
template <typename V>
__global__ void kCgUpdateXR(const double *__restrict__ sc, const V *__restrict__ p, const V *__restrict__ q,
                            V *__restrict__ x, V *__restrict__ r, int64_t n, double *__restrict__ partial) {
  const float alpha = sc[1] != 0.0 ? (float)(sc[0] / sc[1]) : 0.0f;
  double rr = 0.0;
  GRID_STRIDE(i, n) {
    stv(x + i, fmaf(alpha, ldv(p + i), ldv(x + i)));
    const float rn = fmaf(-alpha, ldv(q + i), ldv(r + i));
    stv(r + i, rn);
    const double rs = ldv(r + i);  // the stored value
    rr += rs * rs;
  }
  rr = blockSum(rr);
  if (threadIdx.x == 0) partial[blockIdx.x] = rr;
}
// beta = sc[2] / sc[0]; p = z + beta p
template <typename V>
__global__ void kCgUpdateP(const double *__restrict__ sc, const V *__restrict__ z, V *__restrict__ p, int64_t n) {
  const float beta = sc[0] != 0.0 ? (float)(sc[2] / sc[0]) : 0.0f;
  GRID_STRIDE(i, n) stv(p + i, fmaf(beta, ldv(p + i), ldv(z + i)));
}
template <typename V>
__global__ void kCopy(const V *__restrict__ a, V *__restrict__ b, int64_t n) {
  GRID_STRIDE(i, n) b[i] = a[i];
}
template <typename V>
__global__ void kZero(V *p, int64_t n) {
  GRID_STRIDE(i, n) stv(p + i, 0.0f);
}
// AXPBYChannelCombined: X += aP; P = Q + bP (FP64 arithmetic, src/msbg.cpp:4651-4768)
__global__ void kAxpbyCombined(double a, double b, const float *__restrict__ q, float *__restrict__ x,
                               float *__restrict__ p, int64_t n) {
  GRID_STRIDE(i, n) {
    const double pi = p[i];
    x[i] = (float)((double)x[i] + a * pi);
    p[i] = (float)((double)q[i] + b * pi);
  }
}
// AXPBYChannel: Y = aX + bY (src/msbg.cpp:4773-4872)
__global__ void kAxpby(double a, const float *__restrict__ x, double b, float *__restrict__ y, int64_t n) {
  GRID_STRIDE(i, n) y[i] = (float)(a * (double)x[i] + b * (double)y[i]);
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

// ---- coarsest level: exact solve with a dense inverse ---------------------------
// A[c][c] = d_c, A[c][nb] = -c_f (FP64, row-major, n = cells of the level)
__global__ void kDenseOperator(LvGeom g, const float *__restrict__ cx, const float *__restrict__ cy,
                               const float *__restrict__ cz, const float *__restrict__ d, double *__restrict__ A,
                               int64_t n) {
  GRID_STRIDE(c, g.nCell) {
    const Cell q = cellOf(g, c);
    const Nb6 nb = neighbours(g, c, q);
    double *row = A + c * n;
    row[c] = d[c];
    if (nb.xm >= 0) row[nb.xm] = -(double)cx[c];
    if (nb.xp >= 0) row[nb.xp] = -(double)cx[nb.xp];
    if (nb.ym >= 0) row[nb.ym] = -(double)cy[c];
    if (nb.yp >= 0) row[nb.yp] = -(double)cy[nb.yp];
    if (nb.zm >= 0) row[nb.zm] = -(double)cz[c];
    if (nb.zp >= 0) row[nb.zp] = -(double)cz[nb.zp];
  }
}
// x = inv b, one warp per row
template <typename V>
__global__ void kCoarsestDense(const float *__restrict__ inv, const V *__restrict__ b, V *__restrict__ x, int n) {
  const int row = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (row >= n) return;
  const float *a = inv + (int64_t)row * n;
  float s = 0.f;
  for (int j = lane; j < n; j += 32) s = fmaf(a[j], ldv(b + j), s);
#pragma unroll
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) stv(x + row, s);
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
  return __fadd_rn(0.5f, __fmul_rn(__fmul_rn(1.5f, (float)(h >> 8)), 1.0f / 16777216.0f));
}
// cx, cy, cz (lower faces) and d (all six faces) of level 0 from the seeded field
__global__ void kProceduralCoeffs(LvGeom g, uint32_t seed, float *__restrict__ cx, float *__restrict__ cy,
                                  float *__restrict__ cz, float *__restrict__ d) {
  GRID_STRIDE(c, g.nCell) {
    const Cell q = cellOf(g, c);
    const float lx = faceCoeff(seed, 0, q.gx, q.gy, q.gz), ly = faceCoeff(seed, 1, q.gx, q.gy, q.gz),
                lz = faceCoeff(seed, 2, q.gx, q.gy, q.gz);
    const float ux = faceCoeff(seed, 0, q.gx + 1, q.gy, q.gz), uy = faceCoeff(seed, 1, q.gx, q.gy + 1, q.gz),
                uz = faceCoeff(seed, 2, q.gx, q.gy, q.gz + 1);
    cx[c] = lx; cy[c] = ly; cz[c] = lz;
    d[c] = __fadd_rn(__fadd_rn(__fadd_rn(lx, ux), __fadd_rn(ly, uy)), __fadd_rn(lz, uz));
  }
}

}  // namespace msbg

using namespace msbg;

// =====================================================================================
// host side
// =====================================================================================
namespace msbg {

static unsigned gridCells(int64_t n) {
  int64_t g = (n + 255) / 256;
  if (g > 152 * 16) g = 152 * 16;
  if (g < 1) g = 1;
  return (unsigned)g;
}

template <typename T>
static int allocT(msbg_gpu_ctx *ctx, T **p, int64_t n) {
  MSBG_CUDA(ctx, cudaMalloc((void **)p, (size_t)(n > 0 ? n : 1) * sizeof(T)));
  return MSBG_GPU_OK;
}

void poissonFree(PoissonState *ps) {
  if (!ps) return;
  for (auto &L : ps->levels) {
    if (L.ownsIndex) {
      if (L.slot) cudaFree(L.slot);
      if (L.active) cudaFree(L.active);
    }
  }
  for (PrecSet *P : {&ps->f32, &ps->f16}) {
    for (auto *v : {&P->x, &P->b, &P->r, &P->cx, &P->cy, &P->cz, &P->d})
      for (void *q : *v) if (q) cudaFree(q);
    for (void *q : {P->vr, P->vp, P->vz, P->vs, P->ve, P->vb}) if (q) cudaFree(q);
  }
  if (ps->dCoarseInv) cudaFree(ps->dCoarseInv);
  if (ps->dNbr) cudaFree(ps->dNbr);
  if (ps->dBpar) cudaFree(ps->dBpar);
  if (ps->dParList) cudaFree(ps->dParList);
  if (ps->dPartial) cudaFree(ps->dPartial);
  if (ps->dListBuf) cudaFree(ps->dListBuf);
  if (ps->dListPart) cudaFree(ps->dListPart);
  if (ps->dScal) cudaFree(ps->dScal);
  if (ps->hScal) cudaFreeHost(ps->hScal);
  delete ps;
}

LvGeom geomOf(const MgLevel &L) {
  LvGeom g;
  g.bs = L.bs; g.log2bs = L.log2bs; g.nbx = L.nbx; g.nby = L.nby; g.nbz = L.nbz;
  g.nCell = L.nCell; g.slot = L.slot; g.active = L.active;
  return g;
}

// Level geometry over the context's current layout and the FP32 arrays.
static int buildHierarchy(msbg_gpu_ctx *ctx, PoissonState *ps) {
  int rc;
  MgLevel L0{};
  L0.bs = ctx->bsx; L0.log2bs = ctx->log2bs;
  L0.nbx = ctx->nbx; L0.nby = ctx->nby; L0.nbz = ctx->nbz;
  L0.nAct = ctx->nActive; L0.nCell = ctx->nActive * ctx->voxPerBlock;
  L0.slot = ctx->dSlot; L0.active = ctx->dActive; L0.ownsIndex = false;
  L0.sameSet = true;
  ps->levels.push_back(L0);
  while (ps->levels.back().bs > 1) {  // block edge halves on the same blocks
    MgLevel c = ps->levels.back();
    c.bs /= 2; c.log2bs -= 1;
    c.nCell = c.nAct << (3 * c.log2bs);
    c.ownsIndex = false;
    ps->levels.push_back(c);
  }
  // smoother tiles: 32x16x8 on bs-32 levels, the block on bs-16 and bs-8 levels,
  // pointwise red-black below
  for (auto &L : ps->levels) L.tile = (L.sameSet && L.bs >= 8) ? L.bs : 0;
  while (true) {  // then 2x2x2 aggregation of the block grid
    const MgLevel &f = ps->levels.back();
    if (f.nCell <= ps->coarsestCells || (f.nbx <= 2 && f.nby <= 2 && f.nbz <= 2)) break;
    MgLevel c{};
    c.bs = 1; c.log2bs = 0;
    c.nbx = (f.nbx + 1) / 2; c.nby = (f.nby + 1) / 2; c.nbz = (f.nbz + 1) / 2;
    const int64_t nB = (int64_t)c.nbx * c.nby * c.nbz;
    MSBG_CUDA(ctx, cudaMalloc(&c.slot, (size_t)nB * 4));
    MSBG_CUDA(ctx, cudaMalloc(&c.active, (size_t)nB * 4));
    c.ownsIndex = true;
    if ((rc = ensureTmpSlab(ctx, (size_t)nB * 12 + 16))) return rc;
    int32_t *mark = (int32_t *)ctx->dTmpSlab;
    int64_t *off = (int64_t *)((char *)ctx->dTmpSlab + (((size_t)nB * 4 + 15) & ~size_t(15)));
    MSBG_CUDA(ctx, cudaMemsetAsync(mark, 0, (size_t)nB * 4, ctx->stream));
    MSBG_LAUNCH(ctx, kMarkParents, gridFor(f.nAct, 256), 256, 0, f.active, f.nAct, f.nbx, f.nby, c.nbx, c.nby, mark);
    if ((rc = exclusiveScanFlags(ctx, mark, nB, off, ctx->dCounters + 5))) return rc;
    MSBG_LAUNCH(ctx, kSlotsFromMarks, gridFor(nB, 256), 256, 0, mark, off, nB, c.slot, c.active);
    int64_t cnt = 0;
    MSBG_CUDA(ctx, cudaMemcpyAsync(&cnt, ctx->dCounters + 5, 8, cudaMemcpyDeviceToHost, ctx->stream));
    MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    c.nAct = cnt;
    c.nCell = cnt;
    ps->levels.push_back(c);
  }
  const size_t nL = ps->levels.size();
  PrecSet &P = ps->f32;
  for (auto *v : {&P.x, &P.b, &P.r, &P.cx, &P.cy, &P.cz, &P.d}) v->assign(nL, nullptr);
  for (size_t l = 0; l < nL; l++) {
    const int64_t n = ps->levels[l].nCell;
    for (auto *v : {&P.cx, &P.cy, &P.cz, &P.d}) if ((rc = allocT(ctx, (float **)&(*v)[l], n))) return rc;
    if (l > 0) for (auto *v : {&P.x, &P.b, &P.r}) if ((rc = allocT(ctx, (float **)&(*v)[l], n))) return rc;
  }
  // the FP32 CG work vectors are allocated by their first user (ensureF32Work): the
  // mixed-precision solve never needs them
  ps->nPartial = 152 * 16;
  MSBG_CUDA(ctx, cudaMalloc(&ps->dPartial, (size_t)ps->nPartial * 2 * sizeof(double)));
  MSBG_CUDA(ctx, cudaMalloc(&ps->dScal, 32 * sizeof(double)));
  MSBG_CUDA(ctx, cudaMallocHost((void **)&ps->hScal, 32 * sizeof(double)));
  return blkBuildTables(ctx, ps);
}

// Inverse of a symmetric positive definite matrix (row-major, n x n) through its
// Cholesky factor, in FP64; false when a pivot is not positive.
static bool spdInverse(std::vector<double> &A, int n, std::vector<float> &inv) {
  std::vector<double> &L = A;  // factor in place (lower triangle)
  for (int j = 0; j < n; j++) {
    double s = L[(size_t)j * n + j];
    for (int k = 0; k < j; k++) s -= L[(size_t)j * n + k] * L[(size_t)j * n + k];
    if (!(s > 0.0)) return false;
    const double dj = sqrt(s);
    L[(size_t)j * n + j] = dj;
    for (int i = j + 1; i < n; i++) {
      double t = L[(size_t)i * n + j];
      for (int k = 0; k < j; k++) t -= L[(size_t)i * n + k] * L[(size_t)j * n + k];
      L[(size_t)i * n + j] = t / dj;
    }
  }
  inv.assign((size_t)n * n, 0.0f);
  std::vector<double> y(n);
  for (int c = 0; c < n; c++) {
    for (int i = 0; i < n; i++) {  // L y = e_c
      double t = i == c ? 1.0 : 0.0;
      for (int k = 0; k < i; k++) t -= L[(size_t)i * n + k] * y[k];
      y[i] = t / L[(size_t)i * n + i];
    }
    for (int i = n - 1; i >= 0; i--) {  // L^T x = y
      double t = y[i];
      for (int k = i + 1; k < n; k++) t -= L[(size_t)k * n + i] * y[k];
      y[i] = t / L[(size_t)i * n + i];
    }
    for (int i = 0; i < n; i++) inv[(size_t)i * n + c] = (float)y[i];
  }
  return true;
}

static int buildCoarseInverse(msbg_gpu_ctx *ctx, PoissonState *ps) {
  const size_t l = ps->levels.size() - 1;
  const MgLevel &C = ps->levels[l];
  const int64_t n = C.nCell;
  ps->coarseInvValid = false;
  if (n <= 0) return MSBG_GPU_OK;
  if (n > 4096) return fail(ctx, MSBG_GPU_ERR_CAPACITY, "coarsest level has %lld cells", (long long)n);
  int rc;
  if ((rc = ensureTmpSlab(ctx, (size_t)n * n * 8))) return rc;
  double *dA = (double *)ctx->dTmpSlab;
  MSBG_CUDA(ctx, cudaMemsetAsync(dA, 0, (size_t)n * n * 8, ctx->stream));
  const PrecSet &P = ps->f32;
  MSBG_LAUNCH(ctx, kDenseOperator, gridCells(n), 256, 0, geomOf(C), (const float *)P.cx[l], (const float *)P.cy[l],
              (const float *)P.cz[l], (const float *)P.d[l], dA, n);
  std::vector<double> A((size_t)n * n);
  MSBG_CUDA(ctx, cudaMemcpyAsync(A.data(), dA, (size_t)n * n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  std::vector<float> inv;
  if (!spdInverse(A, (int)n, inv))
    return fail(ctx, MSBG_GPU_ERR_DIVERGED, "coarsest operator is not positive definite");
  if (ps->coarseInvN != n) {
    if (ps->dCoarseInv) cudaFree(ps->dCoarseInv);
    ps->dCoarseInv = nullptr;
    MSBG_CUDA(ctx, cudaMalloc(&ps->dCoarseInv, (size_t)n * n * 4));
    ps->coarseInvN = n;
  }
  MSBG_CUDA(ctx, cudaMemcpyAsync(ps->dCoarseInv, inv.data(), (size_t)n * n * 4, cudaMemcpyHostToDevice, ctx->stream));
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ps->coarseInvValid = true;
  return MSBG_GPU_OK;
}

// coarse operators of all levels from level 0's coefficients (FP32), the dense
// inverse of the coarsest one; drops FP16 copies
static int buildCoarseOps(msbg_gpu_ctx *ctx, PoissonState *ps) {
  PrecSet &P = ps->f32;
  for (size_t l = 1; l < ps->levels.size(); l++) {
    const MgLevel &F = ps->levels[l - 1], &C = ps->levels[l];
    MSBG_LAUNCH(ctx, kCoarseCoeffs, gridCells(C.nCell), 256, 0, geomOf(F), geomOf(C), (float *)P.cx[l - 1],
                (float *)P.cy[l - 1], (float *)P.cz[l - 1], (float *)P.d[l - 1], (float *)P.cx[l], (float *)P.cy[l],
                (float *)P.cz[l], (float *)P.d[l]);
  }
  ps->f16Valid = false;
  return buildCoarseInverse(ctx, ps);
}

// FP16 copies of every level's coefficients and the FP16 work vectors
static int ensureHalf(msbg_gpu_ctx *ctx, PoissonState *ps) {
  if (ps->f16Valid) return MSBG_GPU_OK;
  int rc;
  PrecSet &H = ps->f16;
  const size_t nL = ps->levels.size();
  if (H.cx.size() != nL) {
    for (auto *v : {&H.x, &H.b, &H.r, &H.cx, &H.cy, &H.cz, &H.d}) v->assign(nL, nullptr);
    for (size_t l = 0; l < nL; l++) {
      const int64_t n = ps->levels[l].nCell;
      for (auto *v : {&H.cx, &H.cy, &H.cz, &H.d}) if ((rc = allocT(ctx, (__half **)&(*v)[l], n))) return rc;
      if (l > 0) for (auto *v : {&H.x, &H.b, &H.r}) if ((rc = allocT(ctx, (__half **)&(*v)[l], n))) return rc;
    }
    const int64_t n0 = ps->levels[0].nCell;
    for (void **q : {&H.vr, &H.vp, &H.vz, &H.vs, &H.ve, &H.vb}) if ((rc = allocT(ctx, (__half **)q, n0))) return rc;
  }
  for (size_t l = 0; l < nL; l++) {
    const int64_t n = ps->levels[l].nCell;
    void *src[4] = {ps->f32.cx[l], ps->f32.cy[l], ps->f32.cz[l], ps->f32.d[l]};
    void *dst[4] = {H.cx[l], H.cy[l], H.cz[l], H.d[l]};
    for (int k = 0; k < 4; k++) MSBG_LAUNCH(ctx, kToHalf, gridCells(n), 256, 0, (const float *)src[k], (__half *)dst[k], n);
  }
  ps->f16Valid = true;
  return MSBG_GPU_OK;
}

template <typename V>
struct Arr {
  const PrecSet &P;
  size_t l;
  V *x() const { return (V *)P.x[l]; }
  V *b() const { return (V *)P.b[l]; }
  V *r() const { return (V *)P.r[l]; }
  V *cx() const { return (V *)P.cx[l]; }
  V *cy() const { return (V *)P.cy[l]; }
  V *cz() const { return (V *)P.cz[l]; }
  V *d() const { return (V *)P.d[l]; }
};

// Smoothing passes on level l.  Tile levels: per pass the two tile colours (0,1;
// reversed 1,0) with k in-tile red-black sweeps each.  Pointwise levels: k
// red-black sweeps per pass.  first: kOwnZero for a pre-smoother whose x starts
// at zero (x is not read), kOwnCorr for a post-smoother that adds the coarse
// correction xc while it loads; other levels do those steps as separate kernels.
enum { kFirstNone = 0, kFirstZero = 1, kFirstCorr = 2 };

template <typename V>
static int smoothLevel(msbg_gpu_ctx *ctx, PoissonState *ps, const PrecSet &P, size_t l, V *x, const V *b,
                       int passes, bool reverse, int first, const V *xc) {
  const MgLevel &L = ps->levels[l];
  const int k = ps->tileIters;
  int rc;
  if (L.tile) {
    if (passes == 0) {
      if (first == kFirstZero) MSBG_LAUNCH(ctx, (kZero<V>), gridCells(L.nCell), 256, 0, x, L.nCell);
      if (first == kFirstCorr) {
        const MgLevel &C = ps->levels[l + 1];
        MSBG_LAUNCH(ctx, (kProlongAdd<V>), gridCells(L.nCell), 256, 0, geomOf(L), geomOf(C), xc, x);
      }
      return MSBG_GPU_OK;
    }
    for (int p = 0; p < passes; p++)
      for (int i = 0; i < 2; i++) {
        const int tc = reverse ? 1 - i : i;
        int flags = 0;
        if (p == 0 && first == kFirstZero) flags = i == 0 ? (kOwnZero | kHaloZero) : kOwnZero;
        if (p == 0 && first == kFirstCorr) flags = i == 0 ? (kOwnCorr | kHaloCorr) : kOwnCorr;
        if ((rc = blkSmoothColor<V>(ctx, ps, l, P, x, b, xc, tc, k, reverse ? 1 : 0, flags))) return rc;
      }
    return MSBG_GPU_OK;
  }
  const LvGeom g = geomOf(L);
  const Arr<V> a{P, l};
  if (first == kFirstZero) MSBG_LAUNCH(ctx, (kZero<V>), gridCells(L.nCell), 256, 0, x, L.nCell);
  if (first == kFirstCorr) {
    const MgLevel &C = ps->levels[l + 1];
    MSBG_LAUNCH(ctx, (kProlongAdd<V>), gridCells(L.nCell), 256, 0, g, geomOf(C), xc, x);
  }
  for (int s = 0; s < passes * k; s++)
    for (int i = 0; i < 2; i++) {
      const int color = reverse ? 1 - i : i;
      MSBG_LAUNCH(ctx, (kRBGS<V, V>), gridCells(L.nCell), 256, 0, g, x, b, a.cx(), a.cy(), a.cz(), a.d(), color);
    }
  return MSBG_GPU_OK;
}

// y = A x (mode 0) or y = b - A x (mode 1); dotOut: also sum x.y into *dotOut (device)
template <typename V>
static int applyT(msbg_gpu_ctx *ctx, PoissonState *ps, const PrecSet &P, size_t l, const V *x, const V *b, V *y,
                  int mode, double *dotOut = nullptr) {
  const MgLevel &L = ps->levels[l];
  if (L.sameSet && L.bs >= 4) return blkApply<V>(ctx, ps, l, P, x, b, y, mode, dotOut, nullptr, nullptr);
  const Arr<V> a{P, l};
  MSBG_LAUNCH(ctx, (kApply<V, V>), gridCells(L.nCell), 256, 0, geomOf(L), x, b, a.cx(), a.cy(), a.cz(), a.d(), y,
              mode);
  if (dotOut) {
    MSBG_LAUNCH(ctx, (kDotPartial<V>), (unsigned)ps->nPartial, kRedThreads, 0, x, (const V *)y, L.nCell, ps->dPartial);
    MSBG_LAUNCH(ctx, kSumPartials, 1, kRedThreads, 0, ps->dPartial, ps->nPartial, dotOut);
  }
  return MSBG_GPU_OK;
}

// One V-cycle: x = M^{-1} b on level l (x starts at zero; its old content is ignored).
template <typename V>
static int vcycleT(msbg_gpu_ctx *ctx, PoissonState *ps, const PrecSet &P, size_t l, V *x, const V *b, V *r) {
  const MgLevel &L = ps->levels[l];
  const LvGeom g = geomOf(L);
  const Arr<V> a{P, l};
  int rc;
  if (l + 1 == ps->levels.size()) {
    if (ps->coarsestIter > 0) {
      MSBG_LAUNCH(ctx, (kCoarsestGS<V, V>), 1, 1024, 0, g, x, b, a.cx(), a.cy(), a.cz(), a.d(), ps->coarsestIter);
    } else {
      if (!ps->coarseInvValid) return fail(ctx, MSBG_GPU_ERR_STATE, "coarsest inverse missing");
      MSBG_LAUNCH(ctx, (kCoarsestDense<V>), gridFor(L.nCell * 32, 256), 256, 0, ps->dCoarseInv, b, x, (int)L.nCell);
    }
    return MSBG_GPU_OK;
  }
  if ((rc = smoothLevel<V>(ctx, ps, P, l, x, b, ps->preSweeps, false, kFirstZero, nullptr))) return rc;
  const MgLevel &C = ps->levels[l + 1];
  const Arr<V> ac{P, l + 1};
  if (L.sameSet && L.bs >= 4) {  // residual and restriction in one pass
    if ((rc = blkApply<V>(ctx, ps, l, P, x, b, nullptr, 1, nullptr, ac.b(), ac.x()))) return rc;
  } else {
    if ((rc = applyT<V>(ctx, ps, P, l, x, b, r, 1))) return rc;
    MSBG_LAUNCH(ctx, (kRestrictSum<V>), gridCells(C.nCell), 256, 0, g, geomOf(C), (const V *)r, ac.b(), ac.x());
  }
  if ((rc = vcycleT<V>(ctx, ps, P, l + 1, ac.x(), ac.b(), ac.r()))) return rc;
  return smoothLevel<V>(ctx, ps, P, l, x, b, ps->postSweeps, true, kFirstCorr, (const V *)ac.x());
}

template <typename V>
static int dotDev(msbg_gpu_ctx *ctx, PoissonState *ps, const V *a, const V *b, int64_t n, double *dOut) {
  MSBG_LAUNCH(ctx, (kDotPartial<V>), (unsigned)ps->nPartial, kRedThreads, 0, a, b, n, ps->dPartial);
  MSBG_LAUNCH(ctx, kSumPartials, 1, kRedThreads, 0, ps->dPartial, ps->nPartial, dOut);
  return MSBG_GPU_OK;
}

static int fetchScal(msbg_gpu_ctx *ctx, PoissonState *ps, int i, int n) {
  MSBG_CUDA(ctx, cudaMemcpyAsync(ps->hScal + i, ps->dScal + i, (size_t)n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return MSBG_GPU_OK;
}

// ||b - A x||^2 and ||b||^2 with the residual in double-float arithmetic
static int trueResidual(msbg_gpu_ctx *ctx, PoissonState *ps, const float *x, const float *b, double *rr, double *bb) {
  int rc;
  if ((rc = blkApply<float>(ctx, ps, 0, ps->f32, x, b, nullptr, 2, ps->dScal + 8, nullptr, nullptr))) return rc;
  if ((rc = fetchScal(ctx, ps, 8, 2))) return rc;
  *rr = ps->hScal[8];
  *bb = ps->hScal[9];
  return MSBG_GPU_OK;
}

// Preconditioned CG on level 0 in storage type V.  r must hold b - A x on entry.
// Stops when the recurrence residual drops to relTol * r0norm (or maxIter); when
// checkTrue (FP32 only) the stop is confirmed on the FP64 true residual of (x, b).
// sc[0] rz, sc[1] pq, sc[2] rz_new, sc[3] rr.
template <typename V>
static int pcgT(msbg_gpu_ctx *ctx, PoissonState *ps, const PrecSet &P, V *x, const V *b, V *r, double stopNorm,
                int maxIter, bool checkTrue, double bnorm, int *itersOut, double *relOut) {
  const int64_t n = ps->levels[0].nCell;
  V *p = (V *)P.vp, *z = (V *)P.vz, *s = (V *)P.vs;
  double *sc = ps->dScal;
  int rc;
  if ((rc = vcycleT<V>(ctx, ps, P, 0, z, r, s))) return rc;
  MSBG_LAUNCH(ctx, (kCopy<V>), gridCells(n), 256, 0, z, p, n);
  if ((rc = blkDot<V>(ctx, ps, r, z, n, sc + 0))) return rc;
  double prev = 1e300, rel = 0.0;
  int growth = 0, it;
  for (it = 1; it <= maxIter; it++) {
    if ((rc = applyT<V>(ctx, ps, P, 0, p, nullptr, s, 0, sc + 1))) return rc;  // s = A p, sc[1] = p.s
    if ((rc = blkUpdateXR<V>(ctx, ps, sc, p, s, x, r, n, sc + 3))) return rc;
    if ((rc = fetchScal(ctx, ps, 3, 1))) return rc;
    const double rn = sqrt(ps->hScal[3]);
    rel = rn / bnorm;
    if (!isfinite(rn)) return fail(ctx, MSBG_GPU_ERR_DIVERGED, "residual is not finite at iteration %d", it);
    growth = rn > prev ? growth + 1 : 0;
    if (growth >= 8) return fail(ctx, MSBG_GPU_ERR_DIVERGED, "residual grew for 8 iterations (%g)", rel);
    prev = rn;
    if (rn <= stopNorm) {
      if (!checkTrue) break;
      double rr, bb;
      if ((rc = trueResidual(ctx, ps, (const float *)x, (const float *)b, &rr, &bb))) return rc;
      rel = sqrt(rr) / bnorm;
      if (sqrt(rr) <= stopNorm) break;
      if ((rc = applyT<V>(ctx, ps, P, 0, x, b, r, 1))) return rc;  // restart from the true residual
    }
    if ((rc = vcycleT<V>(ctx, ps, P, 0, z, r, s))) return rc;
    if ((rc = blkDot<V>(ctx, ps, r, z, n, sc + 2))) return rc;
    if ((rc = blkUpdateP<V>(ctx, ps, sc, z, p, n))) return rc;
    MSBG_CUDA(ctx, cudaMemcpyAsync(sc + 0, sc + 2, 8, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  if (it > maxIter) it = maxIter;
  *itersOut = it;
  *relOut = rel;
  return MSBG_GPU_OK;
}

// Device status after smoother launches: a bounded shared-memory wait that gave up
// sets bit 1 (the launch then wrote nothing).
static int checkStatus(msbg_gpu_ctx *ctx) {
  int st = 0;
  MSBG_CUDA(ctx, cudaMemcpyAsync(&st, ctx->dStatus, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (st) {
    MSBG_CUDA(ctx, cudaMemsetAsync(ctx->dStatus, 0, sizeof(int), ctx->stream));
    return fail(ctx, MSBG_GPU_ERR_TIMEOUT, "a bounded device wait timed out (status bits %d)", st);
  }
  return MSBG_GPU_OK;
}

// The level-0 FP32 work vectors r, p, z, s of the FP32 solves (4 x 4 B per cell).
int ensureF32Work(msbg_gpu_ctx *ctx, PoissonState *ps) {
  PrecSet &P = ps->f32;
  if (P.vr) return MSBG_GPU_OK;
  const int64_t n0 = ps->levels[0].nCell;
  int rc;
  for (void **q : {&P.vr, &P.vp, &P.vz, &P.vs}) if ((rc = allocT(ctx, (float **)q, n0))) return rc;
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_poisson_release_work(msbg_gpu_ctx *ctx) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  if (!ctx->poisson) return MSBG_GPU_OK;
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  for (PrecSet *P : {&ctx->poisson->f32, &ctx->poisson->f16}) {
    for (void **q : {&P->vr, &P->vp, &P->vz, &P->vs, &P->ve, &P->vb}) {
      if (*q) cudaFree(*q);
      *q = nullptr;
    }
  }
  // the FP16 set (coefficient copies, coarse-level vectors) is rebuilt on demand
  PrecSet &H = ctx->poisson->f16;
  for (auto *v : {&H.x, &H.b, &H.r, &H.cx, &H.cy, &H.cz, &H.d}) {
    for (void *q : *v) if (q) cudaFree(q);
    v->clear();
  }
  ctx->poisson->f16Valid = false;
  return MSBG_GPU_OK;
}

// level-0 operator and V-cycle for the batched solver (FP32)
int batchApply(msbg_gpu_ctx *ctx, const float *x, const float *b, float *y, int mode) {
  return applyT<float>(ctx, ctx->poisson, ctx->poisson->f32, 0, x, b, y, mode);
}
int batchVcycle(msbg_gpu_ctx *ctx, float *x, const float *b) {
  PoissonState *ps = ctx->poisson;
  int rc = ensureF32Work(ctx, ps);
  if (rc) return rc;
  return vcycleT<float>(ctx, ps, ps->f32, 0, x, b, (float *)ps->f32.vs);
}

int poissonEnsure(msbg_gpu_ctx *ctx) {
  if (ctx->poisson && ctx->poisson->layoutStamp == ctx->layoutStamp) return MSBG_GPU_OK;
  if (ctx->poisson) { poissonFree(ctx->poisson); ctx->poisson = nullptr; }
  PoissonState *ps = new PoissonState();
  ctx->poisson = ps;
  ps->layoutStamp = ctx->layoutStamp;
  ps->preSweeps = ctx->mgPre; ps->postSweeps = ctx->mgPost;
  ps->tileIters = ctx->mgTileIters; ps->coarsestIter = ctx->mgCoarsestIter;
  ps->relaxOmega = ctx->relaxOmega; ps->relaxBlockIter = ctx->relaxBlockIter;
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
  const int64_t n = ps->levels[0].nCell;
  float *src[4];
  const int ch[4] = {chanCx, chanCy, chanCz, chanDiag};
  for (int k = 0; k < 4; k++) if ((rc = chanF32(ctx, ch[k], &src[k]))) return rc;
  void *dst[4] = {ps->f32.cx[0], ps->f32.cy[0], ps->f32.cz[0], ps->f32.d[0]};
  for (int k = 0; k < 4; k++)
    MSBG_CUDA(ctx, cudaMemcpyAsync(dst[k], src[k], (size_t)n * 4, cudaMemcpyDeviceToDevice, ctx->stream));
  ps->coeffsValid = true;
  return buildCoarseOps(ctx, ps);
}

extern "C" int msbg_gpu_poisson_procedural_coefficients(msbg_gpu_ctx *ctx, uint32_t seed, int chanCx, int chanCy,
                                                       int chanCz, int chanDiag) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  int rc = needLayoutP(ctx);
  if (rc) return rc;
  PoissonState *ps = ctx->poisson;
  const MgLevel &L = ps->levels[0];
  float *dst[4] = {(float *)ps->f32.cx[0], (float *)ps->f32.cy[0], (float *)ps->f32.cz[0], (float *)ps->f32.d[0]};
  MSBG_LAUNCH(ctx, kProceduralCoeffs, gridCells(L.nCell), 256, 0, geomOf(L), seed, dst[0], dst[1], dst[2], dst[3]);
  ps->coeffsValid = true;
  const int ch[4] = {chanCx, chanCy, chanCz, chanDiag};
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

// Levels other than the value blocks' (levelMg 0) have no channel payload here.
static int needLevel0(msbg_gpu_ctx *ctx, int levelMg) {
  if (levelMg != 0)
    return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED, "levelMg %d: channels hold the value blocks (levelMg 0) only",
                levelMg);
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_multiply_laplacian(msbg_gpu_ctx *ctx, unsigned options, int levelMg, int chanX, int chanB,
                                           float kap, int chanDstY, double *pDotprod, const int32_t *dBlockList,
                                           int64_t nBlockList) {
  (void)kap;  // the reference's sparse-level path does not use it either (src/msbg3.cpp:1826-1911)
  if (!ctx || nBlockList < 0 || (nBlockList > 0 && !dBlockList)) return MSBG_GPU_ERR_ARG;
  const bool residual = (options & MSBG_GPU_OPT_CALC_RESIDUAL) != 0;
  if (options & ~(unsigned)MSBG_GPU_OPT_CALC_RESIDUAL)
    return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED, "multiply options 0x%x", options);
  if (residual && pDotprod)  // as the reference asserts (src/msbg3.cpp:1884)
    return fail(ctx, MSBG_GPU_ERR_ARG, "no dot product with OPT_CALC_RESIDUAL");
  int rc = needLevel0(ctx, levelMg);
  if (rc) return rc;
  if ((rc = needCoeffs(ctx))) return rc;
  float *x, *b = nullptr, *y;
  if ((rc = chanF32(ctx, chanX, &x)) || (rc = chanF32(ctx, chanDstY, &y))) return rc;
  if (residual && (rc = chanF32(ctx, chanB, &b))) return rc;
  PoissonState *ps = ctx->poisson;
  // the reference's operator form (kApplyList) over the list, or over every value block;
  // the multigrid keeps its own operator kernels
  if (!dBlockList) {
    dBlockList = ctx->dActive;
    nBlockList = ctx->nActive;
  }
  SlotLists L;
  if ((rc = listSlots(ctx, ps, dBlockList, nBlockList, &L))) return rc;
  if ((rc = applyList(ctx, ps, L, x, b, y, residual ? 1 : 0, pDotprod ? ps->dScal + 13 : nullptr))) return rc;
  if (pDotprod) {
    if ((rc = fetchScal(ctx, ps, 13, 1))) return rc;
    *pDotprod = ps->hScal[13];
  }
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_set_relax_params(msbg_gpu_ctx *ctx, float omega, int blockIter) {
  if (!ctx || !(omega > 0.0f && omega < 2.0f) || blockIter < 0 || blockIter > 64) return MSBG_GPU_ERR_ARG;
  ctx->relaxOmega = omega;
  ctx->relaxBlockIter = blockIter;
  if (ctx->poisson) {
    ctx->poisson->relaxOmega = omega;
    ctx->poisson->relaxBlockIter = blockIter;
  }
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_relax(msbg_gpu_ctx *ctx, int boundaryZoneOnly, int reverseOrder, int levelMg, int chanX,
                              int chanB, int chanTmp, int nIter, unsigned options, const int32_t *dBlockList,
                              int64_t nBlockList) {
  (void)chanTmp;  // in place, as the reference's red-black block order runs it (src/msbg3.cpp:2322-2336)
  if (!ctx || nIter < 0 || nBlockList < 0 || (nBlockList > 0 && !dBlockList)) return MSBG_GPU_ERR_ARG;
  if (boundaryZoneOnly)
    return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED, "boundary-zone relaxation (no boundary zones on this path)");
  if (options & ~(unsigned)MSBG_GPU_RELAX_TILES) return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED, "relax options 0x%x", options);
  int rc = needLevel0(ctx, levelMg);
  if (rc) return rc;
  if ((rc = needCoeffs(ctx))) return rc;
  PoissonState *ps = ctx->poisson;
  if ((options & MSBG_GPU_RELAX_TILES) && chanX >= 0 && chanX < kMaxChannels && chanB >= 0 &&
      chanB < kMaxChannels && ctx->ch[chanX].exists && ctx->ch[chanB].exists &&
      ctx->ch[chanX].storage == MSBG_GPU_F16 && ctx->ch[chanB].storage == MSBG_GPU_F16) {
    // FP16 channels: the mixed solve's FP16-storage smoother on the FP16 copies of
    // the coefficients
    if (dBlockList) return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED, "the tile smoother relaxes all value blocks");
    if ((rc = ensureHalf(ctx, ps))) return rc;
    if ((rc = smoothLevel<__half>(ctx, ps, ps->f16, 0, (__half *)ctx->ch[chanX].d, (const __half *)ctx->ch[chanB].d,
                                  nIter, reverseOrder != 0, kFirstNone, nullptr)))
      return rc;
    return checkStatus(ctx);
  }
  float *x, *b;
  if ((rc = chanF32(ctx, chanX, &x)) || (rc = chanF32(ctx, chanB, &b))) return rc;
  if (options & MSBG_GPU_RELAX_TILES) {
    if (dBlockList) return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED, "the tile smoother relaxes all value blocks");
    if ((rc = smoothLevel<float>(ctx, ps, ps->f32, 0, x, b, nIter, reverseOrder != 0, kFirstNone, nullptr)))
      return rc;
    return checkStatus(ctx);
  }
  SlotLists L;
  if (dBlockList && (rc = listSlots(ctx, ps, dBlockList, nBlockList, &L))) return rc;
  return relaxReference(ctx, ps, dBlockList ? &L : nullptr, x, b, nIter, reverseOrder ? 1 : 0, ps->relaxBlockIter,
                        ps->relaxOmega);
}

extern "C" int msbg_gpu_vcycle(msbg_gpu_ctx *ctx, int chanX, int chanB) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  int rc = needCoeffs(ctx);
  if (rc) return rc;
  float *x, *b;
  if ((rc = chanF32(ctx, chanX, &x)) || (rc = chanF32(ctx, chanB, &b))) return rc;
  PoissonState *ps = ctx->poisson;
  if ((rc = ensureF32Work(ctx, ps))) return rc;
  if ((rc = vcycleT<float>(ctx, ps, ps->f32, 0, x, b, (float *)ps->f32.vs))) return rc;
  return checkStatus(ctx);
}

extern "C" int msbg_gpu_dot(msbg_gpu_ctx *ctx, int chanA, int chanB, int levelMg, const int32_t *dBlockList,
                            int64_t nBlockList, double *out) {
  if (!ctx || !out || nBlockList < 0 || (nBlockList > 0 && !dBlockList)) return MSBG_GPU_ERR_ARG;
  int rc = needLevel0(ctx, levelMg);
  if (rc) return rc;
  if ((rc = needLayoutP(ctx))) return rc;
  float *a, *b;
  if ((rc = chanF32(ctx, chanA, &a)) || (rc = chanF32(ctx, chanB, &b))) return rc;
  PoissonState *ps = ctx->poisson;
  if (dBlockList) {
    SlotLists L;
    if ((rc = listSlots(ctx, ps, dBlockList, nBlockList, &L))) return rc;
    if ((rc = dotList(ctx, ps, L, a, b, ps->dScal + 12))) return rc;
  } else if ((rc = dotDev<float>(ctx, ps, a, b, ps->levels[0].nCell, ps->dScal + 12))) {
    return rc;
  }
  if ((rc = fetchScal(ctx, ps, 12, 1))) return rc;
  *out = ps->hScal[12];
  if (!isfinite(*out)) return fail(ctx, MSBG_GPU_ERR_NONFINITE, "dot product is not finite");  // src/msbg.cpp:4635
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_axpby(msbg_gpu_ctx *ctx, double a, int chanX, double b, int chanY, int levelMax, int levelMg,
                              const int32_t *dBlockList, int64_t nBlockList) {
  if (!ctx || nBlockList < 0 || (nBlockList > 0 && !dBlockList)) return MSBG_GPU_ERR_ARG;
  int rc = needLevel0(ctx, levelMg);
  if (rc) return rc;
  if ((rc = needLayoutP(ctx))) return rc;
  float *x, *y;
  if ((rc = chanF32(ctx, chanX, &x)) || (rc = chanF32(ctx, chanY, &y))) return rc;
  if (levelMax < 0) return MSBG_GPU_OK;  // value blocks are level 0: none is at or below levelMax
  if (dBlockList) {
    SlotLists L;
    if ((rc = listSlots(ctx, ctx->poisson, dBlockList, nBlockList, &L))) return rc;
    return axpbyList(ctx, L, a, x, b, y);
  }
  const int64_t n = ctx->poisson->levels[0].nCell;
  MSBG_LAUNCH(ctx, kAxpby, gridCells(n), 256, 0, a, x, b, y, n);
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_axpby_combined(msbg_gpu_ctx *ctx, double a, double b, int chanQ, int chanX, int chanP,
                                       const int32_t *dBlockList, int64_t nBlockList) {
  if (!ctx || nBlockList < 0 || (nBlockList > 0 && !dBlockList)) return MSBG_GPU_ERR_ARG;
  int rc = needLayoutP(ctx);
  if (rc) return rc;
  float *q, *x, *p;
  if ((rc = chanF32(ctx, chanQ, &q)) || (rc = chanF32(ctx, chanX, &x)) || (rc = chanF32(ctx, chanP, &p))) return rc;
  if (dBlockList) {
    SlotLists L;
    if ((rc = listSlots(ctx, ctx->poisson, dBlockList, nBlockList, &L))) return rc;
    return axpbyCombinedList(ctx, L, a, b, q, x, p);
  }
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
  if ((rc = ensureF32Work(ctx, ps))) return rc;
  float *r = (float *)ps->f32.vr;
  if ((rc = applyT<float>(ctx, ps, ps->f32, 0, x, b, r, 1))) return rc;
  double rr0, bb;
  if ((rc = trueResidual(ctx, ps, x, b, &rr0, &bb))) return rc;
  // a NaN or Inf in B or in the start X makes the first residual non-finite
  if (!isfinite(rr0) || !isfinite(bb))
    return fail(ctx, MSBG_GPU_ERR_DIVERGED, "initial residual is not finite (B or X holds NaN/Inf)");
  const double bnorm = sqrt(bb);
  double rel = bnorm > 0 ? sqrt(rr0) / bnorm : 0.0;
  int it = 0;
  if (bnorm > 0 && rel > tol) {
    if ((rc = pcgT<float>(ctx, ps, ps->f32, x, b, r, tol * bnorm, maxIter, true, bnorm, &it, &rel))) return rc;
  }
  if (itersOut) *itersOut = it;
  if (relResOut) *relResOut = rel;
  return checkStatus(ctx);
}

extern "C" int msbg_gpu_mgpcg_solve_mixed(msbg_gpu_ctx *ctx, int chanX, int chanB, double tol, int maxOuter,
                                          double innerTol, int maxInner, int *outerOut, int *innerTotalOut,
                                          double *relResOut) {
  if (!ctx || maxOuter < 0 || maxInner < 1 || !(tol > 0) || !(innerTol > 0 && innerTol < 1))
    return MSBG_GPU_ERR_ARG;
  int rc = needCoeffs(ctx);
  if (rc) return rc;
  float *x, *b;
  if ((rc = chanF32(ctx, chanX, &x)) || (rc = chanF32(ctx, chanB, &b))) return rc;
  PoissonState *ps = ctx->poisson;
  if ((rc = ensureHalf(ctx, ps))) return rc;
  const int64_t n = ps->levels[0].nCell;
  __half *rw = (__half *)ps->f16.vr, *e = (__half *)ps->f16.ve;
  // Each outer step: x += s e (the pending correction), then one pass forms the
  // residual b - A x in double-float arithmetic with the FP32 operator, its FP64
  // norm, and the FP16 right-hand side rw = (b - A x) / s' of the next correction
  // solve, s' being the predicted rms of that residual (recomputed exactly and
  // the pass redone when the prediction is off by more than 30x).
  float invScale = 1.0f, eScale = 0.0f;
  bool haveE = false;
  int outer = 0, innerTotal = 0;
  double rel = 0.0;
  for (;;) {
    if (haveE && (rc = blkAddScaled(ctx, ps, e, eScale, x, n))) return rc;
    haveE = false;
    if ((rc = blkApply<float>(ctx, ps, 0, ps->f32, x, b, nullptr, 2, ps->dScal + 8, nullptr, nullptr, rw, invScale)))
      return rc;
    if ((rc = fetchScal(ctx, ps, 8, 2))) return rc;
    const double rr = ps->hScal[8], bb = ps->hScal[9];
    if (!isfinite(rr)) return fail(ctx, MSBG_GPU_ERR_DIVERGED, "outer residual not finite");
    const double bnorm = sqrt(bb);
    rel = bnorm > 0 ? sqrt(rr) / bnorm : 0.0;
    if (bnorm == 0.0 || rel <= tol || outer >= maxOuter) break;
    const double rms = sqrt(rr / (double)n);
    const double ratio = rms * invScale;
    if (!(ratio > 1.0 / 30.0 && ratio < 30.0)) {  // rescale the FP16 right-hand side
      invScale = (float)(1.0 / rms);
      continue;
    }
    outer++;
    MSBG_LAUNCH(ctx, (kZero<__half>), gridCells(n), 256, 0, e, n);
    const double rhn = sqrt(rr) * invScale;
    int itIn = 0;
    double relIn = 0.0;
    if ((rc = pcgT<__half>(ctx, ps, ps->f16, e, rw, rw, innerTol * rhn, maxInner, false, rhn, &itIn, &relIn)))
      return rc;
    innerTotal += itIn;
    eScale = 1.0f / invScale;
    haveE = true;
    invScale = (float)(1.0 / (rms * fmax(relIn, 1e-3)));
  }
  if (outerOut) *outerOut = outer;
  if (innerTotalOut) *innerTotalOut = innerTotal;
  if (relResOut) *relResOut = rel;
  return checkStatus(ctx);
}

extern "C" int msbg_gpu_poisson_set_params(msbg_gpu_ctx *ctx, int preSweeps, int postSweeps, int tileIters,
                                           int coarsestIter) {
  if (!ctx || preSweeps < 0 || postSweeps < 0 || preSweeps > 16 || postSweeps > 16 || tileIters < 1 ||
      tileIters > 16 || coarsestIter < 0 || coarsestIter > 100000)
    return MSBG_GPU_ERR_ARG;
  ctx->mgPre = preSweeps; ctx->mgPost = postSweeps;
  ctx->mgTileIters = tileIters; ctx->mgCoarsestIter = coarsestIter;
  if (ctx->poisson) {
    PoissonState *ps = ctx->poisson;
    ps->preSweeps = preSweeps; ps->postSweeps = postSweeps;
    ps->tileIters = tileIters; ps->coarsestIter = coarsestIter;
  }
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_poisson_tuning(msbg_gpu_ctx *ctx, int enable, int32_t *hOut, int cap, int *nOut) {
  if (!ctx || enable < -1 || enable > 1 || cap < 0) return MSBG_GPU_ERR_ARG;
  int rc = needLayoutP(ctx);
  if (rc) return rc;
  PoissonState *ps = ctx->poisson;
  if (enable >= 0) ps->autotune = enable != 0;
  int n = 0;
  for (const auto &kv : ps->applyShape) {
    if (hOut && n < cap) {
      int32_t *e = hOut + 5 * n;
      e[0] = std::get<0>(kv.first);
      e[1] = std::get<1>(kv.first);
      e[2] = std::get<2>(kv.first);
      e[3] = kv.second >> 16;
      e[4] = kv.second & 0xffff;
    }
    n++;
  }
  if (nOut) *nOut = n;
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
