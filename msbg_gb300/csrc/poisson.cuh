// Internal declarations of the sparse Poisson solver (poisson.cu).
#pragma once

#include <cuda.h>
#include <cuda_fp16.h>

#include <map>
#include <tuple>
#include <vector>

#include "internal.cuh"

namespace msbg {

// storage types: FP32, or FP16 (mixed precision); arithmetic is FP32
__device__ __forceinline__ float ldv(const float *p) { return *p; }
__device__ __forceinline__ float ldv(const __half *p) { return __half2float(*p); }
__device__ __forceinline__ void stv(float *p, float v) { *p = v; }
__device__ __forceinline__ void stv(__half *p, float v) { *p = __float2half_rn(v); }

// ---------------------------------------------------------------------------------
// vector loads and stores of N consecutive values (N = 2, 4, 8, 16)
// ---------------------------------------------------------------------------------
__device__ __forceinline__ void unpackH2(uint32_t u, float &a, float &b) {
  __half2 h = *reinterpret_cast<__half2 *>(&u);
  const float2 f = __half22float2(h);
  a = f.x;
  b = f.y;
}
__device__ __forceinline__ uint32_t packH2(float a, float b) {
  __half2 h = __floats2half2_rn(a, b);
  return *reinterpret_cast<uint32_t *>(&h);
}

template <int N>
__device__ __forceinline__ void ldRow(const float *__restrict__ p, float *o) {
  if constexpr (N == 2) {
    const float2 v = *reinterpret_cast<const float2 *>(p);
    o[0] = v.x; o[1] = v.y;
  } else {
#pragma unroll
    for (int i = 0; i < N; i += 4) {
      const float4 v = *reinterpret_cast<const float4 *>(p + i);
      o[i] = v.x; o[i + 1] = v.y; o[i + 2] = v.z; o[i + 3] = v.w;
    }
  }
}
template <int N>
__device__ __forceinline__ void ldRow(const __half *__restrict__ p, float *o) {
  if constexpr (N == 2) {
    unpackH2(*reinterpret_cast<const uint32_t *>(p), o[0], o[1]);
  } else if constexpr (N == 4) {
    const uint2 v = *reinterpret_cast<const uint2 *>(p);
    unpackH2(v.x, o[0], o[1]);
    unpackH2(v.y, o[2], o[3]);
  } else {
#pragma unroll
    for (int i = 0; i < N; i += 8) {
      const uint4 v = *reinterpret_cast<const uint4 *>(p + i);
      unpackH2(v.x, o[i], o[i + 1]);
      unpackH2(v.y, o[i + 2], o[i + 3]);
      unpackH2(v.z, o[i + 4], o[i + 5]);
      unpackH2(v.w, o[i + 6], o[i + 7]);
    }
  }
}
template <int N>
__device__ __forceinline__ void stRow(float *__restrict__ p, const float *v) {
  if constexpr (N == 2) {
    *reinterpret_cast<float2 *>(p) = make_float2(v[0], v[1]);
  } else {
#pragma unroll
    for (int i = 0; i < N; i += 4)
      *reinterpret_cast<float4 *>(p + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
  }
}
template <int N>
__device__ __forceinline__ void stRow(__half *__restrict__ p, const float *v) {
  if constexpr (N == 2) {
    *reinterpret_cast<uint32_t *>(p) = packH2(v[0], v[1]);
  } else if constexpr (N == 4) {
    *reinterpret_cast<uint2 *>(p) = make_uint2(packH2(v[0], v[1]), packH2(v[2], v[3]));
  } else {
#pragma unroll
    for (int i = 0; i < N; i += 8)
      *reinterpret_cast<uint4 *>(p + i) = make_uint4(packH2(v[i], v[i + 1]), packH2(v[i + 2], v[i + 3]),
                                                     packH2(v[i + 4], v[i + 5]), packH2(v[i + 6], v[i + 7]));
  }
}

// N consecutive values of a row held in their storage form (FP16 stays packed two
// per register) and widened to FP32 where the arithmetic reads them; a kernel
// that keeps many rows live then needs half the registers for FP16 rows.
template <typename V, int N> struct RawRow;
template <int N> struct RawRow<float, N> {
  float v[N];
  __device__ __forceinline__ void ld(const float *__restrict__ p) { ldRow<N>(p, v); }
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int i = 0; i < N; i++) v[i] = 0.f;
  }
  __device__ __forceinline__ float operator[](int i) const { return v[i]; }
};
template <int N> struct RawRow<__half, N> {
  static_assert(N == 4 || N == 8, "rows of 4 or 8 FP16 values");
  uint32_t u[N / 2];
  __device__ __forceinline__ void ld(const __half *__restrict__ p) {
    if constexpr (N == 4) {
      const uint2 w = *reinterpret_cast<const uint2 *>(p);
      u[0] = w.x; u[1] = w.y;
    } else {
      const uint4 w = *reinterpret_cast<const uint4 *>(p);
      u[0] = w.x; u[1] = w.y; u[2] = w.z; u[3] = w.w;
    }
  }
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int i = 0; i < N / 2; i++) u[i] = 0u;
  }
  __device__ __forceinline__ float operator[](int i) const {
    const uint32_t w = u[i >> 1];
    const __half2 h = *reinterpret_cast<const __half2 *>(&w);
    return (i & 1) ? __high2float(h) : __low2float(h);
  }
};

constexpr int kRedThreads = 256;

// CTA-wide FP64 sum (blockDim.x == kRedThreads); every thread gets the total
__device__ __forceinline__ double blockSum(double v) {
  __shared__ double ws[kRedThreads / 32];
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) ws[w] = v;
  __syncthreads();
  v = 0.0;
#pragma unroll
  for (int i = 0; i < kRedThreads / 32; i++) v += ws[i];
  __syncthreads();
  return v;
}

// Levels that keep level 0's block set (block edge bs >= 4): per-block neighbour
// slots and the slot list ordered by block parity, passed by value to kernels.
struct BlkGeom {
  int bs, log2bs;
  int64_t nAct;
  const int32_t *nbr;      // [nAct][6]: slot of the -x,+x,-y,+y,-z,+z block or -1
  const int32_t *parList;  // [nAct]: slots with (bx+by+bz) even first, then odd
  int64_t nEven;
  const uint8_t *bpar;     // [nAct]: bit 0 bx&1, bit 1 by&1, bit 2 bz&1
};

// Geometry of one multigrid level, passed by value to kernels.
struct LvGeom {
  int bs, log2bs, nbx, nby, nbz;
  int64_t nCell;
  const int32_t *slot;    // [nbx*nby*nbz] slot or -1
  const int32_t *active;  // [nAct] block ids
};

struct MgLevel {  // geometry of one level (arrays live in PrecSet)
  int bs = 0, log2bs = 0, nbx = 0, nby = 0, nbz = 0;
  int64_t nAct = 0, nCell = 0;
  int32_t *slot = nullptr, *active = nullptr;
  bool ownsIndex = false;
  bool sameSet = false;  // shares level 0's block set (block edge halved)
  int tile = 0;          // tile smoother for this block edge (32, 16, 8), 0 = pointwise red-black
};

// Arrays of one storage precision: per level x, b, r (levels >= 1) and the
// coefficients (lower faces cx, cy, cz and diagonal d); level-0 work vectors.
struct PrecSet {
  std::vector<void *> x, b, r, cx, cy, cz, d;
  void *vr = nullptr, *vp = nullptr, *vz = nullptr, *vs = nullptr, *ve = nullptr, *vb = nullptr;
};

struct PoissonState {
  int64_t layoutStamp = -1;
  std::vector<MgLevel> levels;
  bool coeffsValid = false, f16Valid = false;
  PrecSet f32, f16;
  double *dPartial = nullptr;
  int nPartial = 0;
  double *dScal = nullptr, *hScal = nullptr;
  int preSweeps = 2, postSweeps = 2, tileIters = 3;
  int coarsestIter = 0;  // 0: exact solve with the dense inverse below
  int64_t coarsestCells = 512;
  float *dCoarseInv = nullptr;  // [n][n] inverse of the coarsest operator
  int64_t coarseInvN = 0;
  bool coarseInvValid = false;
  int32_t *dNbr = nullptr, *dParList = nullptr;  // block tables of level 0's set
  uint8_t *dBpar = nullptr;
  std::map<std::tuple<const void *, int, int>, CUtensorMap> tmaMaps;  // smoother tensor maps
  int64_t nEven = 0;
  int32_t *dListBuf = nullptr;   // block-list calls: slots, parity lists, counters
  double *dListPart = nullptr;   // per-listed-block partial sums
  int64_t listCap = 0;
  float relaxOmega = 6.0f / 7.0f;  // the reference's smoother constants (src/msbg.cpp:814-843)
  int relaxBlockIter = 5;
  // Launch shapes of the operator kernel picked by the autotuner: key (level, bytes per
  // value, mode), value cells-per-thread * 65536 + grid cap (CTAs).  Filled on the first
  // call of each key on a large enough level, by timing the candidates on that call's data.
  std::map<std::tuple<int, int, int>, int> applyShape;
  bool autotune = true;
};

void poissonFree(PoissonState *ps);
// Allocates the level-0 FP32 CG work vectors on first use.
int ensureF32Work(msbg_gpu_ctx *ctx, PoissonState *ps);

// A caller's block list (device block ids) as value-block slots (-1 for blocks without
// payload), and its value blocks split by block parity (bx+by+bz)&1 (poisson_ref.cu).
struct SlotLists {
  const int32_t *all = nullptr;
  int64_t nAll = 0;
  const int32_t *par[2] = {nullptr, nullptr};
  int64_t nPar[2] = {0, 0};
};
int listSlots(msbg_gpu_ctx *ctx, PoissonState *ps, const int32_t *dBids, int64_t n, SlotLists *out);
// y = A x (residual: b - A x) on the listed blocks; dDot (device) = sum of y x over them
int applyList(msbg_gpu_ctx *ctx, PoissonState *ps, const SlotLists &L, const float *x, const float *b, float *y,
              int residual, double *dDot);
int dotList(msbg_gpu_ctx *ctx, PoissonState *ps, const SlotLists &L, const float *a, const float *b, double *dOut);
int axpbyList(msbg_gpu_ctx *ctx, const SlotLists &L, double a, const float *x, double b, float *y);
int axpbyCombinedList(msbg_gpu_ctx *ctx, const SlotLists &L, double a, double b, const float *q, float *x, float *p);
// The reference's block smoother (relax / relaxBlockList), `passes` times, on the listed
// blocks (L) or all value blocks (L == nullptr).
int relaxReference(msbg_gpu_ctx *ctx, PoissonState *ps, const SlotLists *L, float *x, const float *b, int passes,
                   int reverse, int blockIter, float omega);
int poissonEnsure(msbg_gpu_ctx *ctx);
LvGeom geomOf(const MgLevel &L);
BlkGeom blkOf(const PoissonState *ps, const MgLevel &L);

// Block-structured kernels (poisson_blk.cu), levels with sameSet and bs >= 4.
// Neighbour table and parity list of the level-0 block set.
int blkBuildTables(msbg_gpu_ctx *ctx, PoissonState *ps);
// mode 0: y = A x (dotOut != null: partial sums of x.y to ps->dPartial, summed
// into *dotOut); mode 1: r = b - A x written to y, or, when bc != null,
// restricted (sum of 8 children) into the coarse b and the coarse x zeroed;
// mode 2: dotOut[0] = sum (b - A x)^2 with the residual formed in double-float
// arithmetic, dotOut[1] = sum b^2; rhOut != null: also rhOut = (b - A x) * rhScale
// in FP16.
template <typename V>
int blkApply(msbg_gpu_ctx *ctx, PoissonState *ps, size_t l, const PrecSet &P, const V *x, const V *b, V *y,
             int mode, double *dotOut, V *bc, V *xc, __half *rhOut = nullptr, float rhScale = 0.f);
// x += scale * e on level-0 vectors
int blkAddScaled(msbg_gpu_ctx *ctx, PoissonState *ps, const __half *e, float scale, float *x, int64_t n);
// CG vector operations on level-0 vectors (n a multiple of 4): dot into *dOut;
// x += alpha p, r -= alpha q with alpha = sc[0]/sc[1] and *rrOut = r.r; p = z + beta p
// with beta = sc[2]/sc[0].  Products are summed in FP32 per 4 values, then in FP64.
template <typename V>
int blkDot(msbg_gpu_ctx *ctx, PoissonState *ps, const V *a, const V *b, int64_t n, double *dOut);
template <typename V>
int blkUpdateXR(msbg_gpu_ctx *ctx, PoissonState *ps, const double *sc, const V *p, const V *q, V *x, V *r, int64_t n,
                double *rrOut);
template <typename V>
int blkUpdateP(msbg_gpu_ctx *ctx, PoissonState *ps, const double *sc, const V *z, V *p, int64_t n);
// One tile colour pass of the smoother; flags: kOwnZero, kHaloZero, kOwnCorr, kHaloCorr.
enum { kOwnZero = 1, kHaloZero = 2, kOwnCorr = 4, kHaloCorr = 8 };
template <typename V>
int blkSmoothColor(msbg_gpu_ctx *ctx, PoissonState *ps, size_t l, const PrecSet &P, V *x, const V *b,
                   const V *xc, int tileColor, int k, int reverse, int flags);

}  // namespace msbg
