// Restriction of a channel to the next coarser multigrid level:
// downsampleFloatChannelNew (src/msbg4.cpp:1035-1379) for the value blocks, the
// case levelMg = 1 of a layout whose value blocks are the level-0 blocks.
//
// A coarse cell v (block edge bs/2) is the sum over the fine cells 2v-1 .. 2v+2
// with weights (1,3,3,1)x(1,3,3,1)x(1,3,3,1)/512 (G3D_GetGausslikeKernel4x4x4,
// src/grid.c:30-70), or with simpleAverage the mean of its 8 children
// (OPT_SIMPLE_AVERAGE).  The fine halo is that of fillHaloBlock_ with
// OPT_BC_COARSE_LEVEL (src/halo.cpp:266-479, src/halo.h:288-300): a cell outside
// the domain takes the value at the clamped position, a cell in a block without
// payload the channel's empty value (0).
//
// Summation order, shared with the CPU restatement: per x offset i and row j an
// accumulator over the 4 planes, S[j][i] = fma(w, f, S[j][i]); then per i
// T[i] = ((S0 + S1) + S2) + S3 and the value (T0 + T1) + (T2 + T3).  This is the
// reference's four 4-wide accumulators (one per row, lanes = x offsets) and its
// horizontal add.
//
// One CTA per value block, one thread per coarse (x, y) column, marching the
// coarse planes in z.  Fine planes with their 1-cell x/y halo are staged as FP32
// in a 4-plane shared-memory ring ([bs+2][bs+2] each, rows coalesced along x), two
// new planes per coarse plane, so each fine plane is read from memory once; the
// loads of the next two planes are in flight while the current two are used.  Each
// thread carries its 16 partial sums of the coarse plane above in registers.
// Bytes: S per fine cell read (plus the halo), 4 per coarse cell written, i.e.
// HBM-bound at S + 1/2 bytes per fine cell.
#include "internal.cuh"

namespace msbg {

// Four consecutive values of a block row as floats (one 8- or 16-byte load; x is a
// multiple of 4), converted as Store<T>::load does.
template <typename T> __device__ __forceinline__ void ldQuad(const T *p, float v[4]);
template <> __device__ __forceinline__ void ldQuad<float>(const float *p, float v[4]) {
  const float4 q = *reinterpret_cast<const float4 *>(p);
  v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
}
template <> __device__ __forceinline__ void ldQuad<__half>(const __half *p, float v[4]) {
  const uint2 q = *reinterpret_cast<const uint2 *>(p);
  const float2 lo = __half22float2(*reinterpret_cast<const __half2 *>(&q.x));
  const float2 hi = __half22float2(*reinterpret_cast<const __half2 *>(&q.y));
  v[0] = lo.x; v[1] = lo.y; v[2] = hi.x; v[3] = hi.y;
}
template <> __device__ __forceinline__ void ldQuad<uint16_t>(const uint16_t *p, float v[4]) {
  const uint2 q = *reinterpret_cast<const uint2 *>(p);
  v[0] = __fmul_rn((float)(q.x & 0xffffu), kU16ToF);
  v[1] = __fmul_rn((float)(q.x >> 16), kU16ToF);
  v[2] = __fmul_rn((float)(q.y & 0xffffu), kU16ToF);
  v[3] = __fmul_rn((float)(q.y >> 16), kU16ToF);
}

template <int BS>
constexpr int dsThreads() {
  return (BS / 2) * (BS / 2) < 32 ? 32 : (BS / 2) * (BS / 2);
}

template <typename T, int BS, bool SIMPLE>
__global__ void __launch_bounds__(dsThreads<BS>(), 4) kDownsample(const T *__restrict__ pay,
                                                                 const int32_t *__restrict__ active,
                                                                 const int32_t *__restrict__ slot, int nbx,
                                                                 int nby, int nbz, float *__restrict__ out) {
  constexpr int NT = dsThreads<BS>(), CB = BS / 2, H = BS + 2, HH = H * H;
  constexpr int L = BS == 32 ? 5 : BS == 16 ? 4 : 3, m = BS - 1;
  __shared__ __align__(16) float st[4 * HH];  // fine plane p (-1..BS) in slot (p + 1) & 3
  __shared__ int nbs[27];
  const int t = blockIdx.x, tid = threadIdx.x;
  const int bid = active[t];
  const int bx = bid % nbx, by = (bid / nbx) % nby, bz = bid / (nbx * nby);
  if (tid < 27) {
    const int x = bx + tid % 3 - 1, y = by + (tid / 3) % 3 - 1, z = bz + tid / 9 - 1;
    int s = -1;  // outside the domain: never read (coordinates are clamped first)
    if (x >= 0 && y >= 0 && z >= 0 && x < nbx && y < nby && z < nbz)
      s = slot[(int64_t)z * nbx * nby + (int64_t)y * nbx + x];
    nbs[tid] = s;
  }
  __syncthreads();
  const int sx = nbx << L, sy = nby << L, sz = nbz << L;
  // Fine plane p (local z) with its x/y halo.  The plane's BS x BS interior comes
  // from one block (the own block, its z-neighbour, or the clamped own plane at the
  // domain face), 4 consecutive values per thread; the ring of 4 (BS + 1) halo cells
  // goes cell by cell.  fetch issues the loads into registers, put stores them into
  // the ring slot.
  constexpr int NI = BS * BS / 4, NR = 4 * (BS + 1), PR = (NR + NT - 1) / NT;
  static_assert(NI <= NT, "one interior quad per thread");
  struct Plane {
    float in[4], ring[PR];
  };
  auto fetch = [&](int p, Plane &v) {
    const int gz = min(max((bz << L) + p, 0), sz - 1);
    const int nz = ((gz >> L) - bz + 1) * 9 + 1;
    const int64_t zoff = (int64_t)(gz & m) << (2 * L);
    if (tid < NI) {
      const int sc = nbs[nz + 3];  // the block above / below (or the own block)
      v.in[0] = v.in[1] = v.in[2] = v.in[3] = 0.0f;
      if (sc >= 0) ldQuad<T>(pay + ((int64_t)sc << (3 * L)) + zoff + 4 * tid, v.in);
    }
#pragma unroll
    for (int k = 0; k < PR; k++) {
      const int e = tid + k * NT;
      v.ring[k] = 0.0f;  // the empty value
      if (e < NR) {
        // ring cell e: rows 0 and H-1 (e < 2H), then columns 0 and H-1 of rows 1..H-2
        int r, c;
        if (e < 2 * H) { r = e < H ? 0 : H - 1; c = e < H ? e : e - H; }
        else { const int f = e - 2 * H; r = 1 + (f >> 1); c = (f & 1) ? H - 1 : 0; }
        const int gy = min(max((by << L) + r - 1, 0), sy - 1), gx = min(max((bx << L) + c - 1, 0), sx - 1);
        const int sn = nbs[nz + ((gy >> L) - by + 1) * 3 + (gx >> L) - bx];
        if (sn >= 0) v.ring[k] = Store<T>::load(pay + ((int64_t)sn << (3 * L)) + zoff + ((gy & m) << L) + (gx & m));
      }
    }
  };
  auto put = [&](int p, const Plane &v) {
    float *dst = st + ((p + 1) & 3) * HH;
    if (tid < NI) {
      const int r = (4 * tid) >> L, c = (4 * tid) & m;
      float *q = dst + (r + 1) * H + c + 1;
#pragma unroll
      for (int k = 0; k < 4; k++) q[k] = v.in[k];
    }
#pragma unroll
    for (int k = 0; k < PR; k++) {
      const int e = tid + k * NT;
      if (e < NR) {
        int r, c;
        if (e < 2 * H) { r = e < H ? 0 : H - 1; c = e < H ? e : e - H; }
        else { const int f = e - 2 * H; r = 1 + (f >> 1); c = (f & 1) ? H - 1 : 0; }
        dst[r * H + c] = v.ring[k];
      }
    }
  };
  const bool own = tid < CB * CB;
  const int vx = tid & (CB - 1), vy = tid / CB;
  // exact weights k1[k] k1[j] k1[i] / 512 of (plane k, row j, column i)
  auto wgt = [](int k, int j, int i) {
    const float k1[4] = {1.f, 3.f, 3.f, 1.f};
    return k1[k] * k1[j] * k1[i] / 512.0f;
  };
  // row j (fine row 2vy-1+j, columns 2vx-1 .. 2vx+2) of fine plane p
  auto row = [&](int p, int j, float (&r)[4]) {
    const float *src = st + ((p + 1) & 3) * HH + (2 * vy + j) * H + 2 * vx;
    const float2 a = *reinterpret_cast<const float2 *>(src);
    const float2 b = *reinterpret_cast<const float2 *>(src + 2);
    r[0] = a.x; r[1] = a.y; r[2] = b.x; r[3] = b.y;
  };
  // Coarse plane vz reads fine planes 2vz-1 .. 2vz+2 (k = 0..3).  The accumulators of
  // plane vz over k = 0, 1 come from the previous pair of fine planes; the pair
  // (2vz+1, 2vz+2) completes them (k = 2, 3) and starts those of plane vz+1.  The
  // next pair's loads are in flight while a pair is used.
  float acc[4][4], part = 0.0f;  // acc[j][i] over k = 0, 1; part: the children sum in plane 2vz
  // Fine-plane pairs go through two register sets (A: pairs of even coarse planes, B:
  // odd), so the loads of the next two pairs are in flight while a pair is used.
  Plane va, vb, vc, vd;
  fetch(-1, va);
  fetch(0, vb);
  put(-1, va);
  put(0, vb);
  __syncthreads();
  fetch(1, va);
  fetch(2, vb);
  fetch(3, vc);
  fetch(4, vd);
  if (own) {
#pragma unroll
    for (int j = 0; j < 4; j++) {
      float r0[4], r1[4];
      row(-1, j, r0);
      row(0, j, r1);
#pragma unroll
      for (int i = 0; i < 4; i++)
        if (!SIMPLE) acc[j][i] = __fmaf_rn(wgt(1, j, i), r1[i], __fmaf_rn(wgt(0, j, i), r0[i], 0.0f));
      if (SIMPLE && j == 1) part = __fadd_rn(r1[1], r1[2]);
      if (SIMPLE && j == 2) part = __fadd_rn(__fadd_rn(part, r1[1]), r1[2]);
    }
  }
  // one coarse plane from the pair (p, q) of fine planes 2vz+1, 2vz+2
  auto step = [&](int vz, Plane &p, Plane &q) {
    // the pair's ring slots are not the previous pair's, whose last reads were
    // before the previous barrier
    put(2 * vz + 1, p);
    put(2 * vz + 2, q);
    __syncthreads();
    if (vz + 2 < CB) {  // the pair after next into the registers just emptied
      fetch(2 * vz + 5, p);
      fetch(2 * vz + 6, q);
    }
    if (!own) return;
    float T4[4], sum = part, npart = 0.0f;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      float r2[4], r3[4];
      row(2 * vz + 1, j, r2);
      row(2 * vz + 2, j, r3);
#pragma unroll
      for (int i = 0; i < 4; i++) {
        if (SIMPLE) break;
        const float S = __fmaf_rn(wgt(3, j, i), r3[i], __fmaf_rn(wgt(2, j, i), r2[i], acc[j][i]));
        T4[i] = j == 0 ? S : __fadd_rn(T4[i], S);
        acc[j][i] = __fmaf_rn(wgt(1, j, i), r3[i], __fmaf_rn(wgt(0, j, i), r2[i], 0.0f));
      }
      if (SIMPLE && (j == 1 || j == 2)) {  // children in plane 2vz+1 (this cell) and 2vz+2 (the next)
        sum = __fadd_rn(__fadd_rn(sum, r2[1]), r2[2]);
        npart = j == 1 ? __fadd_rn(r3[1], r3[2]) : __fadd_rn(__fadd_rn(npart, r3[1]), r3[2]);
      }
    }
    part = npart;
    const float val = SIMPLE ? __fmul_rn(sum, 0.125f)
                             : __fadd_rn(__fadd_rn(T4[0], T4[1]), __fadd_rn(T4[2], T4[3]));
    out[(int64_t)t * CB * CB * CB + ((int64_t)vz * CB + vy) * CB + vx] = val;
  };
  static_assert(CB % 2 == 0, "coarse planes in pairs");
#pragma unroll 1
  for (int vz = 0; vz < CB; vz += 2) {
    step(vz, va, vb);
    step(vz + 1, vc, vd);
  }
}

template <typename T, int BS>
static int downsampleT(msbg_gpu_ctx *ctx, const Channel &c, float *dDst, int simple) {
  if (simple)
    MSBG_LAUNCH(ctx, (kDownsample<T, BS, true>), (unsigned)ctx->nActive, dsThreads<BS>(), 0, (const T *)c.d,
                ctx->dActive, ctx->dSlot, ctx->nbx, ctx->nby, ctx->nbz, dDst);
  else
    MSBG_LAUNCH(ctx, (kDownsample<T, BS, false>), (unsigned)ctx->nActive, dsThreads<BS>(), 0, (const T *)c.d,
                ctx->dActive, ctx->dSlot, ctx->nbx, ctx->nby, ctx->nbz, dDst);
  return MSBG_GPU_OK;
}

template <typename T>
static int downsampleBs(msbg_gpu_ctx *ctx, const Channel &c, float *dDst, int simple) {
  switch (ctx->bsx) {
    case 8: return downsampleT<T, 8>(ctx, c, dDst, simple);
    case 16: return downsampleT<T, 16>(ctx, c, dDst, simple);
    default: return downsampleT<T, 32>(ctx, c, dDst, simple);
  }
}

}  // namespace msbg

using namespace msbg;

extern "C" int msbg_gpu_downsample_channel(msbg_gpu_ctx *ctx, int chSrc, float *dDst, int simpleAverage) {
  if (!ctx || !dDst) return MSBG_GPU_ERR_ARG;
  if (chSrc < 0 || chSrc >= kMaxChannels || !ctx->ch[chSrc].exists)
    return fail(ctx, MSBG_GPU_ERR_ARG, "channel %d does not exist", chSrc);
  if (!ctx->layoutValid) return fail(ctx, MSBG_GPU_ERR_STATE, "no block layout: call set_refinement_map");
  if (ctx->nActive == 0) return MSBG_GPU_OK;
  const Channel &c = ctx->ch[chSrc];
  switch (c.storage) {
    case MSBG_GPU_F32: return downsampleBs<float>(ctx, c, dDst, simpleAverage);
    case MSBG_GPU_F16: return downsampleBs<__half>(ctx, c, dDst, simpleAverage);
    case MSBG_GPU_U16: return downsampleBs<uint16_t>(ctx, c, dDst, simpleAverage);
    default:
      return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED, "downsample: FP64 channels are not supported");
  }
}
