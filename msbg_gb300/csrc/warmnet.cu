// Learned warm start for the Poisson solve: a 4-layer 3D convolutional network on
// the level-1 cells of the multigrid hierarchy (the value blocks with their edge
// halved), trained and run by the kernels below.
//
//   in  = [ b1 * invS,  d1 * invD - 1 ]     b1 = sum of the 8 level-0 children of b,
//                                           d1 = level-1 diagonal, invS = 1/rms(b1),
//                                           invD = 1/mean(d1)
//   h1 = relu(conv(in, W1) + c1),  h2 = relu(conv(h1, W2) + c2),
//   h3 = relu(conv(h2, W3) + c3),  o = conv(h3, W4) + c4       channels 2-16-16-16-2
//   x1 = S * (o0 + avg2(o1))        S = rms(b1); avg2: mean over the 8 level-1 cells
//                                   of a level-2 parent, on every one of them
//   x0 = x1 on each of the 8 level-0 children (the solve's starting point)
//
// conv: 3x3x3, zero outside the active cells, BF16 weights W[tap][cin][cout]
// (tap = (dx+1) + 3(dy+1) + 9(dz+1)), FP32 accumulation.  The forward convolutions
// run on the tensor cores and read their input activations rounded to BF16; the
// backward convolutions (CUDA cores) use the FP32 activations.
// Training loss (x* from the plain solver): "coarse" L = ||x1 - avg1(x*)||^2 /
// ||avg1(x*)||^2, avg1 = mean of the 8 level-0 children (the best coarse starting
// value), or "residual" L = ||A0 (x0 - x*)||^2 / ||b||^2.  Adam on FP32 master
// weights, re-rounded to BF16 after every step.
//
// Activations are channel-last [cell][C] FP32 arrays on level 1.  A cell finds its
// 26 neighbours inside its block by offset and across blocks through a per-block
// table of the 27 blocks around it.
#include <cuda_bf16.h>

#include <vector>

#include "internal.cuh"
#include "poisson.cuh"

namespace msbg {

constexpr int kWnLayers = 4;
constexpr int kWnCh[kWnLayers + 1] = {2, 16, 16, 16, 2};

struct WarmNetState {
  int64_t layoutStamp = -1;
  int64_t n1 = 0, n2 = 0;          // level-1 and level-2 cells
  int32_t *nbr27 = nullptr;        // [nAct][27]
  float *w32[kWnLayers] = {}, *bias[kWnLayers] = {};
  __nv_bfloat16 *wq[kWnLayers] = {};
  float *gw[kWnLayers] = {}, *gb[kWnLayers] = {};
  float *mw[kWnLayers] = {}, *vw[kWnLayers] = {}, *mb[kWnLayers] = {}, *vb[kWnLayers] = {};
  float *act[kWnLayers + 1] = {};  // activations; act[0] = raw inputs (b1, d1)
  float *gact[2] = {};             // ping-pong upstream gradients [n1][16]
  float *x1 = nullptr, *gx1 = nullptr;
  float *t0a = nullptr, *t0b = nullptr;  // level-0 temporaries
  double *dScal = nullptr, *hScal = nullptr;
  double *dPart = nullptr;
  int nPart = 0;
  int step = 0;
  int lossMode = 0;  // 0 coarse, 1 residual
  bool weightsSet = false;
};

int wnWeights(int l) { return 27 * kWnCh[l] * kWnCh[l + 1]; }

// ---------------------------------------------------------------------------------
// neighbours on level 1
// ---------------------------------------------------------------------------------
struct WnGeom {
  int bs, L;         // level-1 block edge
  int64_t nAct;
  const int32_t *nbr27;
};

// index of the level-1 cell at block-local (lx+dx, ly+dy, lz+dz) of slot s, or -1
__device__ __forceinline__ int64_t wnNbr(const WnGeom &g, int s, int lx, int ly, int lz, int dx, int dy, int dz) {
  int x = lx + dx, y = ly + dy, z = lz + dz;
  const int m = g.bs - 1;
  const int ox = x < 0 ? -1 : (x > m ? 1 : 0), oy = y < 0 ? -1 : (y > m ? 1 : 0), oz = z < 0 ? -1 : (z > m ? 1 : 0);
  if (ox | oy | oz) {
    s = g.nbr27[(int64_t)s * 27 + (ox + 1) + 3 * (oy + 1) + 9 * (oz + 1)];
    if (s < 0) return -1;
    x &= m; y &= m; z &= m;
  }
  return ((int64_t)s << (3 * g.L)) + ((int64_t)((z << g.L) + y) << g.L) + x;
}

__global__ void kNbr27(const int32_t *__restrict__ active, int64_t nAct, int nbx, int nby, int nbz,
                       const int32_t *__restrict__ slot, int32_t *__restrict__ nbr) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nAct * 27) return;
  const int64_t s = i / 27;
  const int k = (int)(i % 27);
  const int bid = active[s];
  const int bx = bid % nbx + k % 3 - 1, by = (bid / nbx) % nby + (k / 3) % 3 - 1, bz = bid / (nbx * nby) + k / 9 - 1;
  int v = -1;
  if (bx >= 0 && by >= 0 && bz >= 0 && bx < nbx && by < nby && bz < nbz)
    v = slot[((int64_t)bz * nby + by) * nbx + bx];
  nbr[i] = v;
}

// ---------------------------------------------------------------------------------
// inputs, output head, transfers
// ---------------------------------------------------------------------------------
// act0[c] = (b1, d1) and partial sums of b1^2, d1 (level-1 cell c; its 8 children
// in the level-0 block of the same slot)
__global__ void kWnInputs(const float *__restrict__ b0, const float *__restrict__ d1, int L1, int64_t n1,
                          float2 *__restrict__ act0, double *__restrict__ part) {
  double sb = 0.0, sd = 0.0;
  const int L0 = L1 + 1, m1 = (1 << L1) - 1;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n1; c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = c >> (3 * L1);
    const int v = (int)(c & ((1 << (3 * L1)) - 1));
    const int lx = v & m1, ly = (v >> L1) & m1, lz = v >> (2 * L1);
    const int64_t base = (s << (3 * L0)) + ((int64_t)((2 * lz) << L0) << L0) + ((int64_t)(2 * ly) << L0) + 2 * lx;
    float b = 0.f;
#pragma unroll
    for (int k = 0; k < 8; k++)
      b += b0[base + ((int64_t)((k >> 2) << L0) << L0) + ((int64_t)((k >> 1) & 1) << L0) + (k & 1)];
    const float d = d1[c];
    act0[c] = make_float2(b, d);
    sb += (double)b * b;
    sd += d;
  }
  sb = blockSum(sb);
  sd = blockSum(sd);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = sb;
    part[2 * blockIdx.x + 1] = sd;
  }
}
// sc[0] = S = rms(b1), sc[1] = invS, sc[2] = invD from the partial sums
__global__ void kWnScales(const double *__restrict__ part, int n, int64_t n1, double *__restrict__ sc) {
  double s0 = 0.0, s1 = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) { s0 += part[2 * i]; s1 += part[2 * i + 1]; }
  s0 = blockSum(s0);
  s1 = blockSum(s1);
  if (threadIdx.x == 0) {
    const double rms = n1 > 0 ? sqrt(s0 / (double)n1) : 0.0;
    const double S = rms > 0 ? rms : 1.0;
    const double mean = n1 > 0 ? s1 / (double)n1 : 1.0;
    sc[0] = S;
    sc[1] = 1.0 / S;
    sc[2] = mean != 0.0 ? 1.0 / mean : 1.0;
  }
}

// x1 = S (o0 + avg2(o1)); x0 on the 8 children.  One thread per level-2 parent.
__global__ void kWnHead(const float2 *__restrict__ o, const double *__restrict__ sc, int L1, int64_t n2,
                        float *__restrict__ x1, float *__restrict__ x0) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n2) return;
  const int L2 = L1 - 1, L0 = L1 + 1, m2 = (1 << L2) - 1;
  const int64_t s = p >> (3 * L2);
  const int v = (int)(p & ((1 << (3 * L2)) - 1));
  const int px = v & m2, py = (v >> L2) & m2, pz = v >> (2 * L2);
  int64_t ch[8];
  float o0[8], avg = 0.f;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const int lx = 2 * px + (k & 1), ly = 2 * py + ((k >> 1) & 1), lz = 2 * pz + (k >> 2);
    ch[k] = (s << (3 * L1)) + ((int64_t)((lz << L1) + ly) << L1) + lx;
    const float2 ov = o[ch[k]];
    o0[k] = ov.x;
    avg += ov.y;
  }
  avg *= 0.125f;
  const float S = (float)sc[0];
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const float xv = S * (o0[k] + avg);
    x1[ch[k]] = xv;
    if (x0) {
      const int lx = 2 * (2 * px + (k & 1)), ly = 2 * (2 * py + ((k >> 1) & 1)), lz = 2 * (2 * pz + (k >> 2));
      const int64_t b0 = (s << (3 * L0)) + ((int64_t)((lz << L0) + ly) << L0) + lx;
#pragma unroll
      for (int q = 0; q < 8; q++)
        x0[b0 + ((int64_t)((q >> 2) << L0) << L0) + ((int64_t)((q >> 1) & 1) << L0) + (q & 1)] = xv;
    }
  }
}

// Upstream gradient of the head: g(o0) = S gx1, g(o1) = S avg2(gx1).  gx1 = sum of
// the 8 level-0 children of g0.  One thread per level-2 parent; writes [n1][2].
__global__ void kWnHeadBack(const float *__restrict__ g0, const double *__restrict__ sc, int L1, int64_t n2,
                            float2 *__restrict__ go) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n2) return;
  const int L2 = L1 - 1, L0 = L1 + 1, m2 = (1 << L2) - 1;
  const int64_t s = p >> (3 * L2);
  const int v = (int)(p & ((1 << (3 * L2)) - 1));
  const int px = v & m2, py = (v >> L2) & m2, pz = v >> (2 * L2);
  float gx[8], avg = 0.f;
  int64_t ch[8];
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const int lx = 2 * px + (k & 1), ly = 2 * py + ((k >> 1) & 1), lz = 2 * pz + (k >> 2);
    ch[k] = (s << (3 * L1)) + ((int64_t)((lz << L1) + ly) << L1) + lx;
    const int64_t b0 = (s << (3 * L0)) + ((int64_t)(((2 * lz) << L0) + 2 * ly) << L0) + 2 * lx;
    float t = 0.f;
#pragma unroll
    for (int q = 0; q < 8; q++)
      t += g0[b0 + ((int64_t)((q >> 2) << L0) << L0) + ((int64_t)((q >> 1) & 1) << L0) + (q & 1)];
    gx[k] = t;
    avg += t;
  }
  avg *= 0.125f;
  const float S = (float)sc[0];
#pragma unroll
  for (int k = 0; k < 8; k++) go[ch[k]] = make_float2(S * gx[k], S * avg);
}

// Coarse loss: d = x1 - avg1(x*) stored in gx1; partial sums of d^2 and avg1^2.
__global__ void kWnCoarseDiff(const float *__restrict__ x1, const float *__restrict__ xs0, int L1, int64_t n1,
                              float *__restrict__ dOut, double *__restrict__ part) {
  double sd = 0.0, sx = 0.0;
  const int L0 = L1 + 1, m1 = (1 << L1) - 1;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n1; c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = c >> (3 * L1);
    const int v = (int)(c & ((1 << (3 * L1)) - 1));
    const int lx = v & m1, ly = (v >> L1) & m1, lz = v >> (2 * L1);
    const int64_t base = (s << (3 * L0)) + ((int64_t)((2 * lz) << L0) << L0) + ((int64_t)(2 * ly) << L0) + 2 * lx;
    float t = 0.f;
#pragma unroll
    for (int k = 0; k < 8; k++)
      t += xs0[base + ((int64_t)((k >> 2) << L0) << L0) + ((int64_t)((k >> 1) & 1) << L0) + (k & 1)];
    const float xbar = 0.125f * t;
    const float d = x1[c] - xbar;
    dOut[c] = d;
    sd += (double)d * d;
    sx += (double)xbar * xbar;
  }
  sd = blockSum(sd);
  sx = blockSum(sx);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = sd;
    part[2 * blockIdx.x + 1] = sx;
  }
}
__global__ void kSum2(const double *__restrict__ part, int n, double *__restrict__ out) {
  double s0 = 0.0, s1 = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) { s0 += part[2 * i]; s1 += part[2 * i + 1]; }
  s0 = blockSum(s0);
  s1 = blockSum(s1);
  if (threadIdx.x == 0) { out[0] = s0; out[1] = s1; }
}
// head backward from a level-1 gradient gx1 = k * d / den (den = sc[5]):
// g(o0) = S gx1, g(o1) = S avg2(gx1).  One thread per level-2 parent.
__global__ void kWnHeadBack1(const float *__restrict__ d, const double *__restrict__ sc, float k, int L1, int64_t n2,
                             float2 *__restrict__ go) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n2) return;
  const int L2 = L1 - 1, m2 = (1 << L2) - 1;
  const int64_t s = p >> (3 * L2);
  const int v = (int)(p & ((1 << (3 * L2)) - 1));
  const int px = v & m2, py = (v >> L2) & m2, pz = v >> (2 * L2);
  const float f = sc[5] > 0 ? (float)(k / sc[5]) : 0.f;
  float gx[8], avg = 0.f;
  int64_t ch[8];
#pragma unroll
  for (int q = 0; q < 8; q++) {
    const int lx = 2 * px + (q & 1), ly = 2 * py + ((q >> 1) & 1), lz = 2 * pz + (q >> 2);
    ch[q] = (s << (3 * L1)) + ((int64_t)((lz << L1) + ly) << L1) + lx;
    gx[q] = f * d[ch[q]];
    avg += gx[q];
  }
  avg *= 0.125f;
  const float S = (float)sc[0];
#pragma unroll
  for (int q = 0; q < 8; q++) go[ch[q]] = make_float2(S * gx[q], S * avg);
}

// ---------------------------------------------------------------------------------
// forward convolution on the tensor cores (tcgen05, BF16 x BF16 -> FP32 in TMEM)
// ---------------------------------------------------------------------------------
// Implicit GEMM per tile of 128 consecutive level-1 cells: D[128][16] = sum over the
// 27 taps of A_t[128][16] * B_t[16][16]^T, where row r of A_t holds the input channels
// of the cell at tap t from cell r (BF16, zero where the neighbour is absent; channels
// beyond CIN are zero) and B_t[o][i] = W[t][i][o] (BF16; outputs beyond COUT are zero).
// One thread per cell gathers its rows; thread 0 issues one tcgen05.mma per tap
// (M = 128, N = 16, K = 16) into a 16-column TMEM accumulator and commits it to the
// mbarrier of the A buffer, which frees the buffer for tap t + 4.  The epilogue reads
// row r of D with tcgen05.ld (warp w owns TMEM lanes 32w..32w+31), adds the bias and
// applies the ReLU.  Operands use the K-major, no-swizzle layout of 8-row x 16-byte
// core matrices: K-adjacent core matrices 128 B apart, row groups 256 B apart.
namespace tc {
__device__ __forceinline__ uint32_t sAddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint64_t desc(const void *base) {
  uint64_t d = (uint64_t)((sAddr(base) >> 4) & 0x3FFF);
  d |= (uint64_t)(128 >> 4) << 16;  // leading byte offset: K-adjacent core matrices
  d |= (uint64_t)(256 >> 4) << 32;  // stride byte offset: the next 8 rows
  d |= (uint64_t)1 << 46;           // descriptor version; base offset 0, no swizzle
  return d;
}
// kind::f16 instruction descriptor: FP32 accumulator, BF16 A and B, both K-major, N, M
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((16u >> 3) << 17) | ((128u >> 4) << 24);
__device__ __forceinline__ bool tryWait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
               : "=r"(ok)
               : "r"(sAddr(bar)), "r"(parity)
               : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool waitBounded(uint64_t *bar, uint32_t parity) {
  for (int it = 0; it < (1 << 22); it++)
    if (tryWait(bar, parity)) return true;
  return false;
}
// offset (elements) of row r, channels 8kb..8kb+7 in a 16-wide K-major operand
__device__ __forceinline__ int coreOff(int r, int kb) { return (r >> 3) * 128 + kb * 64 + (r & 7) * 8; }
__device__ __forceinline__ uint32_t pack2(float a, float b) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t *>(&h);
}
}  // namespace tc

constexpr int kTcThreads = 128, kTcBuf = 4;

template <int CIN, int COUT, bool RELU, bool NORM>
__global__ void __launch_bounds__(kTcThreads) kConvTc(WnGeom g, const float *__restrict__ x,
                                                    const __nv_bfloat16 *__restrict__ w,
                                                    const float *__restrict__ bias, const double *__restrict__ sc,
                                                    float *__restrict__ y, int *__restrict__ status) {
  static_assert(CIN <= 16 && COUT <= 16 && (CIN == 2 || CIN == 16), "padded to K = N = 16");
  __shared__ __align__(1024) __nv_bfloat16 sA[kTcBuf][128 * 16];
  __shared__ __align__(1024) __nv_bfloat16 sB[27][16 * 16];
  __shared__ float sBias[16];
  __shared__ __align__(8) uint64_t bar[kTcBuf];
  __shared__ uint32_t tmemSlot;
  const int tid = threadIdx.x, warp = tid >> 5;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 32;" ::"r"(tc::sAddr(&tmemSlot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid < kTcBuf) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc::sAddr(&bar[tid])));
  if (tid == 0) asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  for (int i = tid; i < 27 * 16 * 16; i += kTcThreads) {  // B_t[o][i] = W[t][i][o], zero padded
    const int t = i / 256, o = (i / 16) % 16, c = i % 16;
    const __nv_bfloat16 v = (o < COUT && c < CIN) ? w[(t * CIN + c) * COUT + o] : __float2bfloat16(0.0f);
    sB[t][tc::coreOff(o, c >> 3) + (c & 7)] = v;
  }
  if (tid < 16) sBias[tid] = tid < COUT ? bias[tid] : 0.0f;
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmemSlot;
  const float s0 = NORM ? (float)sc[1] : 1.f, s1 = NORM ? (float)sc[2] : 1.f;
  const int64_t n = g.nAct << (3 * g.L);
  const int64_t nTiles = (n + 127) >> 7;
  const int m = g.bs - 1;
  uint32_t q = 0;  // MMAs issued by this CTA: buffer q % kTcBuf, use q / kTcBuf
  bool ok = true;

  // the 16 (padded) input channels of cell c's neighbour at tap t, as 8 BF16 pairs
  auto gather = [&](int64_t c, int t, uint32_t (&v)[8]) {
#pragma unroll
    for (int k = 0; k < 8; k++) v[k] = 0u;
    if (c >= n) return;
    const int s = (int)(c >> (3 * g.L));
    const int vv = (int)(c & ((1 << (3 * g.L)) - 1));
    const int64_t j = wnNbr(g, s, vv & m, (vv >> g.L) & m, vv >> (2 * g.L), t % 3 - 1, (t / 3) % 3 - 1, t / 9 - 1);
    if (j < 0) return;
    if constexpr (CIN == 2) {
      const float2 a = reinterpret_cast<const float2 *>(x)[j];
      v[0] = tc::pack2(NORM ? a.x * s0 : a.x, NORM ? a.y * s1 - 1.0f : a.y);
    } else {
#pragma unroll
      for (int k = 0; k < 4; k++) {
        const float4 a = *reinterpret_cast<const float4 *>(x + j * 16 + 4 * k);
        v[2 * k] = tc::pack2(a.x, a.y);
        v[2 * k + 1] = tc::pack2(a.z, a.w);
      }
    }
  };

  for (int64_t tile = blockIdx.x; tile < nTiles && ok; tile += gridDim.x) {
    const int64_t c = (tile << 7) + tid;
    uint32_t cur[8], nxt[8];
    gather(c, 0, cur);
    for (int t = 0; t < 27; t++) {
      if (t + 1 < 27) gather(c, t + 1, nxt);  // in flight while this tap's row is stored
      const int b = (int)(q % kTcBuf);
      const uint32_t use = q / kTcBuf;
      bool okw = true;
      if (use > 0) okw = tc::waitBounded(&bar[b], (use - 1) & 1u);  // the MMA that last read buffer b
      __nv_bfloat16 *A = sA[b];
      *reinterpret_cast<uint4 *>(A + tc::coreOff(tid, 0)) = make_uint4(cur[0], cur[1], cur[2], cur[3]);
      *reinterpret_cast<uint4 *>(A + tc::coreOff(tid, 1)) = make_uint4(cur[4], cur[5], cur[6], cur[7]);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;");
      ok = __syncthreads_and(okw);
      if (!ok) break;
      if (tid == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint64_t ad = tc::desc(A), bd = tc::desc(sB[t]);
        asm volatile(
            "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(tc::kIdesc), "r"((uint32_t)(t > 0)));
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         tc::sAddr(&bar[b]))
                     : "memory");
      }
      q++;
#pragma unroll
      for (int k = 0; k < 8; k++) cur[k] = nxt[k];
    }
    if (!ok) break;
    // the tile's last MMA (and with it all earlier ones) has completed
    const uint32_t last = q - 1;
    ok = __syncthreads_and(tc::waitBounded(&bar[last % kTcBuf], (last / kTcBuf) & 1u));
    if (!ok) break;
    asm volatile("tcgen05.fence::after_thread_sync;");
    uint32_t d[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(d[0]), "=r"(d[1]), "=r"(d[2]), "=r"(d[3]), "=r"(d[4]), "=r"(d[5]), "=r"(d[6]), "=r"(d[7]),
          "=r"(d[8]), "=r"(d[9]), "=r"(d[10]), "=r"(d[11]), "=r"(d[12]), "=r"(d[13]), "=r"(d[14]), "=r"(d[15])
        : "r"(tmem + ((uint32_t)(warp * 32) << 16)));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    if (c < n) {
      float o[16];
#pragma unroll
      for (int k = 0; k < 16; k++) {
        const float v = __uint_as_float(d[k]) + sBias[k];
        o[k] = RELU ? fmaxf(v, 0.0f) : v;
      }
      if constexpr (COUT == 16) {
#pragma unroll
        for (int k = 0; k < 4; k++)
          reinterpret_cast<float4 *>(y + c * 16)[k] = make_float4(o[4 * k], o[4 * k + 1], o[4 * k + 2], o[4 * k + 3]);
      } else {
#pragma unroll
        for (int k = 0; k < COUT; k++) y[c * COUT + k] = o[k];
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
  }
  if (!ok && tid == 0) atomicOr(status, 4);
  // every committed MMA has been waited for on the normal path; after a timeout,
  // wait (bounded) for the last one before the accumulator is freed
  if (!ok && tid == 0 && q > 0) tc::waitBounded(&bar[(q - 1) % kTcBuf], ((q - 1) / kTcBuf) & 1u);
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 32;" ::"r"(tmem));
  }
}

// The same convolution with the gather done by the tensor core's operand
// addressing.  A tile's input neighbourhood is staged once, as BF16, in copies
// shifted so that every tap's A operand is a run of consecutive 16-byte rows of one
// copy: a shifted descriptor (8-row core matrices 128 B apart, the two channel halves
// a copy-half apart), and the 27 MMAs issue back to back.
//  - Level-1 blocks of edge 16: a tile is 8 rows of 16 cells (y0..y0+7 of plane lz).
//    The neighbourhood (planes lz-1..lz+1, rows y0-1..y0+8, columns -1..16) is kept in
//    three copies shifted by dx = -1, 0, +1 (copy dx holds at column x the input of
//    column x + dx), rows of 16 cells; row r = 16 y + x of tap (dx, dy, dz) is row
//    ((dz+1) 10 + dy+1) 16 + r of copy dx.
//  - Level-1 blocks of edge 8: a tile is two planes lz0, lz0+1 of 8 x 8 cells.  The
//    neighbourhood (planes lz0-1..lz0+2, rows and columns -1..8) is kept in nine copies
//    shifted by (dx, dy), planes of 8 x 8; row r = 64 z + 8 y + x of tap (dx, dy, dz)
//    is row 64 (dz+1) + r of copy (dx, dy).
template <int BS1> struct StGeom;
template <> struct StGeom<16> {
  static constexpr int L = 4, NX = 18, NY = 10, NZ = 3, NCOPY = 3, ROWS = 3 * 10 * 16, TPB_LOG = 5;
};
template <> struct StGeom<8> {
  static constexpr int L = 3, NX = 10, NY = 10, NZ = 4, NCOPY = 9, ROWS = 4 * 64, TPB_LOG = 2;
};
template <int BS1>
constexpr size_t stSmemBytes() {
  return (size_t)(StGeom<BS1>::NCOPY * 2 * StGeom<BS1>::ROWS * 8 + 27 * 256) * sizeof(__nv_bfloat16);
}

template <int BS1, int CIN, int COUT, bool RELU, bool NORM>
__global__ void __launch_bounds__(kTcThreads, BS1 == 16 ? 3 : 2) kConvTcStaged(WnGeom g, const float *__restrict__ x,
                                                             const __nv_bfloat16 *__restrict__ w,
                                                             const float *__restrict__ bias,
                                                             const double *__restrict__ sc, float *__restrict__ y,
                                                             int *__restrict__ status) {
  using SG = StGeom<BS1>;
  constexpr int L = SG::L, m = BS1 - 1, kStHalf = SG::ROWS * 8, kStCopy = 2 * kStHalf;
  static_assert(CIN <= 16 && COUT <= 16 && (CIN == 2 || CIN == 16), "padded to K = N = 16");
  extern __shared__ __align__(1024) unsigned char wnSmem[];
  __nv_bfloat16 *sX = reinterpret_cast<__nv_bfloat16 *>(wnSmem);   // [copies][2 halves][ROWS][8]
  __nv_bfloat16 *sB = sX + SG::NCOPY * kStCopy;                      // [27][16 x 16] core-matrix layout
  __shared__ float sBias[16];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmemSlot;
  const int tid = threadIdx.x, warp = tid >> 5;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 32;" ::"r"(tc::sAddr(&tmemSlot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc::sAddr(&bar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int i = tid; i < 27 * 16 * 16; i += kTcThreads) {  // B_t[o][i] = W[t][i][o], zero padded
    const int t = i / 256, o = (i / 16) % 16, c = i % 16;
    const __nv_bfloat16 v = (o < COUT && c < CIN) ? w[(t * CIN + c) * COUT + o] : __float2bfloat16(0.0f);
    sB[t * 256 + tc::coreOff(o, c >> 3) + (c & 7)] = v;
  }
  if (tid < 16) sBias[tid] = tid < COUT ? bias[tid] : 0.0f;
  const float s0 = NORM ? (float)sc[1] : 1.f, s1 = NORM ? (float)sc[2] : 1.f;
  const int64_t n = g.nAct << (3 * L);
  const int64_t nTiles = n >> 7;
  uint32_t phase = 0;
  bool ok = true;
  // A tile's neighbourhood: 3 planes x 10 rows x 18 columns of input cells, PER per
  // thread.  load issues all of a thread's global loads (into raw); stage converts
  // them to BF16 and writes the three shifted copies.
  constexpr int NE = SG::NX * SG::NY * SG::NZ, PER = (NE + kTcThreads - 1) / kTcThreads;
  // origin of tile's neighbourhood cell (0, 0, 0) in block coordinates is (-1, oy0-1, oz0-1)
  auto origin = [](int64_t tile, int &oy0, int &oz0) {
    const int sub = (int)(tile & ((1 << SG::TPB_LOG) - 1));
    if constexpr (BS1 == 16) { oy0 = (sub & 1) * 8; oz0 = sub >> 1; }
    else { oy0 = 0; oz0 = 2 * sub; }
  };
  float4 raw[PER][CIN == 2 ? 1 : 4];
  bool have[PER];
  auto load = [&](int64_t tile) {
    const int s = (int)(tile >> SG::TPB_LOG);
    int oy0, oz0;
    origin(tile, oy0, oz0);
    const int32_t *nbg = g.nbr27 + (int64_t)s * 27;
#pragma unroll
    for (int k = 0; k < PER; k++) {
      const int e = tid + k * kTcThreads;
      have[k] = false;
      if (e < NE) {
        const int xi = e % SG::NX, yi = (e / SG::NX) % SG::NY, zi = e / (SG::NX * SG::NY);
        const int cx = xi - 1, cy = oy0 + yi - 1, cz = oz0 + zi - 1;
        const int ox = cx < 0 ? -1 : (cx > m ? 1 : 0), oy = cy < 0 ? -1 : (cy > m ? 1 : 0),
                  oz = cz < 0 ? -1 : (cz > m ? 1 : 0);
        const int sn = (ox | oy | oz) ? nbg[(ox + 1) + 3 * (oy + 1) + 9 * (oz + 1)] : s;
        if (sn >= 0) {
          have[k] = true;
          const int64_t j = ((int64_t)sn << (3 * L)) + ((((cz & m) << L) + (cy & m)) << L) + (cx & m);
          if constexpr (CIN == 2) {
            const float2 v = reinterpret_cast<const float2 *>(x)[j];
            raw[k][0] = make_float4(v.x, v.y, 0.f, 0.f);
          } else {
#pragma unroll
            for (int q = 0; q < 4; q++) raw[k][q] = *reinterpret_cast<const float4 *>(x + j * 16 + 4 * q);
          }
        }
      }
    }
  };
  auto stage = [&]() {
#pragma unroll
    for (int k = 0; k < PER; k++) {
      const int e = tid + k * kTcThreads;
      if (e >= NE) continue;
      const int xi = e % SG::NX, yi = (e / SG::NX) % SG::NY, zi = e / (SG::NX * SG::NY);
      const int cx = xi - 1;
      uint32_t v[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
      if (have[k]) {
        if constexpr (CIN == 2) {
          const float4 a = raw[k][0];
          v[0] = tc::pack2(NORM ? a.x * s0 : a.x, NORM ? a.y * s1 - 1.0f : a.y);
        } else {
#pragma unroll
          for (int q = 0; q < 4; q++) {
            v[2 * q] = tc::pack2(raw[k][q].x, raw[k][q].y);
            v[2 * q + 1] = tc::pack2(raw[k][q].z, raw[k][q].w);
          }
        }
      }
      auto put = [&](int copy, int row) {
        __nv_bfloat16 *dst = sX + copy * kStCopy + row * 8;
        *reinterpret_cast<uint4 *>(dst) = make_uint4(v[0], v[1], v[2], v[3]);
        *reinterpret_cast<uint4 *>(dst + kStHalf) = make_uint4(v[4], v[5], v[6], v[7]);
      };
      if constexpr (BS1 == 16) {
#pragma unroll
        for (int d = 0; d < 3; d++) {  // copy of shift dx = d - 1 holds this cell at column cx - dx
          const int col = cx - (d - 1);
          if (col >= 0 && col <= 15) put(d, (zi * SG::NY + yi) * 16 + col);
        }
      } else {
        const int cy = yi - 1;
#pragma unroll
        for (int dy = -1; dy <= 1; dy++) {
#pragma unroll
          for (int dx = -1; dx <= 1; dx++) {  // copy (dx, dy) holds this cell at (cx - dx, cy - dy)
            const int xc = cx - dx, yc = cy - dy;
            if (xc >= 0 && xc <= 7 && yc >= 0 && yc <= 7) put((dy + 1) * 3 + dx + 1, zi * 64 + yc * 8 + xc);
          }
        }
      }
    }
  };
  // descriptors of the first tap's operands; tap t adds its byte offset (>> 4) to the
  // start-address field (all addresses stay below 256 KB)
  uint64_t adBase = (uint64_t)((tc::sAddr(sX) >> 4) & 0x3FFF);
  adBase |= (uint64_t)((kStHalf * 2) >> 4) << 16;  // leading byte offset: the other channel half
  adBase |= (uint64_t)(128 >> 4) << 32;            // stride byte offset: the next 8 rows
  adBase |= (uint64_t)1 << 46;
  const uint64_t bdBase = tc::desc(sB);

  int64_t tile = blockIdx.x;
  if (tile < nTiles) load(tile);
  for (; tile < nTiles && ok; tile += gridDim.x) {
    // the previous tile's MMAs have completed (waited below), so its staged copies
    // may be overwritten
    stage();
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    const uint32_t tmem = tmemSlot;
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
      for (int t = 0; t < 27; t++) {
        const int dx = t % 3 - 1, dy = (t / 3) % 3 - 1, dz = t / 9 - 1;
        const uint32_t aOff =
            BS1 == 16 ? ((dx + 1) * kStCopy + (((dz + 1) * SG::NY + dy + 1) * 16) * 8) * 2   // bytes
                      : (((dy + 1) * 3 + dx + 1) * kStCopy + ((dz + 1) * 64) * 8) * 2;
        const uint64_t ad = adBase + (aOff >> 4), bd = bdBase + ((uint32_t)(t * 256 * 2) >> 4);
        asm volatile(
            "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(tc::kIdesc), "r"((uint32_t)(t > 0)));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       tc::sAddr(&bar))
                   : "memory");
    }
    // the next tile's loads fly while the tensor core works on this one
    if (tile + gridDim.x < nTiles) load(tile + gridDim.x);
    ok = __syncthreads_and(tc::waitBounded(&bar, phase));
    phase ^= 1u;
    if (!ok) break;
    asm volatile("tcgen05.fence::after_thread_sync;");
    uint32_t d[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(d[0]), "=r"(d[1]), "=r"(d[2]), "=r"(d[3]), "=r"(d[4]), "=r"(d[5]), "=r"(d[6]), "=r"(d[7]),
          "=r"(d[8]), "=r"(d[9]), "=r"(d[10]), "=r"(d[11]), "=r"(d[12]), "=r"(d[13]), "=r"(d[14]), "=r"(d[15])
        : "r"(tmem + ((uint32_t)(warp * 32) << 16)));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    const int64_t c = (tile << 7) + tid;
    float o[16];
#pragma unroll
    for (int k = 0; k < 16; k++) {
      const float v = __uint_as_float(d[k]) + sBias[k];
      o[k] = RELU ? fmaxf(v, 0.0f) : v;
    }
    if constexpr (COUT == 16) {
#pragma unroll
      for (int k = 0; k < 4; k++)
        reinterpret_cast<float4 *>(y + c * 16)[k] = make_float4(o[4 * k], o[4 * k + 1], o[4 * k + 2], o[4 * k + 3]);
    } else {
#pragma unroll
      for (int k = 0; k < COUT; k++) y[c * COUT + k] = o[k];
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
  }
  if (!ok && tid == 0) atomicOr(status, 4);
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 32;" ::"r"(tmemSlot));
  }
}


// ---------------------------------------------------------------------------------
// backward convolutions (CUDA cores; FP32)
// ---------------------------------------------------------------------------------
// gx[c][i] = sum_tap sum_o W[tap][i][o] * gpre[c - tap][o], gpre = gy * (y > 0) when
// the layer has a ReLU.  Written for the layers above the input only.
template <int CIN, int COUT, bool RELU>
__global__ void __launch_bounds__(256) kConvBwdData(WnGeom g, const float *__restrict__ gy,
                                                    const float *__restrict__ y, const __nv_bfloat16 *__restrict__ w,
                                                    float *__restrict__ gx) {
  __shared__ float ws[27 * CIN * COUT];
  for (int i = threadIdx.x; i < 27 * CIN * COUT; i += blockDim.x) ws[i] = __bfloat162float(w[i]);
  __syncthreads();
  const int64_t n = g.nAct << (3 * g.L);
  const int m = g.bs - 1;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    const int s = (int)(c >> (3 * g.L));
    const int v = (int)(c & ((1 << (3 * g.L)) - 1));
    const int lx = v & m, ly = (v >> g.L) & m, lz = v >> (2 * g.L);
    float acc[CIN];
#pragma unroll
    for (int i = 0; i < CIN; i++) acc[i] = 0.f;
    for (int t = 0; t < 27; t++) {
      const int64_t j = wnNbr(g, s, lx, ly, lz, -(t % 3 - 1), -((t / 3) % 3 - 1), -(t / 9 - 1));
      if (j < 0) continue;
      float gp[COUT];
#pragma unroll
      for (int o = 0; o < COUT; o++) {
        const float gv = gy[j * COUT + o];
        gp[o] = (!RELU || y[j * COUT + o] > 0.f) ? gv : 0.f;
      }
      const float *wt = ws + t * CIN * COUT;
#pragma unroll
      for (int i = 0; i < CIN; i++)
#pragma unroll
        for (int o = 0; o < COUT; o++) acc[i] = fmaf(wt[i * COUT + o], gp[o], acc[i]);
    }
#pragma unroll
    for (int i = 0; i < CIN; i++) gx[c * CIN + i] = acc[i];
  }
}

// gw[tap][i][o] += sum_c x[c + tap][i] * gpre[c][o]; gb[o] += sum_c gpre[c][o].
// A CTA takes kWChunk cells: their gpre in shared memory, one thread per (tap, i).
constexpr int kWChunk = 256;
template <int CIN, int COUT, bool RELU, bool NORM>
__global__ void __launch_bounds__(256) kConvBwdWeight(WnGeom g, const float *__restrict__ x,
                                                      const float *__restrict__ gy, const float *__restrict__ y,
                                                      const double *__restrict__ sc, float *__restrict__ gw,
                                                      float *__restrict__ gb) {
  __shared__ float gs[kWChunk * COUT];
  const int64_t n = g.nAct << (3 * g.L);
  const int64_t c0 = (int64_t)blockIdx.x * kWChunk;
  const int nc = (int)min((int64_t)kWChunk, n - c0);
  for (int k = threadIdx.x; k < kWChunk * COUT; k += blockDim.x) {
    const int cc = k / COUT, o = k % COUT;
    float v = 0.f;
    if (cc < nc) {
      const int64_t c = c0 + cc;
      v = gy[c * COUT + o];
      if (RELU && !(y[c * COUT + o] > 0.f)) v = 0.f;
    }
    gs[k] = v;
  }
  __syncthreads();
  if (threadIdx.x < COUT) {
    float t = 0.f;
    for (int cc = 0; cc < nc; cc++) t += gs[cc * COUT + threadIdx.x];
    atomicAdd(gb + threadIdx.x, t);
  }
  const float s0 = NORM ? (float)sc[1] : 1.f, s1 = NORM ? (float)sc[2] : 1.f;
  const int m = g.bs - 1;
  for (int ti = threadIdx.x; ti < 27 * CIN; ti += blockDim.x) {
    const int t = ti / CIN, i = ti % CIN;
    const int dx = t % 3 - 1, dy = (t / 3) % 3 - 1, dz = t / 9 - 1;
    float acc[COUT];
#pragma unroll
    for (int o = 0; o < COUT; o++) acc[o] = 0.f;
    for (int cc = 0; cc < nc; cc++) {
      const int64_t c = c0 + cc;
      const int s = (int)(c >> (3 * g.L));
      const int v = (int)(c & ((1 << (3 * g.L)) - 1));
      const int64_t j = wnNbr(g, s, v & m, (v >> g.L) & m, v >> (2 * g.L), dx, dy, dz);
      if (j < 0) continue;
      float xv;
      if constexpr (CIN == 2) {
        const float2 tv = reinterpret_cast<const float2 *>(x)[j];
        xv = i == 0 ? (NORM ? tv.x * s0 : tv.x) : (NORM ? tv.y * s1 - 1.0f : tv.y);
      } else {
        xv = x[j * CIN + i];
      }
#pragma unroll
      for (int o = 0; o < COUT; o++) acc[o] = fmaf(xv, gs[cc * COUT + o], acc[o]);
    }
#pragma unroll
    for (int o = 0; o < COUT; o++) atomicAdd(gw + (t * CIN + i) * COUT + o, acc[o]);
  }
}

// Adam on FP32 masters; the BF16 copy is refreshed
__global__ void kAdam(float *__restrict__ p, const float *__restrict__ gr, float *__restrict__ m, float *__restrict__ v,
                      __nv_bfloat16 *__restrict__ pq, int n, float lr, float b1t, float b2t) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float g = gr[i];
  const float mi = 0.9f * m[i] + 0.1f * g, vi = 0.999f * v[i] + 0.001f * g * g;
  m[i] = mi;
  v[i] = vi;
  const float mh = mi / (1.0f - b1t), vh = vi / (1.0f - b2t);
  const float np = p[i] - lr * mh / (sqrtf(vh) + 1e-8f);
  p[i] = np;
  if (pq) pq[i] = __float2bfloat16_rn(np);
}
__global__ void kToBf16(const float *__restrict__ a, __nv_bfloat16 *__restrict__ b, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = __float2bfloat16_rn(a[i]);
}
__global__ void kSub(const float *__restrict__ a, const float *__restrict__ b, float *__restrict__ c, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    c[i] = a[i] - b[i];
}
__global__ void kScaleInPlace(float *__restrict__ a, const double *__restrict__ num, const double *__restrict__ den,
                              float k, int64_t n) {
  const float f = den[0] > 0 ? (float)(k / den[0]) : 0.f;
  (void)num;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    a[i] *= f;
}

}  // namespace msbg

using namespace msbg;

// =====================================================================================
// host side
// =====================================================================================
namespace msbg {

void warmNetFree(WarmNetState *w) {
  if (!w) return;
  void *ptrs[] = {w->nbr27, w->x1, w->gx1, w->t0a, w->t0b, w->dScal, w->dPart, w->gact[0], w->gact[1]};
  for (void *p : ptrs) if (p) cudaFree(p);
  for (int l = 0; l < kWnLayers; l++) {
    void *q[] = {w->w32[l], w->bias[l], w->wq[l], w->gw[l], w->gb[l], w->mw[l], w->vw[l], w->mb[l], w->vb[l]};
    for (void *p : q) if (p) cudaFree(p);
  }
  for (int l = 0; l <= kWnLayers; l++) if (w->act[l]) cudaFree(w->act[l]);
  if (w->hScal) cudaFreeHost(w->hScal);
  delete w;
}

// persistent tensor-core convolutions: ctasPerSm resident CTAs per SM (each holds 32
// TMEM columns of the 512)
static unsigned wnTcGrid(int64_t n, int ctasPerSm) {
  int dev = 0, nSm = 152;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&nSm, cudaDevAttrMultiProcessorCount, dev);
  const int64_t tiles = (n + 127) / 128, cap = (int64_t)nSm * ctasPerSm;
  return (unsigned)(tiles < 1 ? 1 : tiles < cap ? tiles : cap);
}

static unsigned wnGrid(int64_t n) {
  int64_t g = (n + 255) / 256;
  if (g > 152 * 8) g = 152 * 8;
  return (unsigned)(g < 1 ? 1 : g);
}

// Level-1 buffers for the current layout (the weights survive a layout change).
static int wnEnsure(msbg_gpu_ctx *ctx) {
  int rc = poissonEnsure(ctx);
  if (rc) return rc;
  PoissonState *ps = ctx->poisson;
  if (ps->levels.size() < 3 || !ps->levels[1].sameSet || !ps->levels[2].sameSet || ps->levels[1].bs < 2)
    return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED, "warm start needs level-0 blocks of edge >= 4");
  if (!ctx->warmnet) {
    ctx->warmnet = new WarmNetState();
    WarmNetState *w = ctx->warmnet;
    for (int l = 0; l < kWnLayers; l++) {
      const int nw = wnWeights(l), nb = kWnCh[l + 1];
      MSBG_CUDA(ctx, cudaMalloc(&w->w32[l], nw * 4));
      MSBG_CUDA(ctx, cudaMalloc(&w->wq[l], nw * 2));
      MSBG_CUDA(ctx, cudaMalloc(&w->bias[l], nb * 4));
      for (float **q : {&w->gw[l], &w->mw[l], &w->vw[l]}) {
        MSBG_CUDA(ctx, cudaMalloc(q, nw * 4));
        MSBG_CUDA(ctx, cudaMemset(*q, 0, nw * 4));
      }
      for (float **q : {&w->gb[l], &w->mb[l], &w->vb[l]}) {
        MSBG_CUDA(ctx, cudaMalloc(q, nb * 4));
        MSBG_CUDA(ctx, cudaMemset(*q, 0, nb * 4));
      }
    }
    MSBG_CUDA(ctx, cudaMalloc(&w->dScal, 16 * 8));
    MSBG_CUDA(ctx, cudaMallocHost((void **)&w->hScal, 16 * 8));
    w->nPart = 152 * 8;
    MSBG_CUDA(ctx, cudaMalloc(&w->dPart, (size_t)w->nPart * 2 * 8));
  }
  WarmNetState *w = ctx->warmnet;
  if (w->layoutStamp == ctx->layoutStamp) return MSBG_GPU_OK;
  void *old[] = {w->nbr27, w->x1, w->gx1, w->t0a, w->t0b, w->gact[0], w->gact[1]};
  for (void *p : old) if (p) cudaFree(p);
  for (int l = 0; l <= kWnLayers; l++) { if (w->act[l]) cudaFree(w->act[l]); w->act[l] = nullptr; }
  w->nbr27 = nullptr; w->x1 = w->gx1 = w->t0a = w->t0b = w->gact[0] = w->gact[1] = nullptr;
  const MgLevel &L0 = ps->levels[0], &L1 = ps->levels[1], &L2 = ps->levels[2];
  w->n1 = L1.nCell;
  w->n2 = L2.nCell;
  const int64_t na = L0.nAct;
  MSBG_CUDA(ctx, cudaMalloc(&w->nbr27, (size_t)(na > 0 ? na : 1) * 27 * 4));
  if (na > 0) {
    MSBG_LAUNCH(ctx, kNbr27, gridFor(na * 27, 256), 256, 0, L0.active, na, L0.nbx, L0.nby, L0.nbz, L0.slot,
                w->nbr27);
  }
  const size_t n1 = (size_t)(w->n1 > 0 ? w->n1 : 1), n0 = (size_t)(L0.nCell > 0 ? L0.nCell : 1);
  for (int l = 0; l <= kWnLayers; l++) MSBG_CUDA(ctx, cudaMalloc(&w->act[l], n1 * kWnCh[l] * 4));
  MSBG_CUDA(ctx, cudaMalloc(&w->gact[0], n1 * 16 * 4));
  MSBG_CUDA(ctx, cudaMalloc(&w->gact[1], n1 * 16 * 4));
  MSBG_CUDA(ctx, cudaMalloc(&w->x1, n1 * 4));
  MSBG_CUDA(ctx, cudaMalloc(&w->gx1, n1 * 4));
  MSBG_CUDA(ctx, cudaMalloc(&w->t0a, n0 * 4));
  MSBG_CUDA(ctx, cudaMalloc(&w->t0b, n0 * 4));
  w->layoutStamp = ctx->layoutStamp;
  return MSBG_GPU_OK;
}

static WnGeom wnGeom(const PoissonState *ps, const WarmNetState *w) {
  const MgLevel &L1 = ps->levels[1];
  WnGeom g;
  g.bs = L1.bs; g.L = L1.log2bs; g.nAct = L1.nAct; g.nbr27 = w->nbr27;
  return g;
}

// the four forward convolutions, staged-neighbourhood tensor-core form
template <int BS1>
static int wnConvStaged(msbg_gpu_ctx *ctx, WarmNetState *w, const WnGeom &g) {
  constexpr size_t smem = stSmemBytes<BS1>();
  static bool attr = false;
  if (!attr) {
    MSBG_CUDA(ctx, cudaFuncSetAttribute(kConvTcStaged<BS1, 2, 16, true, true>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    MSBG_CUDA(ctx, cudaFuncSetAttribute(kConvTcStaged<BS1, 16, 16, true, false>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    MSBG_CUDA(ctx, cudaFuncSetAttribute(kConvTcStaged<BS1, 16, 2, false, false>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = true;
  }
  // resident CTAs per SM: 3 with the 58.5 KB of edge 16, 2 with the 87.5 KB of edge 8
  const unsigned gt = wnTcGrid(w->n1, smem <= 75 * 1024 ? 3 : 2);
  MSBG_LAUNCH(ctx, (kConvTcStaged<BS1, 2, 16, true, true>), gt, kTcThreads, smem, g, w->act[0], w->wq[0],
              w->bias[0], w->dScal, w->act[1], ctx->dStatus);
  MSBG_LAUNCH(ctx, (kConvTcStaged<BS1, 16, 16, true, false>), gt, kTcThreads, smem, g, w->act[1], w->wq[1],
              w->bias[1], w->dScal, w->act[2], ctx->dStatus);
  MSBG_LAUNCH(ctx, (kConvTcStaged<BS1, 16, 16, true, false>), gt, kTcThreads, smem, g, w->act[2], w->wq[2],
              w->bias[2], w->dScal, w->act[3], ctx->dStatus);
  MSBG_LAUNCH(ctx, (kConvTcStaged<BS1, 16, 2, false, false>), gt, kTcThreads, smem, g, w->act[3], w->wq[3],
              w->bias[3], w->dScal, w->act[4], ctx->dStatus);
  return MSBG_GPU_OK;
}

// forward pass from the level-0 right-hand side b0; x0 (level 0) optional
static int wnForward(msbg_gpu_ctx *ctx, const float *b0, float *x0) {
  PoissonState *ps = ctx->poisson;
  WarmNetState *w = ctx->warmnet;
  const WnGeom g = wnGeom(ps, w);
  const int L1 = g.L;
  MSBG_LAUNCH(ctx, kWnInputs, (unsigned)w->nPart, kRedThreads, 0, b0, (const float *)ps->f32.d[1], L1, w->n1,
              (float2 *)w->act[0], w->dPart);
  MSBG_LAUNCH(ctx, kWnScales, 1, kRedThreads, 0, w->dPart, w->nPart, w->n1, w->dScal);
  int rc;
  if (g.bs == 16) {
    if ((rc = wnConvStaged<16>(ctx, w, g))) return rc;
  } else if (g.bs == 8) {
    if ((rc = wnConvStaged<8>(ctx, w, g))) return rc;
  } else {  // level-1 blocks of edge 4: rows gathered per tap
    const unsigned gt = wnTcGrid(w->n1, 4);
    MSBG_LAUNCH(ctx, (kConvTc<2, 16, true, true>), gt, kTcThreads, 0, g, w->act[0], w->wq[0], w->bias[0], w->dScal,
                w->act[1], ctx->dStatus);
    MSBG_LAUNCH(ctx, (kConvTc<16, 16, true, false>), gt, kTcThreads, 0, g, w->act[1], w->wq[1], w->bias[1],
                w->dScal, w->act[2], ctx->dStatus);
    MSBG_LAUNCH(ctx, (kConvTc<16, 16, true, false>), gt, kTcThreads, 0, g, w->act[2], w->wq[2], w->bias[2],
                w->dScal, w->act[3], ctx->dStatus);
    MSBG_LAUNCH(ctx, (kConvTc<16, 2, false, false>), gt, kTcThreads, 0, g, w->act[3], w->wq[3], w->bias[3],
                w->dScal, w->act[4], ctx->dStatus);
  }
  MSBG_LAUNCH(ctx, kWnHead, gridFor(w->n2, 256), 256, 0, (const float2 *)w->act[4], w->dScal, L1, w->n2, w->x1, x0);
  return MSBG_GPU_OK;
}

// loss into hScal[4] (and dScal[4]); gradients into gw/gb (zeroed first)
static int wnLossGrad(msbg_gpu_ctx *ctx, const float *b0, const float *xs0) {
  PoissonState *ps = ctx->poisson;
  WarmNetState *w = ctx->warmnet;
  const WnGeom g = wnGeom(ps, w);
  const int64_t n0 = ps->levels[0].nCell;
  int rc;
  if (w->lossMode == 0) {  // coarse: loss and its gradient on level 1
    if ((rc = wnForward(ctx, b0, nullptr))) return rc;
    MSBG_LAUNCH(ctx, kWnCoarseDiff, (unsigned)w->nPart, kRedThreads, 0, w->x1, xs0, g.L, w->n1, w->gx1, w->dPart);
    MSBG_LAUNCH(ctx, kSum2, 1, kRedThreads, 0, w->dPart, w->nPart, w->dScal + 4);
    MSBG_LAUNCH(ctx, kWnHeadBack1, gridFor(w->n2, 256), 256, 0, w->gx1, w->dScal, 2.0f, g.L, w->n2,
                (float2 *)w->gact[0]);
  } else {
  if ((rc = wnForward(ctx, b0, w->t0a))) return rc;  // t0a = x0
  MSBG_LAUNCH(ctx, kSub, wnGrid(n0), 256, 0, w->t0a, xs0, w->t0a, n0);  // t0a = x0 - x*
  if ((rc = blkApply<float>(ctx, ps, 0, ps->f32, w->t0a, nullptr, w->t0b, 0, nullptr, nullptr, nullptr)))
    return rc;  // t0b = e = A (x0 - x*)
  if ((rc = blkDot<float>(ctx, ps, w->t0b, w->t0b, n0, w->dScal + 4))) return rc;   // sum e^2
  if ((rc = blkDot<float>(ctx, ps, b0, b0, n0, w->dScal + 5))) return rc;           // ||b||^2
  if ((rc = blkApply<float>(ctx, ps, 0, ps->f32, w->t0b, nullptr, w->t0a, 0, nullptr, nullptr, nullptr)))
    return rc;  // t0a = A e
  MSBG_LAUNCH(ctx, kScaleInPlace, wnGrid(n0), 256, 0, w->t0a, w->dScal + 4, w->dScal + 5, 2.0f, n0);  // g0
  MSBG_LAUNCH(ctx, kWnHeadBack, gridFor(w->n2, 256), 256, 0, w->t0a, w->dScal, g.L, w->n2, (float2 *)w->gact[0]);
  }
  for (int l = 0; l < kWnLayers; l++) {
    MSBG_CUDA(ctx, cudaMemsetAsync(w->gw[l], 0, wnWeights(l) * 4, ctx->stream));
    MSBG_CUDA(ctx, cudaMemsetAsync(w->gb[l], 0, kWnCh[l + 1] * 4, ctx->stream));
  }
  const unsigned gr = wnGrid(w->n1);
  const unsigned gwc = (unsigned)((w->n1 + kWChunk - 1) / kWChunk);
  // layer 3 (no ReLU): upstream gact[0] [n1][2]
  MSBG_LAUNCH(ctx, (kConvBwdWeight<16, 2, false, false>), gwc, 256, 0, g, w->act[3], w->gact[0], w->act[4], w->dScal,
              w->gw[3], w->gb[3]);
  MSBG_LAUNCH(ctx, (kConvBwdData<16, 2, false>), gr, 256, 0, g, w->gact[0], w->act[4], w->wq[3], w->gact[1]);
  // layer 2: upstream gact[1] [n1][16], ReLU on act[3]
  MSBG_LAUNCH(ctx, (kConvBwdWeight<16, 16, true, false>), gwc, 256, 0, g, w->act[2], w->gact[1], w->act[3],
              w->dScal, w->gw[2], w->gb[2]);
  MSBG_LAUNCH(ctx, (kConvBwdData<16, 16, true>), gr, 256, 0, g, w->gact[1], w->act[3], w->wq[2], w->gact[0]);
  // layer 1
  MSBG_LAUNCH(ctx, (kConvBwdWeight<16, 16, true, false>), gwc, 256, 0, g, w->act[1], w->gact[0], w->act[2],
              w->dScal, w->gw[1], w->gb[1]);
  MSBG_LAUNCH(ctx, (kConvBwdData<16, 16, true>), gr, 256, 0, g, w->gact[0], w->act[2], w->wq[1], w->gact[1]);
  // layer 0 (input scaling applied on load)
  MSBG_LAUNCH(ctx, (kConvBwdWeight<2, 16, true, true>), gwc, 256, 0, g, w->act[0], w->gact[1], w->act[1], w->dScal,
              w->gw[0], w->gb[0]);
  MSBG_CUDA(ctx, cudaMemcpyAsync(w->hScal + 4, w->dScal + 4, 2 * 8, cudaMemcpyDeviceToHost, ctx->stream));
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return MSBG_GPU_OK;
}

}  // namespace msbg

// ---- ABI --------------------------------------------------------------------------------
static int wnChanF32(msbg_gpu_ctx *ctx, int chan, float **p) {
  if (chan < 0 || chan >= kMaxChannels || !ctx->ch[chan].exists)
    return fail(ctx, MSBG_GPU_ERR_ARG, "channel %d does not exist", chan);
  if (ctx->ch[chan].storage != MSBG_GPU_F32) return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED, "channel %d is not FP32", chan);
  *p = (float *)ctx->ch[chan].d;
  return MSBG_GPU_OK;
}

static int wnReady(msbg_gpu_ctx *ctx) {
  if (!ctx->layoutValid) return fail(ctx, MSBG_GPU_ERR_STATE, "no block layout");
  int rc = poissonEnsure(ctx);
  if (rc) return rc;
  if (!ctx->poisson->coeffsValid) return fail(ctx, MSBG_GPU_ERR_STATE, "no Poisson coefficients set");
  return wnEnsure(ctx);
}

extern "C" int msbg_gpu_warmnet_param_count(int *nWeights, int *nBiases) {
  if (!nWeights || !nBiases) return MSBG_GPU_ERR_ARG;
  int a = 0, b = 0;
  for (int l = 0; l < kWnLayers; l++) { a += wnWeights(l); b += kWnCh[l + 1]; }
  *nWeights = a;
  *nBiases = b;
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_warmnet_set_weights(msbg_gpu_ctx *ctx, const float *hW, const float *hB, int resetOptimizer) {
  if (!ctx || !hW || !hB) return MSBG_GPU_ERR_ARG;
  int rc = wnReady(ctx);
  if (rc) return rc;
  WarmNetState *w = ctx->warmnet;
  int ow = 0, ob = 0;
  for (int l = 0; l < kWnLayers; l++) {
    const int nw = wnWeights(l), nb = kWnCh[l + 1];
    MSBG_CUDA(ctx, cudaMemcpyAsync(w->w32[l], hW + ow, nw * 4, cudaMemcpyHostToDevice, ctx->stream));
    MSBG_CUDA(ctx, cudaMemcpyAsync(w->bias[l], hB + ob, nb * 4, cudaMemcpyHostToDevice, ctx->stream));
    MSBG_LAUNCH(ctx, kToBf16, (nw + 255) / 256, 256, 0, w->w32[l], w->wq[l], nw);
    if (resetOptimizer) {
      for (float *q : {w->mw[l], w->vw[l]}) MSBG_CUDA(ctx, cudaMemsetAsync(q, 0, nw * 4, ctx->stream));
      for (float *q : {w->mb[l], w->vb[l]}) MSBG_CUDA(ctx, cudaMemsetAsync(q, 0, nb * 4, ctx->stream));
    }
    ow += nw;
    ob += nb;
  }
  if (resetOptimizer) w->step = 0;
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  w->weightsSet = true;
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_warmnet_get_weights(msbg_gpu_ctx *ctx, float *hW, float *hB) {
  if (!ctx || !hW || !hB) return MSBG_GPU_ERR_ARG;
  if (!ctx->warmnet || !ctx->warmnet->weightsSet) return fail(ctx, MSBG_GPU_ERR_STATE, "warm-start weights not set");
  WarmNetState *w = ctx->warmnet;
  int ow = 0, ob = 0;
  for (int l = 0; l < kWnLayers; l++) {
    const int nw = wnWeights(l), nb = kWnCh[l + 1];
    MSBG_CUDA(ctx, cudaMemcpyAsync(hW + ow, w->w32[l], nw * 4, cudaMemcpyDeviceToHost, ctx->stream));
    MSBG_CUDA(ctx, cudaMemcpyAsync(hB + ob, w->bias[l], nb * 4, cudaMemcpyDeviceToHost, ctx->stream));
    ow += nw;
    ob += nb;
  }
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_warmnet_set_loss(msbg_gpu_ctx *ctx, int lossMode) {
  if (!ctx || lossMode < 0 || lossMode > 1) return MSBG_GPU_ERR_ARG;
  int rc = wnReady(ctx);
  if (rc) return rc;
  ctx->warmnet->lossMode = lossMode;
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_warmnet_predict(msbg_gpu_ctx *ctx, int chanB, int chanX0) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  int rc = wnReady(ctx);
  if (rc) return rc;
  if (!ctx->warmnet->weightsSet) return fail(ctx, MSBG_GPU_ERR_STATE, "warm-start weights not set");
  float *b, *x;
  if ((rc = wnChanF32(ctx, chanB, &b)) || (rc = wnChanF32(ctx, chanX0, &x))) return rc;
  return wnForward(ctx, b, x);
}

static int wnGradsCore(msbg_gpu_ctx *ctx, const float *b, const float *xs, double *loss) {
  int rc = wnReady(ctx);
  if (rc) return rc;
  if (!ctx->warmnet->weightsSet) return fail(ctx, MSBG_GPU_ERR_STATE, "warm-start weights not set");
  if ((rc = wnLossGrad(ctx, b, xs))) return rc;
  WarmNetState *w = ctx->warmnet;
  const double bb = w->hScal[5];
  *loss = bb > 0 ? w->hScal[4] / bb : 0.0;
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_warmnet_loss_grad(msbg_gpu_ctx *ctx, int chanB, int chanXstar, double *loss, float *hGW,
                                          float *hGB) {
  if (!ctx || !loss) return MSBG_GPU_ERR_ARG;
  float *b, *xs;
  int rc;
  if ((rc = wnChanF32(ctx, chanB, &b)) || (rc = wnChanF32(ctx, chanXstar, &xs))) return rc;
  if ((rc = wnGradsCore(ctx, b, xs, loss))) return rc;
  WarmNetState *w = ctx->warmnet;
  int ow = 0, ob = 0;
  for (int l = 0; l < kWnLayers; l++) {
    const int nw = wnWeights(l), nb = kWnCh[l + 1];
    if (hGW) MSBG_CUDA(ctx, cudaMemcpyAsync(hGW + ow, w->gw[l], nw * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (hGB) MSBG_CUDA(ctx, cudaMemcpyAsync(hGB + ob, w->gb[l], nb * 4, cudaMemcpyDeviceToHost, ctx->stream));
    ow += nw;
    ob += nb;
  }
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_warmnet_train_step(msbg_gpu_ctx *ctx, const float *dB, const float *dXstar, float lr,
                                           double *loss) {
  if (!ctx || !dB || !dXstar || !loss || !(lr > 0)) return MSBG_GPU_ERR_ARG;
  int rc = wnGradsCore(ctx, dB, dXstar, loss);
  if (rc) return rc;
  WarmNetState *w = ctx->warmnet;
  w->step++;
  const float b1t = powf(0.9f, (float)w->step), b2t = powf(0.999f, (float)w->step);
  for (int l = 0; l < kWnLayers; l++) {
    const int nw = wnWeights(l), nb = kWnCh[l + 1];
    MSBG_LAUNCH(ctx, kAdam, (nw + 255) / 256, 256, 0, w->w32[l], w->gw[l], w->mw[l], w->vw[l], w->wq[l], nw, lr, b1t,
                b2t);
    MSBG_LAUNCH(ctx, kAdam, 1, 256, 0, w->bias[l], w->gb[l], w->mb[l], w->vb[l], (__nv_bfloat16 *)nullptr, nb, lr,
                b1t, b2t);
  }
  return MSBG_GPU_OK;
}
