// Batched Poisson solves: many independent sparse volumes on one combined block
// layout (each volume in its own region of the block grid, with empty blocks
// between volumes, so every operator, smoother and multigrid level is
// block-diagonal over the volumes), solved together by a segmented MG-PCG.
//
// Every CG scalar is per volume: dot products sum per block (one CTA per block),
// then per volume over its block list in a fixed order (deterministic); the step
// lengths alpha_v, beta_v are formed on the device; a volume whose recurrence
// residual reaches tol * ||b_v|| is frozen (alpha_v = beta_v = 0) and records its
// iteration.  One PCG iteration -- operator, V-cycle, segmented dots, updates -- is
// captured once in a CUDA graph and replayed; the host reads one counter (the
// number of converged volumes) per iteration and records an event per iteration,
// from which each volume's time to tolerance follows.
//
// Autotuning: the grid of the per-block dot kernel and of the vector updates (CTAs
// per SM) is chosen once per layout by timing the candidates on the live data.
#include <algorithm>
#include <vector>

#include "internal.cuh"
#include "poisson.cuh"

namespace msbg {

struct BatchState {
  int64_t layoutStamp = -1;
  int nVol = 0;
  int32_t *volOfSlot = nullptr;  // [nAct]
  int32_t *volStart = nullptr;   // [nVol + 1] offsets into volSlots
  int32_t *volSlots = nullptr;   // [nAct] slots grouped by volume
  double *blockPart = nullptr;   // [nAct]
  double *vs = nullptr;          // per-volume scalars [kVsCount][nVol]
  int32_t *conv = nullptr;       // [nVol] iteration at which the volume converged (0: not yet)
  int32_t *dCounters = nullptr;  // [0] converged volumes, [1] iteration
  int32_t *hCounters = nullptr;
  int updGrid = 0;               // autotuned grid of the vector kernels
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  const void *graphKey[3] = {};  // x, b, tol bits of the captured iteration
  double graphTol = 0.0;
};

// rows of the per-volume scalar array
enum { kVsRz = 0, kVsPq, kVsRr, kVsRzn, kVsAlpha, kVsBeta, kVsBn, kVsCount };

// ---- kernels --------------------------------------------------------------------------
// blockPart[s] = sum over block s of a*b (FP32 products per 4 values, FP64 sums)
template <typename V>
__global__ void __launch_bounds__(256) kBlockDot(const V *__restrict__ a, const V *__restrict__ b, int log2vpb,
                                                 double *__restrict__ blockPart) {
  const int64_t s = blockIdx.x;
  const int64_t base = s << log2vpb;
  const int nq = (1 << log2vpb) / 4;
  double acc = 0.0;
  for (int q = threadIdx.x; q < nq; q += blockDim.x) {
    float av[4], bv[4];
    ldRow<4>(a + base + 4 * q, av);
    ldRow<4>(b + base + 4 * q, bv);
    float t = 0.f;
#pragma unroll
    for (int i = 0; i < 4; i++) t = fmaf(av[i], bv[i], t);
    acc += (double)t;
  }
  acc = blockSum(acc);
  if (threadIdx.x == 0) blockPart[s] = acc;
}
// out[v] = sum of blockPart over the volume's blocks (fixed order)
__global__ void kVolReduce(const double *__restrict__ blockPart, const int32_t *__restrict__ volStart,
                           const int32_t *__restrict__ volSlots, double *__restrict__ out) {
  const int v = blockIdx.x;
  double acc = 0.0;
  for (int i = volStart[v] + threadIdx.x; i < volStart[v + 1]; i += blockDim.x) acc += blockPart[volSlots[i]];
  acc = blockSum(acc);
  if (threadIdx.x == 0) out[v] = acc;
}
// stage 0 (after p.s): alpha; stage 1 (after r.r): convergence; stage 2 (after r.z):
// beta, rz, next iteration.  One CTA loops over the volumes.
__global__ void kVolScalars(double *__restrict__ vs, int nVol, int stage, double tol, int32_t *__restrict__ conv,
                            int32_t *__restrict__ counters) {
  const int it = counters[1];
  double *rz = vs + kVsRz * nVol, *pq = vs + kVsPq * nVol, *rr = vs + kVsRr * nVol, *rzn = vs + kVsRzn * nVol;
  double *al = vs + kVsAlpha * nVol, *be = vs + kVsBeta * nVol, *bn = vs + kVsBn * nVol;
  int newly = 0;
  for (int v = threadIdx.x; v < nVol; v += blockDim.x) {
    const bool done = conv[v] != 0;
    if (stage == 0) {
      al[v] = (!done && pq[v] != 0.0) ? rz[v] / pq[v] : 0.0;
    } else if (stage == 1) {
      if (!done && sqrt(rr[v]) <= tol * sqrt(bn[v])) {
        conv[v] = it;
        newly++;
      }
    } else {
      be[v] = (!done && rz[v] != 0.0) ? rzn[v] / rz[v] : 0.0;
      rz[v] = rzn[v];
    }
  }
  if (newly) atomicAdd(counters, newly);
  __syncthreads();
  if (stage == 2 && threadIdx.x == 0) counters[1] = it + 1;
}
// initial state: volumes with ||b|| = 0 or an initial residual within tolerance are done
__global__ void kVolInit(double *__restrict__ vs, int nVol, double tol, int32_t *__restrict__ conv,
                         int32_t *__restrict__ counters) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v == 0) counters[1] = 1;
  if (v >= nVol) return;
  const double bn = vs[kVsBn * nVol + v], rr = vs[kVsRr * nVol + v];
  conv[v] = 0;
  if (bn == 0.0 || sqrt(rr) <= tol * sqrt(bn)) {
    conv[v] = -1;  // converged before the first iteration
    atomicAdd(counters, 1);
  }
}

// after every volume met the tolerance on its recurrence residual: vs[rr] now holds
// the true ||b - A x||^2 of each volume; volumes that miss the tolerance on it resume
__global__ void kVolRecheck(const double *__restrict__ vs, int nVol, double tol, int32_t *__restrict__ conv,
                            int32_t *__restrict__ counters) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nVol) return;
  const double bn = vs[kVsBn * nVol + v], rr = vs[kVsRr * nVol + v];
  if (conv[v] != 0 && !(bn == 0.0 || sqrt(rr) <= tol * sqrt(bn))) {
    conv[v] = 0;
    atomicSub(counters, 1);
  }
}

template <typename V>
__global__ void __launch_bounds__(256) kUpdateXRVol(const double *__restrict__ alpha, const int32_t *__restrict__ vol,
                                                    int log2vpb, const V *__restrict__ p, const V *__restrict__ q,
                                                    V *__restrict__ x, V *__restrict__ r, int64_t nq) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nq; k += (int64_t)gridDim.x * blockDim.x) {
    const float a = (float)alpha[vol[(4 * k) >> log2vpb]];
    if (a == 0.f) continue;
    float pv[4], qv[4], xv[4], rv[4];
    ldRow<4>(p + 4 * k, pv);
    ldRow<4>(q + 4 * k, qv);
    ldRow<4>(x + 4 * k, xv);
    ldRow<4>(r + 4 * k, rv);
#pragma unroll
    for (int i = 0; i < 4; i++) {
      xv[i] = fmaf(a, pv[i], xv[i]);
      rv[i] = fmaf(-a, qv[i], rv[i]);
    }
    stRow<4>(x + 4 * k, xv);
    stRow<4>(r + 4 * k, rv);
  }
}
template <typename V>
__global__ void __launch_bounds__(256) kUpdatePVol(const double *__restrict__ beta, const int32_t *__restrict__ vol,
                                                   int log2vpb, const V *__restrict__ z, V *__restrict__ p, int64_t nq) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nq; k += (int64_t)gridDim.x * blockDim.x) {
    const float bt = (float)beta[vol[(4 * k) >> log2vpb]];
    float zv[4], pv[4];
    ldRow<4>(z + 4 * k, zv);
    ldRow<4>(p + 4 * k, pv);
#pragma unroll
    for (int i = 0; i < 4; i++) pv[i] = fmaf(bt, pv[i], zv[i]);
    stRow<4>(p + 4 * k, pv);
  }
}
__global__ void kVolOfSlot(const int32_t *__restrict__ active, int64_t nAct, const int32_t *__restrict__ volOfBlock,
                           int32_t *__restrict__ volOfSlot) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nAct) volOfSlot[s] = volOfBlock[active[s]];
}

// ---- host ------------------------------------------------------------------------------
void batchFree(BatchState *b) {
  if (!b) return;
  void *p[] = {b->volOfSlot, b->volStart, b->volSlots, b->blockPart, b->vs, b->conv, b->dCounters};
  for (void *q : p) if (q) cudaFree(q);
  if (b->hCounters) cudaFreeHost(b->hCounters);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

// Host-side declarations of the Poisson pieces used here (poisson.cu)
int batchApply(msbg_gpu_ctx *ctx, const float *x, const float *b, float *y, int mode);
int batchVcycle(msbg_gpu_ctx *ctx, float *x, const float *b);

}  // namespace msbg

using namespace msbg;

namespace {

int segDot(msbg_gpu_ctx *ctx, BatchState *bs, const float *a, const float *b, double *out) {
  const int64_t nAct = ctx->poisson->levels[0].nAct;
  const int lv = 3 * ctx->poisson->levels[0].log2bs;
  MSBG_LAUNCH(ctx, kBlockDot<float>, (unsigned)nAct, 256, 0, a, b, lv, bs->blockPart);
  MSBG_LAUNCH(ctx, kVolReduce, (unsigned)bs->nVol, kRedThreads, 0, bs->blockPart, bs->volStart, bs->volSlots, out);
  return MSBG_GPU_OK;
}

constexpr double kRecurMargin = 0.8;

// One PCG iteration on every volume (what the graph holds).
int batchIteration(msbg_gpu_ctx *ctx, BatchState *bs, float *x, double tol) {
  PoissonState *ps = ctx->poisson;
  const MgLevel &L0 = ps->levels[0];
  const int64_t n = L0.nCell;
  const int lv = 3 * L0.log2bs, nV = bs->nVol;
  float *r = (float *)ps->f32.vr, *p = (float *)ps->f32.vp, *z = (float *)ps->f32.vz, *s = (float *)ps->f32.vs;
  double *vs = bs->vs;
  int rc;
  if ((rc = batchApply(ctx, p, nullptr, s, 0))) return rc;
  if ((rc = segDot(ctx, bs, p, s, vs + kVsPq * nV))) return rc;
  MSBG_LAUNCH(ctx, kVolScalars, 1, 1024, 0, vs, nV, 0, tol, bs->conv, bs->dCounters);
  MSBG_LAUNCH(ctx, kUpdateXRVol<float>, (unsigned)bs->updGrid, 256, 0, vs + kVsAlpha * nV, bs->volOfSlot, lv, p, s,
              x, r, n / 4);
  if ((rc = segDot(ctx, bs, r, r, vs + kVsRr * nV))) return rc;
  // the recurrence residual may drift from the true one by a few FP32 roundings: stop
  // it at kRecurMargin * tol so that the true-residual confirmation rarely restarts
  MSBG_LAUNCH(ctx, kVolScalars, 1, 1024, 0, vs, nV, 1, kRecurMargin * tol, bs->conv, bs->dCounters);
  if ((rc = batchVcycle(ctx, z, r))) return rc;
  if ((rc = segDot(ctx, bs, r, z, vs + kVsRzn * nV))) return rc;
  MSBG_LAUNCH(ctx, kVolScalars, 1, 1024, 0, vs, nV, 2, tol, bs->conv, bs->dCounters);
  MSBG_LAUNCH(ctx, kUpdatePVol<float>, (unsigned)bs->updGrid, 256, 0, vs + kVsBeta * nV, bs->volOfSlot, lv, z, p,
              n / 4);
  return MSBG_GPU_OK;
}

// Picks the grid of the vector updates (CTAs per SM) by timing the candidates.
int autotune(msbg_gpu_ctx *ctx, BatchState *bs) {
  PoissonState *ps = ctx->poisson;
  const int64_t n = ps->levels[0].nCell;
  const int lv = 3 * ps->levels[0].log2bs;
  float *p = (float *)ps->f32.vp, *z = (float *)ps->f32.vz;
  const int cands[] = {2, 4, 8, 16, 32};
  cudaEvent_t e0, e1;
  MSBG_CUDA(ctx, cudaEventCreate(&e0));
  MSBG_CUDA(ctx, cudaEventCreate(&e1));
  float best = 1e30f;
  int bestG = 152 * 8;
  const int64_t maxG = (n / 4 + 255) / 256;
  for (int c : cands) {
    int64_t gsz = 152LL * c;
    if (gsz > maxG) gsz = maxG;
    if (gsz < 1) gsz = 1;
    MSBG_LAUNCH(ctx, kUpdatePVol<float>, (unsigned)gsz, 256, 0, bs->vs + kVsBeta * bs->nVol, bs->volOfSlot, lv, z, p,
                n / 4);  // warm
    MSBG_CUDA(ctx, cudaEventRecord(e0, ctx->stream));
    for (int k = 0; k < 3; k++)
      MSBG_LAUNCH(ctx, kUpdatePVol<float>, (unsigned)gsz, 256, 0, bs->vs + kVsBeta * bs->nVol, bs->volOfSlot, lv, z,
                  p, n / 4);
    MSBG_CUDA(ctx, cudaEventRecord(e1, ctx->stream));
    MSBG_CUDA(ctx, cudaEventSynchronize(e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) { best = ms; bestG = (int)gsz; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  bs->updGrid = bestG;
  return MSBG_GPU_OK;
}

int chanF32b(msbg_gpu_ctx *ctx, int chan, float **p) {
  if (chan < 0 || chan >= kMaxChannels || !ctx->ch[chan].exists)
    return fail(ctx, MSBG_GPU_ERR_ARG, "channel %d does not exist", chan);
  if (ctx->ch[chan].storage != MSBG_GPU_F32) return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED, "channel %d is not FP32", chan);
  *p = (float *)ctx->ch[chan].d;
  return MSBG_GPU_OK;
}

}  // namespace

extern "C" int msbg_gpu_batch_set_volumes(msbg_gpu_ctx *ctx, const int32_t *hVolOfBlock, int nVol) {
  if (!ctx || !hVolOfBlock || nVol < 1) return MSBG_GPU_ERR_ARG;
  if (!ctx->layoutValid) return fail(ctx, MSBG_GPU_ERR_STATE, "no block layout: call set_refinement_map");
  int rc = poissonEnsure(ctx);
  if (rc) return rc;
  if (ctx->batch) { batchFree(ctx->batch); ctx->batch = nullptr; }
  BatchState *bs = new BatchState();
  ctx->batch = bs;
  bs->nVol = nVol;
  const int64_t nAct = ctx->nActive;
  // volume of every active slot
  int32_t *dVB = nullptr;
  MSBG_CUDA(ctx, cudaMalloc(&dVB, (size_t)ctx->nBlocks * 4));
  MSBG_CUDA(ctx, cudaMemcpyAsync(dVB, hVolOfBlock, (size_t)ctx->nBlocks * 4, cudaMemcpyHostToDevice, ctx->stream));
  MSBG_CUDA(ctx, cudaMalloc(&bs->volOfSlot, (size_t)(nAct > 0 ? nAct : 1) * 4));
  if (nAct > 0) MSBG_LAUNCH(ctx, kVolOfSlot, gridFor(nAct, 256), 256, 0, ctx->dActive, nAct, dVB, bs->volOfSlot);
  std::vector<int32_t> vos(nAct);
  if (nAct > 0)
    MSBG_CUDA(ctx, cudaMemcpyAsync(vos.data(), bs->volOfSlot, (size_t)nAct * 4, cudaMemcpyDeviceToHost, ctx->stream));
  MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  cudaFree(dVB);
  std::vector<int32_t> start(nVol + 1, 0), slots(nAct);
  for (int64_t s = 0; s < nAct; s++) {
    if (vos[s] < 0 || vos[s] >= nVol)
      return fail(ctx, MSBG_GPU_ERR_ARG, "active block %lld has no volume (%d)", (long long)s, vos[s]);
    start[vos[s] + 1]++;
  }
  for (int v = 0; v < nVol; v++) start[v + 1] += start[v];
  std::vector<int32_t> fillp(start.begin(), start.end() - 1);
  for (int64_t s = 0; s < nAct; s++) slots[fillp[vos[s]]++] = (int32_t)s;
  MSBG_CUDA(ctx, cudaMalloc(&bs->volStart, (size_t)(nVol + 1) * 4));
  MSBG_CUDA(ctx, cudaMalloc(&bs->volSlots, (size_t)(nAct > 0 ? nAct : 1) * 4));
  MSBG_CUDA(ctx, cudaMemcpy(bs->volStart, start.data(), (size_t)(nVol + 1) * 4, cudaMemcpyHostToDevice));
  if (nAct > 0) MSBG_CUDA(ctx, cudaMemcpy(bs->volSlots, slots.data(), (size_t)nAct * 4, cudaMemcpyHostToDevice));
  MSBG_CUDA(ctx, cudaMalloc(&bs->blockPart, (size_t)(nAct > 0 ? nAct : 1) * 8));
  MSBG_CUDA(ctx, cudaMalloc(&bs->vs, (size_t)kVsCount * nVol * 8));
  MSBG_CUDA(ctx, cudaMemset(bs->vs, 0, (size_t)kVsCount * nVol * 8));
  MSBG_CUDA(ctx, cudaMalloc(&bs->conv, (size_t)nVol * 4));
  MSBG_CUDA(ctx, cudaMalloc(&bs->dCounters, 16));
  MSBG_CUDA(ctx, cudaMallocHost((void **)&bs->hCounters, 16));
  MSBG_CUDA(ctx, cudaStreamCreateWithFlags(&bs->stream, cudaStreamNonBlocking));
  bs->layoutStamp = ctx->layoutStamp;
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_batch_mgpcg_solve(msbg_gpu_ctx *ctx, int chanX, int chanB, double tol, int maxIter,
                                          int useGraph, int32_t *hIters, float *hMsToTol, double *hRelRes,
                                          float *hTotalMs) {
  if (!ctx || !(tol > 0) || maxIter < 1) return MSBG_GPU_ERR_ARG;
  BatchState *bs = ctx->batch;
  if (!bs || bs->layoutStamp != ctx->layoutStamp) return fail(ctx, MSBG_GPU_ERR_STATE, "call batch_set_volumes");
  int rc = poissonEnsure(ctx);
  if (rc) return rc;
  PoissonState *ps = ctx->poisson;
  if (!ps->coeffsValid) return fail(ctx, MSBG_GPU_ERR_STATE, "no Poisson coefficients set");
  if ((rc = ensureF32Work(ctx, ps))) return rc;
  float *x, *b;
  if ((rc = chanF32b(ctx, chanX, &x)) || (rc = chanF32b(ctx, chanB, &b))) return rc;
  const int nV = bs->nVol;
  const int64_t n = ps->levels[0].nCell;
  float *r = (float *)ps->f32.vr, *p = (float *)ps->f32.vp, *z = (float *)ps->f32.vz;
  // run on the batch's own stream (graph capture needs a non-legacy stream)
  cudaStream_t userStream = ctx->stream;
  MSBG_CUDA(ctx, cudaStreamSynchronize(userStream));
  ctx->stream = bs->stream;
  struct Restore {
    msbg_gpu_ctx *c;
    cudaStream_t s;
    ~Restore() { c->stream = s; }
  } restore{ctx, userStream};
  if (bs->updGrid == 0 && (rc = autotune(ctx, bs))) return rc;

  std::vector<cudaEvent_t> ev(maxIter + 1);
  for (auto &e : ev) MSBG_CUDA(ctx, cudaEventCreate(&e));
  struct Events {
    std::vector<cudaEvent_t> &v;
    ~Events() { for (auto &e : v) cudaEventDestroy(e); }
  } evGuard{ev};
  MSBG_CUDA(ctx, cudaEventRecord(ev[0], ctx->stream));
  // r = b - A x; ||b_v||^2, ||r_v||^2; z = M r; p = z; rz_v
  if ((rc = batchApply(ctx, x, b, r, 1))) return rc;
  if ((rc = segDot(ctx, bs, b, b, bs->vs + kVsBn * nV))) return rc;
  if ((rc = segDot(ctx, bs, r, r, bs->vs + kVsRr * nV))) return rc;
  MSBG_CUDA(ctx, cudaMemsetAsync(bs->dCounters, 0, 16, ctx->stream));
  MSBG_LAUNCH(ctx, kVolInit, (unsigned)((nV + 127) / 128), 128, 0, bs->vs, nV, tol, bs->conv, bs->dCounters);
  if ((rc = batchVcycle(ctx, z, r))) return rc;
  MSBG_CUDA(ctx, cudaMemcpyAsync(p, z, (size_t)n * 4, cudaMemcpyDeviceToDevice, ctx->stream));
  if ((rc = segDot(ctx, bs, r, z, bs->vs + kVsRz * nV))) return rc;

  const bool graphOk = useGraph && bs->graph && bs->graphKey[0] == x && bs->graphKey[1] == b && bs->graphTol == tol;
  int it = 1;
  // iterations it, it+1, ... until every volume has met the tolerance on its
  // recurrence residual (it is then the last iteration run) or maxIter has run
  auto iterate = [&]() -> int {
    for (; it <= maxIter; it++) {
      if (useGraph && !graphOk && it == 2) {  // capture after one eager iteration (caches warm)
        if (bs->graph) { cudaGraphExecDestroy(bs->graph); bs->graph = nullptr; }
        cudaGraph_t gr;
        MSBG_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        const int64_t l0 = ctx->launches;
        int rc2 = batchIteration(ctx, bs, x, tol);
        cudaError_t ce = cudaStreamEndCapture(ctx->stream, &gr);
        if (rc2) return rc2;
        MSBG_CUDA(ctx, ce);
        MSBG_CUDA(ctx, cudaGraphInstantiate(&bs->graph, gr, 0));
        cudaGraphDestroy(gr);
        ctx->launches = l0;  // captured, not launched
        bs->graphKey[0] = x; bs->graphKey[1] = b; bs->graphTol = tol;
      }
      if (useGraph && bs->graph && (graphOk || it >= 2)) {
        MSBG_CUDA(ctx, cudaGraphLaunch(bs->graph, ctx->stream));
        ctx->launches += 1;
      } else {
        int rc2 = batchIteration(ctx, bs, x, tol);
        if (rc2) return rc2;
      }
      MSBG_CUDA(ctx, cudaEventRecord(ev[it], ctx->stream));
      MSBG_CUDA(ctx, cudaMemcpyAsync(bs->hCounters, bs->dCounters, 8, cudaMemcpyDeviceToHost, ctx->stream));
      MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      if (bs->hCounters[0] >= nV) return MSBG_GPU_OK;
    }
    return MSBG_GPU_OK;
  };
  if ((rc = iterate())) return rc;
  // Confirm on the true residual (as the single solve does): volumes whose
  // ||b - A x|| misses the tolerance resume CG from it; the others stay frozen.
  for (int check = 0; check < 8 && it < maxIter && bs->hCounters[0] >= nV; check++) {
    if ((rc = batchApply(ctx, x, b, r, 1))) return rc;
    if ((rc = segDot(ctx, bs, r, r, bs->vs + kVsRr * nV))) return rc;
    MSBG_LAUNCH(ctx, kVolRecheck, (unsigned)((nV + 127) / 128), 128, 0, bs->vs, nV, tol, bs->conv, bs->dCounters);
    MSBG_CUDA(ctx, cudaMemcpyAsync(bs->hCounters, bs->dCounters, 8, cudaMemcpyDeviceToHost, ctx->stream));
    MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (bs->hCounters[0] >= nV) break;
    if ((rc = batchVcycle(ctx, z, r))) return rc;
    MSBG_CUDA(ctx, cudaMemcpyAsync(p, z, (size_t)n * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    if ((rc = segDot(ctx, bs, r, z, bs->vs + kVsRz * nV))) return rc;
    it++;
    if ((rc = iterate())) return rc;
  }
  if (it > maxIter) it = maxIter;
  // per-volume results: iterations, time to tolerance, FP64-checked relative residual
  std::vector<int32_t> conv(nV);
  MSBG_CUDA(ctx, cudaMemcpy(conv.data(), bs->conv, (size_t)nV * 4, cudaMemcpyDeviceToHost));
  float total = 0.f;
  MSBG_CUDA(ctx, cudaEventElapsedTime(&total, ev[0], ev[it]));
  if (hTotalMs) *hTotalMs = total;
  for (int v = 0; v < nV; v++) {
    const int k = conv[v] < 0 ? 0 : conv[v];  // -1: done at start; 0: not converged
    if (hIters) hIters[v] = conv[v] == 0 ? -1 : k;
    if (hMsToTol) {
      float ms = -1.f;
      if (conv[v] != 0) cudaEventElapsedTime(&ms, ev[0], ev[k]);
      hMsToTol[v] = ms;
    }
  }
  if (hRelRes) {
    if ((rc = batchApply(ctx, x, b, r, 1))) return rc;
    if ((rc = segDot(ctx, bs, r, r, bs->vs + kVsRr * nV))) return rc;
    std::vector<double> rr(nV), bb(nV);
    MSBG_CUDA(ctx, cudaMemcpyAsync(rr.data(), bs->vs + kVsRr * nV, (size_t)nV * 8, cudaMemcpyDeviceToHost,
                                   ctx->stream));
    MSBG_CUDA(ctx, cudaMemcpyAsync(bb.data(), bs->vs + kVsBn * nV, (size_t)nV * 8, cudaMemcpyDeviceToHost,
                                   ctx->stream));
    MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int v = 0; v < nV; v++) hRelRes[v] = bb[v] > 0 ? sqrt(rr[v] / bb[v]) : 0.0;
  }
  int st = 0;
  MSBG_CUDA(ctx, cudaMemcpy(&st, ctx->dStatus, sizeof(int), cudaMemcpyDeviceToHost));
  if (st) {
    MSBG_CUDA(ctx, cudaMemset(ctx->dStatus, 0, sizeof(int)));
    return fail(ctx, MSBG_GPU_ERR_TIMEOUT, "a bounded device wait timed out (status bits %d)", st);
  }
  return MSBG_GPU_OK;
}
