// Grid-to-particle trilinear interpolation (G2P): the value of a channel at n points.
//
// SparseGrid<float>::interpolateFloatFast (src/sbg.h:4623-4792),
// SparseGrid<uint16_t>::interpolateUint16ToFloatFast (src/sbg.h:4920-5032) and, with
// MSBG_GPU_IP_RENDER_DENS, interpolateRenderDensity (src/msbg.h:478-484), called once per
// point in the reference.  The per-point arithmetic is ipValue (interp_common.cuh).
//
// One thread per point.  A point whose 8 corners lie in one block (bs-1 of bs cells per
// axis) reads one slot and 8 values within 2 rows of 2 planes.  A point on a block's
// upper face looks up the slot of each corner's block.  Bytes: 12 per point read plus 4
// written; the corner reads are gathers served mostly by L1/L2, since neighbouring points
// share blocks.
#include "interp_common.cuh"

namespace msbg {

namespace {

template <typename T>
__global__ void __launch_bounds__(256) kInterpolate(IpGeom g, const int32_t *__restrict__ slot,
                                                    const T *__restrict__ payload,
                                                    const float *__restrict__ pts, int64_t n,
                                                    float *__restrict__ out) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  out[k] = ipValue<T>(g, slot, payload, __ldg(pts + 3 * k), __ldg(pts + 3 * k + 1), __ldg(pts + 3 * k + 2));
}

template <typename T>
int interpolateLaunch(msbg_gpu_ctx *ctx, const Channel &c, const IpGeom &g, const float *dPts,
                      int64_t n, float *dOut) {
  MSBG_LAUNCH(ctx, kInterpolate<T>, gridFor(n, 256), 256, 0, g, ctx->dSlot,
              static_cast<const T *>(c.d), dPts, n, dOut);
  return MSBG_GPU_OK;
}

}  // namespace

}  // namespace msbg

using namespace msbg;

extern "C" int msbg_gpu_interpolate(msbg_gpu_ctx *ctx, int chan, const float *dPts, int64_t n,
                                    float *dOut, int opt) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  if (n < 0) return fail(ctx, MSBG_GPU_ERR_ARG, "interpolate: negative point count");
  if (n > 0 && (!dPts || !dOut)) return fail(ctx, MSBG_GPU_ERR_ARG, "interpolate: null buffer");
  if (chan < 0 || chan >= kMaxChannels || !ctx->ch[chan].exists)
    return fail(ctx, MSBG_GPU_ERR_ARG, "channel %d does not exist", chan);
  const int known = MSBG_GPU_IP_CORNER | MSBG_GPU_IP_CHKBLK | MSBG_GPU_IP_BC_DIRICHLET |
                    MSBG_GPU_IP_BC_DIRICHLET_OLD | MSBG_GPU_IP_NO_BORDER_CHECK |
                    MSBG_GPU_IP_RENDER_DENS;
  if (opt & ~known)
    return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED, "interpolate: unsupported option bits 0x%x", opt & ~known);
  if (!ctx->layoutValid) return fail(ctx, MSBG_GPU_ERR_STATE, "no block layout: call set_refinement_map");
  if (n == 0) return MSBG_GPU_OK;
  const Channel &c = ctx->ch[chan];
  IpGeom g;
  g.sx = ctx->sx; g.sy = ctx->sy; g.sz = ctx->sz;
  g.log2bs = ctx->log2bs;
  g.nbx = ctx->nbx;
  g.nxy = (int64_t)ctx->nbx * ctx->nby;
  g.vpb = ctx->voxPerBlock;
  g.po = (opt & MSBG_GPU_IP_CORNER) ? 0.0f : 0.5f;
  g.dirichlet = (opt & MSBG_GPU_IP_BC_DIRICHLET) != 0;
  g.dirichletOld = (opt & MSBG_GPU_IP_BC_DIRICHLET_OLD) != 0;
  g.renderDens = (opt & MSBG_GPU_IP_RENDER_DENS) != 0 && c.storage == MSBG_GPU_U16;
  switch (c.storage) {
    case MSBG_GPU_F32: return interpolateLaunch<float>(ctx, c, g, dPts, n, dOut);
    case MSBG_GPU_F16: return interpolateLaunch<__half>(ctx, c, g, dPts, n, dOut);
    case MSBG_GPU_U16: return interpolateLaunch<uint16_t>(ctx, c, g, dPts, n, dOut);
    default:
      return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED, "interpolate: FP64 channels are not supported");
  }
}
