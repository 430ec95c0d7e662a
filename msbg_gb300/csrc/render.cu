// Ray-march render of the iso-0.5 surface of a value-block channel into an RGB buffer.
//
// Reference: RDR::RaymarchRenderer (src/render.h:52-160, src/render.cpp:20-101), the demo's
// visual check of the splatted and smoothed density (src/msbg_demo.cpp:129-175).  There it
// renders a BMP bitmap on the CPU, one thread per image row; here one thread per pixel
// writes 3 bytes of a device buffer (row-major, top row first), with no graphics API.
//
// Per pixel, in FP64 as the reference (RealType = double):
//  - camera basis forward = normalize(lookAt - pos), right = normalize(cross(forward, +y)),
//    up = cross(right, forward); ndc = ((x + .5)/W - .5) * 2 * aspect, (.5 - (y + .5)/H) * 2;
//    dir = normalize(forward * zoom + right * ndcX + up * ndcY);
//  - the ray starts at the camera and moves by dir / res per step (res = max(sx, sy, sz)),
//    at most 2 units;
//  - density(p) (sampleDensity, src/render.h:89-117): 0 outside the domain or in a block
//    without payload, else the trilinear interpolant at res * p (FP32; uint16 times
//    1/65535);
//  - the first step whose density crosses 0.5 upwards is the hit, placed by linear
//    interpolation; normal = -grad of the cubic B-spline interpolant there
//    (interpolateWithDerivs0<IP_BSPLINE_CUBIC>, src/sbg.h:3903-4133; window voxels outside
//    the domain clamped to it), Lambert shading with the sun, channels rounded to 8 bits.
// Where the reference's -ffast-math build fuses a multiply into an add, the code here uses
// the same fused forms (dot products, cross products, ndc, hit placement); every operation
// is an explicitly rounded intrinsic, so nothing else is contracted.  The CPU restatement
// (orc_render) uses the same forms; both agree with the reference's image except for a
// few pixels one step apart in a colour channel.
//
// A ray that has left the domain on an axis while moving outward on it can never read a
// nonzero density again (positions are monotonic per axis under rounded addition), so it
// stops there; the result is the same as marching to the end.
//
// Cost: per step 3 FP64 adds and 3 FP64->FP32 conversions plus one block-slot read; the
// interpolation only inside value blocks.  Bound: the FP64 pipe for rays through empty
// space, gathers near the surface.
#include "interp_common.cuh"

namespace msbg {

namespace {

struct RV {
  double x, y, z;
};

__device__ __forceinline__ RV rsub(RV a, RV b) { return {__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y), __dsub_rn(a.z, b.z)}; }
// a.x*b.x + a.y*b.y + a.z*b.z, fused left to right
__device__ __forceinline__ double rdot(RV a, RV b) {
  return __fma_rn(a.z, b.z, __fma_rn(a.y, b.y, __dmul_rn(a.x, b.x)));
}
__device__ __forceinline__ RV rnormalize(RV v) {
  const double len = __dsqrt_rn(rdot(v, v));
  if (!(len > (double)1e-20f)) return {0.0, 1.0, 0.0};
  return {__ddiv_rn(v.x, len), __ddiv_rn(v.y, len), __ddiv_rn(v.z, len)};
}
// a.y*b.z - a.z*b.y, ... fused as fma(a.y, b.z, -(a.z*b.y))
__device__ __forceinline__ RV rcross(RV a, RV b) {
  return {__fma_rn(a.y, b.z, -__dmul_rn(a.z, b.y)), __fma_rn(a.z, b.x, -__dmul_rn(a.x, b.z)),
          __fma_rn(a.x, b.y, -__dmul_rn(a.y, b.x))};
}

struct RenderArgs {
  IpGeom g;
  const int32_t *slot;
  const void *payload;
  int width, height, maxSteps;
  float res;
  double hstep, invW, invH, aspect, zoom;
  RV camPos, lookAt, sun, color;
  float domMin[3], domMax[3];
  uint8_t *out;
};

// MtCubicBSplineWeights1D (src/mtool.h:344-362), each operation rounded in source order
__device__ __forceinline__ void bspline3(float t, float w[4], float d[4]) {
  const float s = __fsub_rn(1.0f, t), c6 = 1.0f / 6.0f, c23 = 2.0f / 3.0f;
  w[0] = __fmul_rn(__fmul_rn(__fmul_rn(c6, s), s), s);
  w[1] = __fsub_rn(c23, __fmul_rn(__fmul_rn(__fmul_rn(0.5f, t), t), __fsub_rn(2.0f, t)));
  w[2] = __fsub_rn(c23, __fmul_rn(__fmul_rn(__fmul_rn(0.5f, s), s), __fadd_rn(1.0f, t)));
  w[3] = __fmul_rn(__fmul_rn(__fmul_rn(c6, t), t), t);
  d[0] = __fdiv_rn(__fmul_rn(-s, s), 2.0f);
  d[1] = __fsub_rn(__fmul_rn(__fmul_rn(0.5f, t), t), __fmul_rn(__fmul_rn(1.0f, __fsub_rn(2.0f, t)), t));
  d[2] = __fsub_rn(__fmul_rn(__fmul_rn(1.0f, s), __fadd_rn(t, 1.0f)), __fmul_rn(__fmul_rn(0.5f, s), s));
  d[3] = __fdiv_rn(__fmul_rn(t, t), 2.0f);
}

template <typename T>
__device__ float density(const RenderArgs &a, const float q[3]) {
  const int s[3] = {a.g.sx, a.g.sy, a.g.sz};
  int ip[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    ip[k] = (int)floorf(q[k]);
    if (ip[k] < 0 || ip[k] > s[k] - 1) return 0.0f;
  }
  const int L = a.g.log2bs;
  const int64_t bid = (int64_t)(ip[0] >> L) + (int64_t)(ip[1] >> L) * a.g.nbx + (int64_t)(ip[2] >> L) * a.g.nxy;
  if (__ldg(a.slot + bid) < 0) return 0.0f;  // skip fast over empty blocks
  return ipValue<T>(a.g, a.slot, (const T *)a.payload, q[0], q[1], q[2]);
}

template <typename T>
__device__ RV gradient(const RenderArgs &a, RV p) {
  const float q[3] = {__fmul_rn(a.res, __double2float_rn(p.x)), __fmul_rn(a.res, __double2float_rn(p.y)),
                      __fmul_rn(a.res, __double2float_rn(p.z))};
#pragma unroll
  for (int k = 0; k < 3; k++)
    if (q[k] < a.domMin[k] || q[k] > a.domMax[k]) return {-0.0, -0.0, -0.0};
  const int s[3] = {a.g.sx, a.g.sy, a.g.sz};
  float w[3][4], d[3][4];
  int i0[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const float pos = __fsub_rn(q[k], 0.5f), pf = floorf(pos);
    i0[k] = (int)pf - 1;
    bspline3(__fsub_rn(pos, pf), w[k], d[k]);
  }
  const T *pay = (const T *)a.payload;
  float gx = 0.0f, gy = 0.0f, gz = 0.0f;
  for (int dz = 0; dz < 4; dz++) {
    const int z = min(max(i0[2] + dz, 0), s[2] - 1);
    for (int dy = 0; dy < 4; dy++) {
      const int y = min(max(i0[1] + dy, 0), s[1] - 1);
      const float wyz = __fmul_rn(w[2][dz], w[1][dy]);
      const float wgy = __fmul_rn(w[2][dz], d[1][dy]);
      const float wgz = __fmul_rn(d[2][dz], w[1][dy]);
#pragma unroll
      for (int dx = 0; dx < 4; dx++) {
        const int x = min(max(i0[0] + dx, 0), s[0] - 1);
        const float f = voxel(a.g, a.slot, pay, x, y, z);
        gx = __fmaf_rn(__fmul_rn(wyz, d[0][dx]), f, gx);
        gy = __fmaf_rn(__fmul_rn(wgy, w[0][dx]), f, gy);
        gz = __fmaf_rn(__fmul_rn(wgz, w[0][dx]), f, gz);
      }
    }
  }
  if (a.g.renderDens) {
    gx = __fmul_rn(gx, kU16ToF);
    gy = __fmul_rn(gy, kU16ToF);
    gz = __fmul_rn(gz, kU16ToF);
  }
  return {-(double)gx, -(double)gy, -(double)gz};
}

template <typename T>
__global__ void __launch_bounds__(128) kRender(RenderArgs a) {
  const int x = blockIdx.x * 16 + (threadIdx.x & 15), y = blockIdx.y * 8 + (threadIdx.x >> 4);
  if (x >= a.width || y >= a.height) return;
  const RV fwd = rnormalize(rsub(a.lookAt, a.camPos));
  const RV right = rnormalize(rcross(fwd, RV{0.0, 1.0, 0.0}));
  const RV up = rcross(right, fwd);
  const double ndcX = __dmul_rn(__dmul_rn(__fma_rn((double)__fadd_rn((float)x, 0.5f), a.invW, -0.5), 2.0), a.aspect);
  const double ndcY = __dmul_rn(__fma_rn(-(double)__fadd_rn((float)y, 0.5f), a.invH, 0.5), 2.0);
  const RV dir = rnormalize({__fma_rn(up.x, ndcY, __fma_rn(right.x, ndcX, __dmul_rn(fwd.x, a.zoom))),
                             __fma_rn(up.y, ndcY, __fma_rn(right.y, ndcX, __dmul_rn(fwd.y, a.zoom))),
                             __fma_rn(up.z, ndcY, __fma_rn(right.z, ndcX, __dmul_rn(fwd.z, a.zoom)))});
  const RV inc = {__dmul_rn(dir.x, a.hstep), __dmul_rn(dir.y, a.hstep), __dmul_rn(dir.z, a.hstep)};
  const int s[3] = {a.g.sx, a.g.sy, a.g.sz};
  const double incv[3] = {inc.x, inc.y, inc.z};
  RV pos = a.camPos, prevPos = a.camPos, hitPos = a.camPos;
  float q[3] = {__fmul_rn(a.res, __double2float_rn(pos.x)), __fmul_rn(a.res, __double2float_rn(pos.y)),
                __fmul_rn(a.res, __double2float_rn(pos.z))};
  float prev = density<T>(a, q);
  bool hit = false;
  for (int step = 0; step < a.maxSteps; step++) {
    pos = {__dadd_rn(pos.x, inc.x), __dadd_rn(pos.y, inc.y), __dadd_rn(pos.z, inc.z)};
    q[0] = __fmul_rn(a.res, __double2float_rn(pos.x));
    q[1] = __fmul_rn(a.res, __double2float_rn(pos.y));
    q[2] = __fmul_rn(a.res, __double2float_rn(pos.z));
    bool gone = false;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const float f = floorf(q[k]);
      gone |= (f < 0.0f && incv[k] <= 0.0) || (f > (float)(s[k] - 1) && incv[k] >= 0.0);
    }
    if (gone) break;  // outside and moving away: the density stays 0
    const float d = density<T>(a, q);
    if (prev < 0.5f && d >= 0.5f) {
      const double t = __ddiv_rn(__dsub_rn(0.5, (double)prev), __dsub_rn((double)d, (double)prev));
      hitPos = {__fma_rn(__dsub_rn(pos.x, prevPos.x), t, prevPos.x),
                __fma_rn(__dsub_rn(pos.y, prevPos.y), t, prevPos.y),
                __fma_rn(__dsub_rn(pos.z, prevPos.z), t, prevPos.z)};
      hit = true;
      break;
    }
    prev = d;
    prevPos = pos;
  }
  uint8_t rgb[3] = {0, 0, 0};
  if (hit) {
    const RV nrm = rnormalize(gradient<T>(a, hitPos));
    const RV ld = rnormalize(rsub(a.sun, hitPos));
    double diff = rdot(nrm, ld);
    diff = diff > 0.0 ? diff : 0.0;
    const double col[3] = {a.color.x, a.color.y, a.color.z};
#pragma unroll
    for (int k = 0; k < 3; k++) {
      double v = __dmul_rn(col[k], diff);
      v = v < 0.0 ? 0.0 : v > 1.0 ? 1.0 : v;
      rgb[k] = (uint8_t)(int)__fma_rn(v, 255.0, 0.5);
    }
  }
  uint8_t *o = a.out + ((int64_t)y * a.width + x) * 3;
  o[0] = rgb[0];
  o[1] = rgb[1];
  o[2] = rgb[2];
}

}  // namespace

}  // namespace msbg

using namespace msbg;

extern "C" int msbg_gpu_render(msbg_gpu_ctx *ctx, int chan, int width, int height, const msbg_gpu_camera *cam,
                               uint8_t *dRGB) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  if (width <= 0 || height <= 0 || height > 65535 * 8 || (int64_t)width * height > ((int64_t)1 << 31) || !cam ||
      !dRGB)
    return fail(ctx, MSBG_GPU_ERR_ARG, "render: bad image size or null argument");
  if (chan < 0 || chan >= kMaxChannels || !ctx->ch[chan].exists)
    return fail(ctx, MSBG_GPU_ERR_ARG, "channel %d does not exist", chan);
  if (!ctx->layoutValid) return fail(ctx, MSBG_GPU_ERR_STATE, "no block layout: call set_refinement_map");
  const Channel &c = ctx->ch[chan];
  RenderArgs a;
  a.g.sx = ctx->sx; a.g.sy = ctx->sy; a.g.sz = ctx->sz;
  a.g.log2bs = ctx->log2bs;
  a.g.nbx = ctx->nbx;
  a.g.nxy = (int64_t)ctx->nbx * ctx->nby;
  a.g.vpb = ctx->voxPerBlock;
  a.g.po = 0.5f;
  a.g.dirichlet = a.g.dirichletOld = 0;
  a.g.renderDens = c.storage == MSBG_GPU_U16;
  a.slot = ctx->dSlot;
  a.payload = c.d;
  a.width = width;
  a.height = height;
  const int res = ctx->sx > ctx->sy ? (ctx->sx > ctx->sz ? ctx->sx : ctx->sz) : (ctx->sy > ctx->sz ? ctx->sy : ctx->sz);
  a.res = (float)res;
  a.hstep = 1.0 / (double)res;
  a.maxSteps = (int)(2.0 / a.hstep);
  a.invW = 1.0 / (double)width;
  a.invH = 1.0 / (double)height;
  a.aspect = (double)width / (double)height;
  a.zoom = cam->zoom;
  a.camPos = {cam->pos[0], cam->pos[1], cam->pos[2]};
  a.lookAt = {cam->lookAt[0], cam->lookAt[1], cam->lookAt[2]};
  a.sun = {cam->sun[0], cam->sun[1], cam->sun[2]};
  a.color = {cam->color[0], cam->color[1], cam->color[2]};
  for (int k = 0; k < 3; k++) {
    a.domMin[k] = ctx->domMin[k];
    a.domMax[k] = ctx->domMax[k];
  }
  a.out = dRGB;
  const dim3 grid((unsigned)((width + 15) / 16), (unsigned)((height + 7) / 8));
  switch (c.storage) {
    case MSBG_GPU_F32: MSBG_LAUNCH(ctx, kRender<float>, grid, 128, 0, a); break;
    case MSBG_GPU_F16: MSBG_LAUNCH(ctx, kRender<__half>, grid, 128, 0, a); break;
    case MSBG_GPU_U16: MSBG_LAUNCH(ctx, kRender<uint16_t>, grid, 128, 0, a); break;
    default: return fail(ctx, MSBG_GPU_ERR_UNSUPPORTED, "render: FP64 channels are not supported");
  }
  return MSBG_GPU_OK;
}
