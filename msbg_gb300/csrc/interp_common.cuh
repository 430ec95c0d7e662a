// Trilinear interpolation of one point on the value blocks, shared by the G2P kernel
// (interpolate.cu) and the ray-march renderer (render.cu).
//
// SparseGrid<float>::interpolateFloatFast (src/sbg.h:4623-4792) and
// SparseGrid<uint16_t>::interpolateUint16ToFloatFast (src/sbg.h:4920-5032):
//  - pos = p - 0.5 (not with OPT_IPCORNER); i = floor(pos); t = pos - i.
//  - Corner c = (c&1, (c>>1)&1, c>>2) is added to i and read as a float: FP32 as stored,
//    uint16 unscaled, FP16 widened.  A block without payload reads the empty value, 0.
//  - lerp(t, a, b) = fma(b - a, t, a) (vlerp_ps, src/vectorclass_util.h:143-146), along x
//    for the pairs (0,1) (2,3) (4,5) (6,7), then along y, then along z.
// Border path, for points with i outside [0, s-2] on some axis: interpolateGen0<IP_LINEAR>
// (src/sbg.h:3109-3246).
//  - Corner coordinates are clamped to the domain.  With OPT_IPBC_DIRICHLET a corner with
//    a clamped coordinate reads the empty value; with OPT_IPBC_DIRICHLET_OLD the result
//    is the empty value.
//  - Interpolate1D (src/sbg.h:2934-2940) lerps in the same order, p1*t + p0*(1-t).  The
//    reference's build (-O3 -ffast-math on FMA hardware) evaluates it as
//    fma(p1, t, p0*(1-t)), the form used here.
// renderDens scales a uint16 channel's value by 1/65535 (interpolateRenderDensity,
// src/msbg.h:478-484).
#pragma once

#include "internal.cuh"

namespace msbg {

struct IpGeom {
  int sx, sy, sz;
  int log2bs;
  int nbx;
  int64_t nxy;  // nbx * nby
  int64_t vpb;  // bs^3
  float po;     // half-voxel shift (0 with OPT_IPCORNER)
  int dirichlet, dirichletOld, renderDens;
};

template <typename T> __device__ __forceinline__ float rawLoad(const T *p);
template <> __device__ __forceinline__ float rawLoad<float>(const float *p) { return __ldg(p); }
template <> __device__ __forceinline__ float rawLoad<uint16_t>(const uint16_t *p) {
  return (float)__ldg(p);
}
template <> __device__ __forceinline__ float rawLoad<__half>(const __half *p) {
  return __half2float(__ldg(p));
}

__device__ __forceinline__ float ipLerp(float t, float a, float b) {
  return __fmaf_rn(__fsub_rn(b, a), t, a);
}
__device__ __forceinline__ float ipLin(float p0, float p1, float t) {
  return __fmaf_rn(p1, t, __fmul_rn(p0, __fsub_rn(1.0f, t)));
}

// Value of voxel (x, y, z), which must lie inside the domain.
template <typename T>
__device__ __forceinline__ float voxel(const IpGeom &g, const int32_t *__restrict__ slot,
                                       const T *__restrict__ payload, int x, int y, int z) {
  const int L = g.log2bs, m = (1 << L) - 1;
  const int64_t bid = (int64_t)(x >> L) + (int64_t)(y >> L) * g.nbx + (int64_t)(z >> L) * g.nxy;
  const int32_t s = __ldg(slot + bid);
  if (s < 0) return 0.0f;
  return rawLoad(payload + (int64_t)s * g.vpb + ((((z & m) << L) + (y & m)) << L) + (x & m));
}

// The interpolant at point (x, y, z) in voxel units (voxel centres at i + 0.5).
template <typename T>
__device__ __forceinline__ float ipValue(const IpGeom &g, const int32_t *__restrict__ slot,
                                         const T *__restrict__ payload, float x, float y, float z) {
  const float px = __fsub_rn(x, g.po), py = __fsub_rn(y, g.po), pz = __fsub_rn(z, g.po);
  const float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
  const int ix = (int)fx, iy = (int)fy, iz = (int)fz;
  const float tx = __fsub_rn(px, fx), ty = __fsub_rn(py, fy), tz = __fsub_rn(pz, fz);
  float val;
  if ((unsigned)ix < (unsigned)(g.sx - 1) && (unsigned)iy < (unsigned)(g.sy - 1) &&
      (unsigned)iz < (unsigned)(g.sz - 1)) {
    const int L = g.log2bs, m = (1 << L) - 1, bs = 1 << L;
    float c[8];
    if (((ix & m) != m) & ((iy & m) != m) & ((iz & m) != m)) {
      // all 8 corners in one block
      const int64_t bid = (int64_t)(ix >> L) + (int64_t)(iy >> L) * g.nbx + (int64_t)(iz >> L) * g.nxy;
      const int32_t s = __ldg(slot + bid);
      if (s < 0) {
#pragma unroll
        for (int i = 0; i < 8; i++) c[i] = 0.0f;
      } else {
        const T *p = payload + (int64_t)s * g.vpb + ((((iz & m) << L) + (iy & m)) << L) + (ix & m);
#pragma unroll
        for (int i = 0; i < 8; i++) c[i] = rawLoad(p + (i & 1) + ((i >> 1) & 1) * bs + (i >> 2) * bs * bs);
      }
    } else {
#pragma unroll
      for (int i = 0; i < 8; i++)
        c[i] = voxel(g, slot, payload, ix + (i & 1), iy + ((i >> 1) & 1), iz + (i >> 2));
    }
    const float a0 = ipLerp(tx, c[0], c[1]), a1 = ipLerp(tx, c[2], c[3]);
    const float a2 = ipLerp(tx, c[4], c[5]), a3 = ipLerp(tx, c[6], c[7]);
    const float b0 = ipLerp(ty, a0, a1), b1 = ipLerp(ty, a2, a3);
    val = ipLerp(tz, b0, b1);
  } else if (g.dirichletOld) {
    val = 0.0f;
  } else {
    float c[8];
#pragma unroll
    for (int i = 0; i < 8; i++) {
      const int x = ix + (i & 1), y = iy + ((i >> 1) & 1), z = iz + (i >> 2);
      const int cx = min(max(x, 0), g.sx - 1), cy = min(max(y, 0), g.sy - 1), cz = min(max(z, 0), g.sz - 1);
      const bool clipped = (cx != x) | (cy != y) | (cz != z);
      c[i] = (g.dirichlet && clipped) ? 0.0f : voxel(g, slot, payload, cx, cy, cz);
    }
    const float a0 = ipLin(c[0], c[1], tx), a1 = ipLin(c[2], c[3], tx);
    const float a2 = ipLin(c[4], c[5], tx), a3 = ipLin(c[6], c[7], tx);
    const float b0 = ipLin(a0, a1, ty), b1 = ipLin(a2, a3, ty);
    val = ipLin(b0, b1, tz);
  }
  if (g.renderDens) val = __fmul_rn(val, kU16ToF);
  return val;
}

}  // namespace msbg
