// Per-voxel arithmetic of applyChannelPdeFast (src/msbg4.cpp:559-825), shared by
// the gather kernel (sweep.cu) and the streaming colored kernel (sweep_color.cu).
#pragma once

#include "internal.cuh"

namespace msbg {

enum { K_MCF = 4, K_JACOBI = 17, K_PM_JACOBI = 15, K_PM = 14, K_DIFF = 3, K_LAPL = 1 };
enum { FK_CLAMP = 256 };  // sweep kernel flag: results clamped to [0,1]

struct SweepParams {
  int kind, constr01;
  float dt, anisAlpha;
};

// Correctly rounded scalar ops; no contraction, so results follow the written
// expression order exactly (the reference's and the CPU restatement's).
template <typename R> struct Op;
template <> struct Op<float> {
  static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
  static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
  static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
  static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
  static __device__ __forceinline__ float sqrt_(float a) { return __fsqrt_rn(a); }
};
template <> struct Op<double> {
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
  static __device__ __forceinline__ double sqrt_(double a) { return __dsqrt_rn(a); }
};

// Mean curvature flow update, laplTyp 4 (src/msbg4.cpp:559-637), in the
// reference's expression order.  F(dx,dy,dz) reads the neighbourhood.
template <typename R, typename P>
__device__ __forceinline__ R mcfExact(const P &F, R dt) {
  using O = Op<R>;
  const R h = (R)0.5, two = (R)2;
  const R f0 = F(0, 0, 0), f1 = F(-1, 0, 0), f2 = F(1, 0, 0), f3 = F(0, -1, 0), f4 = F(0, 1, 0),
          f5 = F(0, 0, -1), f6 = F(0, 0, 1);
  const R fx = O::mul(h, O::sub(f2, f1)), fy = O::mul(h, O::sub(f4, f3)), fz = O::mul(h, O::sub(f6, f5));
  const R f02 = O::mul(two, f0);
  const R fxx = O::sub(O::add(f1, f2), f02), fyy = O::sub(O::add(f3, f4), f02),
          fzz = O::sub(O::add(f5, f6), f02);
  const R fy_r = O::mul(O::sub(F(1, 1, 0), F(1, -1, 0)), h);
  const R fy_l = O::mul(O::sub(F(-1, 1, 0), F(-1, -1, 0)), h);
  const R fz_r = O::mul(O::sub(F(1, 0, 1), F(1, 0, -1)), h);
  const R fz_l = O::mul(O::sub(F(-1, 0, 1), F(-1, 0, -1)), h);
  const R fz_u = O::mul(O::sub(F(0, 1, 1), F(0, 1, -1)), h);
  const R fz_d = O::mul(O::sub(F(0, -1, 1), F(0, -1, -1)), h);
  const R fyx = O::mul(O::sub(fy_r, fy_l), h), fzx = O::mul(O::sub(fz_r, fz_l), h),
          fzy = O::mul(O::sub(fz_u, fz_d), h);
  const R xx = O::mul(fx, fx), yy = O::mul(fy, fy), zz = O::mul(fz, fz);
  R H = O::add(O::add(O::mul(O::add(yy, zz), fxx), O::mul(O::add(xx, zz), fyy)), O::mul(O::add(xx, yy), fzz));
  const R cross = O::add(O::add(O::mul(O::mul(fx, fy), fyx), O::mul(O::mul(fx, fz), fzx)),
                         O::mul(O::mul(fy, fz), fzy));
  H = O::sub(H, O::mul(two, cross));
  const R g2 = O::add(O::add(xx, yy), zz);
  H = g2 > (R)1e-7f ? O::div(H, g2) : (R)0;
  R D = O::mul(dt, H);
  D = D < (R)-0.1f ? (R)-0.1f : D;
  D = D > (R)0.1f ? (R)0.1f : D;
  return O::add(f0, D);
}

// 7-point kernels (src/msbg4.cpp:681-805), reference expression order.
template <typename R, typename P>
__device__ __forceinline__ R stencil7(const P &F, const SweepParams &g) {
  using O = Op<R>;
  const R dt = (R)g.dt;
  const R phi = F(0, 0, 0);
  const R F1 = F(-1, 0, 0), F2 = F(1, 0, 0), F3 = F(0, -1, 0), F4 = F(0, 1, 0), F5 = F(0, 0, -1),
          F6 = F(0, 0, 1);
  switch (g.kind) {
    case K_JACOBI: {
      const R s6 = O::add(O::add(O::add(O::add(O::add(F1, F2), F3), F4), F5), F6);
      return O::div(O::add(phi, O::mul(dt, s6)), O::add((R)1, O::mul(dt, (R)6)));
    }
    case K_DIFF: {
      const R s6 = O::add(O::add(O::add(O::add(O::add(F1, F2), F3), F4), F5), F6);
      const R S = O::mul((R)1 / (R)6, s6);
      return O::add(phi, O::mul(dt, O::sub(S, phi)));
    }
    case K_LAPL: {
      const R s6 = O::add(O::add(O::add(O::add(O::add(F1, F2), F3), F4), F5), F6);
      const R L = O::sub(s6, O::mul((R)6, phi));
      const R GX = O::mul((R)0.5, O::sub(F2, F1)), GY = O::mul((R)0.5, O::sub(F4, F3)),
              GZ = O::mul((R)0.5, O::sub(F6, F5));
      const R G = O::sqrt_(O::add(O::add(O::mul(GX, GX), O::mul(GY, GY)), O::mul(GZ, GZ)));
      return O::add(phi, O::mul(O::mul(dt, L), G));
    }
    default: {  // K_PM_JACOBI / K_PM, anisAlpha > 0 (src/msbg4.cpp:738-790)
      const R a = (R)g.anisAlpha;
      const R fn[6] = {F1, F2, F3, F4, F5, F6};
      R sum = 0, wsum = 0, dsum = 0;
#pragma unroll
      for (int k = 0; k < 6; k++) {
        const R gk = O::sub(fn[k], phi);
        const R ag = gk < (R)0 ? -gk : gk;
        const R t = O::div(ag, a);
        const R Gk = O::div((R)1, O::add((R)1, O::mul(t, t)));
        sum = O::add(sum, O::mul(Gk, fn[k]));
        wsum = O::add(wsum, Gk);
        dsum = O::add(dsum, O::mul(Gk, gk));
      }
      if (g.kind == K_PM_JACOBI) return O::div(O::add(phi, O::mul(dt, sum)), O::add((R)1, O::mul(dt, wsum)));
      return O::add(phi, O::mul(dt, dsum));
    }
  }
}

// Fast MCF of four x-consecutive voxels from a register window W[r][c]
// (r: y-1..y+1, c: x-1..x+4 of planes z-1 / z / z+1).  Re-associated with fused
// multiply-adds and shared central differences:
//   D_y(c) = P0(c,y+1) - P0(c,y-1), D_z(c) = Pp(c,y) - Pm(c,y)
//   gx = P0(c+1) - P0(c-1),  gy = D_y(c), gz = D_z(c)            (= 2 f_x ...)
//   Gyx = D_y(c+1) - D_y(c-1), Gzx = D_z(c+1) - D_z(c-1),
//   Gzy = (Pp(c,y+1) - Pm(c,y+1)) - (Pp(c,y-1) - Pm(c,y-1))        (= 4 f_xy ...)
//   H = [ (gy^2+gz^2) fxx + (gx^2+gz^2) fyy + (gx^2+gy^2) fzz
//         - (gx gy Gyx + gx gz Gzx + gy gz Gzy) / 2 ] / |g|^2
// which is the reference's H with |grad f|^2 = |g|^2 / 4 (threshold 4e-7).
__device__ __forceinline__ float2 pr(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, neg2(b)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// What the z-marching kernel keeps of one plane of a thread's neighbourhood
// (rows y-1..y+1, columns x-1..x+4 of the strip x..x+3).  The generic form keeps
// the raw values; the fast forms keep per-plane summaries, computed once when the
// plane is read, so fewer values stay live across the three planes.
struct PlaneRaw {
  float w[3][6];
};
// MCF: centre row, y-difference (row y+1 - row y-1) and y-sum (centre columns).
struct PlaneMcf {
  float r1[6], dy[6], sy[4];
};
// Jacobi: centre row and y-sum (centre columns).
struct PlaneJac {
  float r1[6], sy[4];
};

// Reads one plane from the FP32 ring: row0 = row y-1 at column x-1; rows RS apart.
template <int RS>
__device__ __forceinline__ void loadPlane(const float *row0, PlaneRaw &P) {
#pragma unroll
  for (int r = 0; r < 3; r++) {
    const float *row = row0 + r * RS;
    const float4 m = *reinterpret_cast<const float4 *>(row + 1);
    P.w[r][0] = row[0]; P.w[r][1] = m.x; P.w[r][2] = m.y; P.w[r][3] = m.z; P.w[r][4] = m.w; P.w[r][5] = row[5];
  }
}
template <int RS>
__device__ __forceinline__ void loadRow1(const float *row0, float (&r1)[6]) {
  const float *row = row0 + RS;
  const float4 m = *reinterpret_cast<const float4 *>(row + 1);
  r1[0] = row[0]; r1[1] = m.x; r1[2] = m.y; r1[3] = m.z; r1[4] = m.w; r1[5] = row[5];
}
template <int RS>
__device__ __forceinline__ void loadPlane(const float *row0, PlaneMcf &P) {
  loadRow1<RS>(row0, P.r1);
  const float4 u = *reinterpret_cast<const float4 *>(row0 + 1);
  const float4 v = *reinterpret_cast<const float4 *>(row0 + 2 * RS + 1);
  const float2 d01 = sub2(pr(v.x, v.y), pr(u.x, u.y)), d23 = sub2(pr(v.z, v.w), pr(u.z, u.w));
  const float2 s01 = add2(pr(u.x, u.y), pr(v.x, v.y)), s23 = add2(pr(u.z, u.w), pr(v.z, v.w));
  P.dy[0] = row0[2 * RS] - row0[0];
  P.dy[1] = d01.x; P.dy[2] = d01.y; P.dy[3] = d23.x; P.dy[4] = d23.y;
  P.dy[5] = row0[2 * RS + 5] - row0[5];
  P.sy[0] = s01.x; P.sy[1] = s01.y; P.sy[2] = s23.x; P.sy[3] = s23.y;
}
template <int RS>
__device__ __forceinline__ void loadPlane(const float *row0, PlaneJac &P) {
  loadRow1<RS>(row0, P.r1);
  const float4 u = *reinterpret_cast<const float4 *>(row0 + 1);
  const float4 v = *reinterpret_cast<const float4 *>(row0 + 2 * RS + 1);
  const float2 s01 = add2(pr(u.x, u.y), pr(v.x, v.y)), s23 = add2(pr(u.z, u.w), pr(v.z, v.w));
  P.sy[0] = s01.x; P.sy[1] = s01.y; P.sy[2] = s23.x; P.sy[3] = s23.y;
}

// 1/x from the hardware's approximate reciprocal (PTX rcp.approx.ftz.f32).
__device__ __forceinline__ float rcpApprox(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Fast MCF of the strip's four voxels.  The voxels go through the arithmetic in
// pairs (columns 1,2 and 3,4) on the packed FP32 pipe (add/mul/fma.rn.f32x2);
// differences along x (whose operands straddle the pairs), the reciprocal and the
// clamps stay scalar.  With central differences g = 2 grad f and the plane
// summaries (Dz = centre row of z+1 - that of z-1):
//   gx = f(x+1) - f(x-1), gy = dy0, gz = Dz
//   Gyx = dy0(x+1) - dy0(x-1), Gzx = Dz(x+1) - Dz(x-1), Gzy = dy(z+1) - dy(z-1)
//   H = [ (gy^2+gz^2) fxx + (gx^2+gz^2) fyy + (gx^2+gy^2) fzz
//         - (gx gy Gyx + gx gz Gzx + gy gz Gzy) / 2 ] / |g|^2
// which is the reference's H with |grad f|^2 = |g|^2 / 4 (threshold 4e-7).
template <bool CLAMP01>
__device__ __forceinline__ void mcfFastStrip(const PlaneMcf &Pm, const PlaneMcf &P0, const PlaneMcf &Pp,
                                             float dt, float out[4]) {
  float Dz[6];
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const int c = 1 + 2 * h;
    const float2 dz = sub2(pr(Pp.r1[c], Pp.r1[c + 1]), pr(Pm.r1[c], Pm.r1[c + 1]));
    Dz[c] = dz.x; Dz[c + 1] = dz.y;
  }
  Dz[0] = Pp.r1[0] - Pm.r1[0]; Dz[5] = Pp.r1[5] - Pm.r1[5];
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const int c = 1 + 2 * h;
    const float *w = P0.r1, *Dy = P0.dy;
    const float2 f0 = pr(w[c], w[c + 1]);
    const float2 gx = pr(w[c + 1] - w[c - 1], w[c + 2] - w[c]);
    const float2 gy = pr(Dy[c], Dy[c + 1]), gz = pr(Dz[c], Dz[c + 1]);
    // second differences as s - 2 f0 with s the neighbour sums; with A = g2 - xx,
    // B = g2 - yy, C = g2 - zz the first numerator term is
    //   A fxx + B fyy + C fzz = g2 (sx + sy + sz - 4 f0) - (xx sx + yy sy + zz sz)
    const float2 sx = pr(w[c - 1] + w[c + 1], w[c] + w[c + 2]);
    const float2 sy = pr(P0.sy[c - 1], P0.sy[c]);
    const float2 sz = add2(pr(Pm.r1[c], Pm.r1[c + 1]), pr(Pp.r1[c], Pp.r1[c + 1]));
    const float2 Gyx = pr(Dy[c + 1] - Dy[c - 1], Dy[c + 2] - Dy[c]);
    const float2 Gzx = pr(Dz[c + 1] - Dz[c - 1], Dz[c + 2] - Dz[c]);
    const float2 Gzy = sub2(pr(Pp.dy[c], Pp.dy[c + 1]), pr(Pm.dy[c], Pm.dy[c + 1]));
    const float2 xx = mul2(gx, gx), yy = mul2(gy, gy), zz = mul2(gz, gz);
    const float2 g2 = add2(add2(xx, yy), zz);
    const float2 L = fma2(pr(-4.0f, -4.0f), f0, add2(add2(sx, sy), sz));
    const float2 T3 = fma2(xx, sx, fma2(yy, sy, mul2(zz, sz)));
    const float2 n1 = fma2(g2, L, neg2(T3));
    const float2 n2 = fma2(gx, fma2(gy, Gyx, mul2(gz, Gzx)), mul2(mul2(gy, gz), Gzy));
    const float2 Hn = fma2(pr(-0.5f, -0.5f), n2, n1);
    const float2 r = pr(g2.x > 4e-7f ? rcpApprox(g2.x) : 0.0f, g2.y > 4e-7f ? rcpApprox(g2.y) : 0.0f);
    const float2 Hr = mul2(Hn, mul2(r, pr(dt, dt)));
    const float D0 = fminf(fmaxf(Hr.x, -0.1f), 0.1f), D1 = fminf(fmaxf(Hr.y, -0.1f), 0.1f);
    out[2 * h] = CLAMP01 ? __saturatef(f0.x + D0) : f0.x + D0;
    out[2 * h + 1] = CLAMP01 ? __saturatef(f0.y + D1) : f0.y + D1;
  }
}

// Fast Jacobi diffusion of four x-consecutive voxels: (phi + dt s6) * 1/(1 + 6 dt),
// the reference's division replaced by a multiplication with the reciprocal.
template <bool CLAMP01>
__device__ __forceinline__ void jacobiFastStrip(const PlaneJac &Pm, const PlaneJac &P0, const PlaneJac &Pp,
                                                float dt, float out[4]) {
  const float inv = 1.0f / fmaf(6.0f, dt, 1.0f);
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const int c = 1 + 2 * h;
    const float *w = P0.r1;
    const float2 sxy = add2(pr(w[c - 1] + w[c + 1], w[c] + w[c + 2]), pr(P0.sy[c - 1], P0.sy[c]));
    const float2 s6 = add2(sxy, add2(pr(Pm.r1[c], Pm.r1[c + 1]), pr(Pp.r1[c], Pp.r1[c + 1])));
    const float2 v = mul2(fma2(pr(dt, dt), s6, pr(w[c], w[c + 1])), pr(inv, inv));
    out[2 * h] = CLAMP01 ? __saturatef(v.x) : v.x;
    out[2 * h + 1] = CLAMP01 ? __saturatef(v.y) : v.y;
  }
}

// Four voxels of a strip, any kernel, from the register window, in the
// reference's operation order.
__device__ __forceinline__ void computeStrip(const float Pm[3][6], const float P0[3][6],
                                             const float Pp[3][6], const SweepParams &p,
                                             float out[4]) {
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int c = i + 1;
    auto F = [&](int dx, int dy, int dz) -> float {
      const float(*W)[6] = dz < 0 ? Pm : dz > 0 ? Pp : P0;
      return W[1 + dy][c + dx];
    };
    float v = p.kind == K_MCF ? mcfExact<float>(F, p.dt) : stencil7<float>(F, p);
    if (p.constr01) {
      v = v > 0.0f ? v : 0.0f;
      v = v < 1.0f ? v : 1.0f;
    }
    out[i] = v;
  }
}

// bids / colorStart: the blocks of each colour (colour c: bids[colorStart[c] ..
// colorStart[c+1]-1]); the context's full colour lists, or a caller's subset.
int colorSweepRun(msbg_gpu_ctx *ctx, Channel &c, bool exact, bool color8, int nIter, const SweepParams &p,
                  const int32_t *bids, const int *colorStart);

}  // namespace msbg
