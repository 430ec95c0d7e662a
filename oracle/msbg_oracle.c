/*
 * CPU restatement of the MSBG hot path -- test infrastructure only (the checker
 * for the GPU library, never linked into it).  See msbg_oracle.h for the data
 * layout.  Built with -ffp-contract=off so float expressions round exactly as
 * written; the GPU library's parity kernels use the same expression order with
 * explicitly rounded operations, so FP32 results compare bit for bit.
 *
 * Parity of this restatement with the reference itself is pinned by the tests,
 * which run the reference library compiled from its own sources (oracle/_ref)
 * on the same seeded inputs.
 */
#include "msbg_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* conversions                                                               */
/* ------------------------------------------------------------------------ */

/* IEEE binary16 round-to-nearest-even conversion (bit manipulation). */
uint16_t orc_f32_to_f16(float f) {
  uint32_t x;
  memcpy(&x, &f, 4);
  uint32_t sign = (x >> 16) & 0x8000u;
  uint32_t absx = x & 0x7fffffffu;
  if (absx >= 0x7f800000u) { /* inf or nan */
    return (uint16_t)(sign | 0x7c00u | (absx > 0x7f800000u ? 0x200u : 0u));
  }
  if (absx >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u); /* rounds to inf */
  if (absx < 0x38800000u) {                                   /* subnormal or zero */
    if (absx < 0x33000000u) return (uint16_t)sign;             /* < 2^-25: rounds to 0 */
    uint32_t e = absx >> 23;
    uint32_t m = (absx & 0x7fffffu) | 0x800000u;
    uint32_t shift = 126u - e; /* 14..24 */
    uint32_t q = m >> shift;
    uint32_t rem = m & ((1u << shift) - 1u);
    uint32_t half = 1u << (shift - 1u);
    if (rem > half || (rem == half && (q & 1u))) q++;
    return (uint16_t)(sign | q);
  }
  uint32_t e = (absx >> 23) - 112u;
  uint32_t m = absx & 0x7fffffu;
  uint32_t q = (e << 10) | (m >> 13);
  uint32_t rem = m & 0x1fffu;
  if (rem > 0x1000u || (rem == 0x1000u && (q & 1u))) q++;
  return (uint16_t)(sign | q);
}

float orc_f16_to_f32(uint16_t h) {
  uint32_t sign = ((uint32_t)h & 0x8000u) << 16;
  uint32_t e = ((uint32_t)h >> 10) & 0x1fu;
  uint32_t m = (uint32_t)h & 0x3ffu;
  uint32_t x;
  if (e == 0) {
    if (m == 0) {
      x = sign;
    } else { /* subnormal */
      float v = (float)m * (1.0f / 16777216.0f);
      memcpy(&x, &v, 4);
      x |= sign;
    }
  } else if (e == 31) {
    x = sign | 0x7f800000u | (m << 13);
  } else {
    x = sign | ((e + 112u) << 23) | (m << 13);
  }
  float f;
  memcpy(&f, &x, 4);
  return f;
}

/* uint16 density: load v*(1/65535) (src/sbg.h:225-247); stores either
 * round-half-even (the SIMD sweep store, src/sbg.h:343-351) or round-half-away
 * (the scalar store used by splat/finalize, src/sbg.h:271-296). */
static const float kU16ToF = 1.0f / 65535.0f;
static inline uint16_t u16_rne(float f) { return (uint16_t)nearbyintf(f * 65535.0f); }
static inline uint16_t u16_rha(float f) { return (uint16_t)roundf(f * 65535.0f); }

static inline double load_val(const orc_grid *g, const void *p, int64_t i) {
  switch (g->storage) {
    case ORC_F32: return ((const float *)p)[i];
    case ORC_U16: return (float)((const uint16_t *)p)[i] * kU16ToF;
    case ORC_F16: return orc_f16_to_f32(((const uint16_t *)p)[i]);
    default: return ((const double *)p)[i];
  }
}

static inline size_t elem_bytes(int storage) {
  return storage == ORC_F32 ? 4 : storage == ORC_F64 ? 8 : 2;
}

void orc_grid_init(orc_grid *g, int sx, int sy, int sz, int bsx, int storage) {
  g->sx = sx; g->sy = sy; g->sz = sz; g->bsx = bsx;
  g->nbx = sx / bsx; g->nby = sy / bsx; g->nbz = sz / bsx;
  g->storage = storage;
  g->emptyValue = 0.0;
}

static inline int ilog2(int v) { int l = 0; while ((1 << l) < v) l++; return l; }
static inline int imin(int a, int b) { return a < b ? a : b; }
static inline int imax(int a, int b) { return a > b ? a : b; }

/* Domain limits of MultiresSparseGrid::isInDomainRange: (0,s) shrunk by 0.005 and
 * snapped to the 24-bit particle quantisation grid (src/sbg.cpp:262-316,
 * src/msbgcell.h:74, src/msbgcell.h:138). */
static float quant24(float x) {
  double scale = ((1 << 24) - 1) * (1.0 / 32768.0);
  return (float)((int32_t)floor(scale * x + 0.5) / scale);
}

static inline int point_valid(const orc_grid *g, float px, float py, float pz, float *dmin,
                              float *dmax) {
  if (px < dmin[0] || px > dmax[0] || py < dmin[1] || py > dmax[1] || pz < dmin[2] ||
      pz > dmax[2])
    return 0;
  int ix = (int)px, iy = (int)py, iz = (int)pz;
  return ix >= 0 && ix < g->sx && iy >= 0 && iy < g->sy && iz >= 0 && iz < g->sz;
}

static void domain_limits(const orc_grid *g, float *dmin, float *dmax) {
  const float beps = 0.005f;
  dmin[0] = quant24(0.0f + beps); dmax[0] = quant24((float)g->sx - beps);
  dmin[1] = quant24(0.0f + beps); dmax[1] = quant24((float)g->sy - beps);
  dmin[2] = quant24(0.0f + beps); dmax[2] = quant24((float)g->sz - beps);
}

/* ------------------------------------------------------------------------ */
/* marking / bucketing / levels                                              */
/* ------------------------------------------------------------------------ */

int64_t orc_mark_blocks(const orc_grid *g, const float *pts, int64_t n, float rScan,
                        int32_t *blockCount, uint8_t *valid) {
  float dmin[3], dmax[3];
  domain_limits(g, dmin, dmax);
  const float scale = 1.0f / (float)g->bsx, rs = rScan / (float)g->bsx;
  const int nbx = g->nbx, nby = g->nby, nbz = g->nbz;
  int64_t nValid = 0;
#pragma omp parallel for schedule(static) reduction(+ : nValid)
  for (int64_t i = 0; i < n; i++) {
    const float px = pts[3 * i], py = pts[3 * i + 1], pz = pts[3 * i + 2];
    if (!point_valid(g, px, py, pz, dmin, dmax)) { valid[i] = 0; continue; }
    valid[i] = 1;
    nValid++;
    const float bx = px * scale, by = py * scale, bz = pz * scale;
    const int x1 = imax((int)(bx - rs), 0), x2 = imin((int)(bx + rs), nbx - 1);
    const int y1 = imax((int)(by - rs), 0), y2 = imin((int)(by + rs), nby - 1);
    const int z1 = imax((int)(bz - rs), 0), z2 = imin((int)(bz + rs), nbz - 1);
    for (int k = z1; k <= z2; k++)
      for (int j = y1; j <= y2; j++)
        for (int l = x1; l <= x2; l++) {
#pragma omp atomic
          blockCount[(int64_t)k * nbx * nby + (int64_t)j * nbx + l]++;
        }
  }
  return nValid;
}

static inline int64_t own_block(const orc_grid *g, const float *p) {
  const int s = ilog2(g->bsx);
  const int ix = (int)p[0], iy = (int)p[1], iz = (int)p[2];
  return (int64_t)(iz >> s) * g->nbx * g->nby + (int64_t)(iy >> s) * g->nbx + (ix >> s);
}

void orc_bucket_points(const orc_grid *g, const float *pts, int64_t n, const uint8_t *valid,
                       int64_t *bucketStart, int64_t *bucketIdx) {
  const int64_t nB = (int64_t)g->nbx * g->nby * g->nbz;
  memset(bucketStart, 0, sizeof(int64_t) * (size_t)(nB + 1));
  for (int64_t i = 0; i < n; i++)
    if (valid[i]) bucketStart[own_block(g, pts + 3 * i) + 1]++;
  for (int64_t b = 0; b < nB; b++) bucketStart[b + 1] += bucketStart[b];
  int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (size_t)nB);
  memcpy(fill, bucketStart, sizeof(int64_t) * (size_t)nB);
  for (int64_t i = 0; i < n; i++)
    if (valid[i]) bucketIdx[fill[own_block(g, pts + 3 * i)]++] = i;
  free(fill);
}

void orc_band_levels(const orc_grid *g, const float *pts, int64_t n, const uint8_t *valid,
                     const float *rBand, int nBands, int nLevels, int32_t *levels) {
  const int64_t nB = (int64_t)g->nbx * g->nby * g->nbz;
  for (int64_t b = 0; b < nB; b++) levels[b] = nLevels - 1;
  const float scale = 1.0f / (float)g->bsx;
  for (int l = nBands - 1; l >= 0; l--) {
    const float rs = rBand[l] / (float)g->bsx;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
      if (!valid[i]) continue;
      const float bx = pts[3 * i] * scale, by = pts[3 * i + 1] * scale, bz = pts[3 * i + 2] * scale;
      const int x1 = imax((int)(bx - rs), 0), x2 = imin((int)(bx + rs), g->nbx - 1);
      const int y1 = imax((int)(by - rs), 0), y2 = imin((int)(by + rs), g->nby - 1);
      const int z1 = imax((int)(bz - rs), 0), z2 = imin((int)(bz + rs), g->nbz - 1);
      for (int k = z1; k <= z2; k++)
        for (int j = y1; j <= y2; j++)
          for (int m = x1; m <= x2; m++) {
            int32_t *lv = &levels[(int64_t)k * g->nbx * g->nby + (int64_t)j * g->nbx + m];
            if (*lv > l) {
#pragma omp atomic write
              *lv = l;
            }
          }
    }
  }
}

void orc_regularize(const int32_t *levelsIn, int32_t *levelsOut, int nbx, int nby, int nbz,
                    int nLevels, int64_t *perLevel) {
  const int64_t nB = (int64_t)nbx * nby * nbz;
  int32_t *src = (int32_t *)malloc(sizeof(int32_t) * (size_t)nB);
  int32_t *dst = (int32_t *)malloc(sizeof(int32_t) * (size_t)nB);
  memcpy(src, levelsIn, sizeof(int32_t) * (size_t)nB);
  memcpy(dst, levelsIn, sizeof(int32_t) * (size_t)nB);
  for (int ll = 1; ll <= nLevels - 2; ll++) {
#pragma omp parallel for schedule(static)
    for (int64_t bid = 0; bid < nB; bid++) {
      const int bz = (int)(bid / ((int64_t)nbx * nby));
      const int rem = (int)(bid % ((int64_t)nbx * nby));
      const int by = rem / nbx, bx = rem % nbx;
      int level = src[bid];
      if (level >= ll) {
        int finest = nLevels - 1;
        for (int dz = -1; dz <= 1; dz++)
          for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++) {
              if (!dx && !dy && !dz) continue;
              const int x = bx + dx, y = by + dy, z = bz + dz;
              if (x < 0 || y < 0 || z < 0 || x >= nbx || y >= nby || z >= nbz) continue;
              const int l2 = src[(int64_t)z * nbx * nby + (int64_t)y * nbx + x];
              if (l2 < finest) finest = l2;
            }
        if (finest == ll - 1) level = ll;
      }
      dst[bid] = level;
    }
    memcpy(src, dst, sizeof(int32_t) * (size_t)nB);
  }
  if (perLevel) {
    for (int l = 0; l < 8; l++) perLevel[l] = 0;
    for (int64_t b = 0; b < nB; b++)
      if (dst[b] >= 0 && dst[b] < 8) perLevel[dst[b]]++;
  }
  memcpy(levelsOut, dst, sizeof(int32_t) * (size_t)nB);
  free(src);
  free(dst);
}

void orc_block_flags(const int32_t *levels, const uint16_t *existsFlags, uint16_t *flags,
                     int nbx, int nby, int nbz) {
  const int64_t nB = (int64_t)nbx * nby * nbz;
#pragma omp parallel for schedule(static)
  for (int64_t bid = 0; bid < nB; bid++) {
    const int bz = (int)(bid / ((int64_t)nbx * nby));
    const int rem = (int)(bid % ((int64_t)nbx * nby));
    const int by = rem / nbx, bx = rem % nbx;
    uint16_t f = existsFlags ? (uint16_t)(existsFlags[bid] & ORC_BLK_EXISTS) : 0;
    if (bx == 0 || bx == nbx - 1 || by == 0 || by == nby - 1 || bz == 0 || bz == nbz - 1)
      f |= ORC_BLK_DOM_BORDER;
    const int level = levels[bid];
    int lmax = 0, lmin = 1 << 20;
    for (int dz = -1; dz <= 1; dz++)
      for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++) {
          if (!dx && !dy && !dz) continue;
          const int x = bx + dx, y = by + dy, z = bz + dz;
          if (x < 0 || y < 0 || z < 0 || x >= nbx || y >= nby || z >= nbz) continue;
          const int l2 = levels[(int64_t)z * nbx * nby + (int64_t)y * nbx + x];
          lmax = imax(lmax, l2);
          lmin = imin(lmin, l2);
        }
    if (lmax > level) f |= ORC_BLK_FINE_COARSE;
    if (lmin < level) f |= ORC_BLK_COARSE_FINE;
    if (!(f & ORC_BLK_EXISTS) && !(f & (ORC_BLK_FINE_COARSE | ORC_BLK_COARSE_FINE)))
      f |= ORC_BLK_UNIFORM_EMPTY;
    flags[bid] = f;
  }
}

int32_t orc_build_slots(const int32_t *levels, int nBlocks, int32_t *slot, int32_t *activeBids) {
  int32_t n = 0;
  for (int b = 0; b < nBlocks; b++) {
    if (levels[b] == 0) {
      slot[b] = n;
      activeBids[n++] = b;
    } else {
      slot[b] = -1;
    }
  }
  return n;
}

void orc_fill(const orc_grid *g, void *payload, int64_t nActive, double v) {
  const int64_t nv = (int64_t)nActive * g->bsx * g->bsx * g->bsx;
  for (int64_t i = 0; i < nv; i++) {
    switch (g->storage) {
      case ORC_F32: ((float *)payload)[i] = (float)v; break;
      case ORC_U16: ((uint16_t *)payload)[i] = u16_rha((float)v); break;
      case ORC_F16: ((uint16_t *)payload)[i] = orc_f32_to_f16((float)v); break;
      default: ((double *)payload)[i] = v; break;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* splat / finalize                                                          */
/* ------------------------------------------------------------------------ */

static inline int block_color8(int bx, int by, int bz) {
  return (bx & 1) + ((by & 1) << 1) + ((bz & 1) << 2); /* src/msbg.h:642-646 */
}

/* min-store of q = distSq/distSqMax into the voxel, in the slab's storage type. */
static inline void splat_store(const orc_grid *g, void *payload, int64_t i, float q) {
  switch (g->storage) {
    case ORC_F32: {
      float *p = (float *)payload + i;
      if (q < *p) *p = q;
      break;
    }
    case ORC_U16: {
      uint16_t *p = (uint16_t *)payload + i, v = u16_rha(q);
      if (v < *p) *p = v;
      break;
    }
    case ORC_F16: {
      uint16_t *p = (uint16_t *)payload + i, v = orc_f32_to_f16(q);
      if (v < *p) *p = v; /* non-negative halves order like their bit patterns */
      break;
    }
    default: {
      double *p = (double *)payload + i;
      if ((double)q < *p) *p = q;
      break;
    }
  }
}

int64_t orc_splat(const orc_grid *g, const float *pts, const int64_t *bucketStart,
                  const int64_t *bucketIdx, const int32_t *slot, const int32_t *activeBids,
                  int32_t nActive, void *payload, float rParticle, float nbDist) {
  const float rScan = rParticle + nbDist;
  const float distSqMax = rScan * rScan, distSqMaxInv = 1.0f / distSqMax;
  const int bs = g->bsx, s = ilog2(bs), s2 = 2 * s, mask = bs - 1;
  const int nx = g->nbx, nxy = g->nbx * g->nby;
  const int64_t nv = (int64_t)bs * bs * bs;
  int64_t nAborted = 0;
  int32_t *lists[8];
  int32_t cnt[8] = {0};
  for (int c = 0; c < 8; c++) lists[c] = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nActive + 1));
  for (int32_t t = 0; t < nActive; t++) {
    const int bid = activeBids[t];
    const int bz = bid / nxy, by = (bid % nxy) / nx, bx = bid % nx;
    const int c = block_color8(bx, by, bz);
    lists[c][cnt[c]++] = bid;
  }
  for (int c = 0; c < 8; c++) {
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : nAborted)
    for (int32_t t = 0; t < cnt[c]; t++) {
      const int bid = lists[c][t];
      for (int64_t q = bucketStart[bid]; q < bucketStart[bid + 1]; q++) {
        const float *p = pts + 3 * bucketIdx[q];
        const int ix1 = imax((int)ceilf(p[0] - rScan - 0.5f), 0);
        const int iy1 = imax((int)ceilf(p[1] - rScan - 0.5f), 0);
        const int iz1 = imax((int)ceilf(p[2] - rScan - 0.5f), 0);
        const int ix2 = imin((int)floorf(p[0] + rScan - 0.5f), g->sx - 1);
        const int iy2 = imin((int)floorf(p[1] + rScan - 0.5f), g->sy - 1);
        const int iz2 = imin((int)floorf(p[2] + rScan - 0.5f), g->sz - 1);
        const float x0 = p[0] - 0.5f, y0 = p[1] - 0.5f, z0 = p[2] - 0.5f;
        for (int iz = iz1; iz <= iz2; iz++) {
          const float dz = (float)iz - z0;
          const int ibz = (iz >> s) * nxy, ivz = (iz & mask) << s2;
          for (int iy = iy1; iy <= iy2; iy++) {
            const float dy = (float)iy - y0;
            const float dzy = dz * dz + dy * dy;
            const int ibzy = ibz + (iy >> s) * nx, ivzy = ivz + ((iy & mask) << s);
            for (int ix = ix1; ix <= ix2; ix++) {
              const float dx = (float)ix - x0;
              const float d2 = dzy + dx * dx;
              if (d2 > distSqMax) continue;
              const int sl = slot[ibzy + (ix >> s)];
              if (sl < 0) { nAborted++; goto next_particle; }
              splat_store(g, payload, (int64_t)sl * nv + ivzy + (ix & mask), d2 * distSqMaxInv);
            }
          }
        }
      next_particle:;
      }
    }
  }
  for (int c = 0; c < 8; c++) free(lists[c]);
  return nAborted;
}

/* MT_LINSTEPF, src/mtool.h:400-408.  The reference is built with -ffast-math,
 * under which the division by the constant (b - a) becomes a multiplication by
 * its rounded reciprocal; that is the rounding reproduced here. */
static inline float linstepf(float a, float b, float x) {
  if (x < a) return 0.0f;
  if (x >= b) return 1.0f;
  const float inv = 1.0f / (b - a);
  return (x - a) * inv;
}

void orc_finalize(const orc_grid *g, void *payload, int64_t nActive, float rParticle,
                  float nbDist) {
  const float rScan = rParticle + nbDist, distSqMax = rScan * rScan;
  const int64_t n = nActive * (int64_t)g->bsx * g->bsx * g->bsx;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++) {
    float d = (float)load_val(g, payload, i);
    float f = 0.0f;
    if (d < 0.999f) {
      d *= distSqMax;
      const float dist = sqrtf(d) - rParticle;
      f = 1.0f - linstepf(-rParticle, rParticle + nbDist, dist);
    }
    switch (g->storage) {
      case ORC_F32: ((float *)payload)[i] = f; break;
      case ORC_U16: ((uint16_t *)payload)[i] = u16_rha(f); break;
      case ORC_F16: ((uint16_t *)payload)[i] = orc_f32_to_f16(f); break;
      default: ((double *)payload)[i] = f; break;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* halo fill + stencil sweeps                                                */
/* ------------------------------------------------------------------------ */

/* Halo of h voxels around block bid, as fillHaloBlock_ with OPT_BC_NEUMANN
 * (src/halo.cpp:266-479, src/halo.h:266-355): in-domain voxels read their block
 * (a constant empty block reads emptyValue); out-of-domain voxels take the value
 * of the nearest voxel of the block itself. */
#define DEFINE_HALO(REAL, NAME)                                                           \
  static void NAME(const orc_grid *g, const int32_t *slot, const void *payload, int bid, \
                   int h, REAL *halo) {                                                   \
    const int bs = g->bsx, hs = bs + 2 * h, s = ilog2(bs);                                \
    const int nx = g->nbx, nxy = g->nbx * g->nby;                                         \
    const int bz = bid / nxy, by = (bid % nxy) / nx, bx = bid % nx;                       \
    const int x0 = bx * bs, y0 = by * bs, z0 = bz * bs;                                   \
    const int64_t nv = (int64_t)bs * bs * bs;                                             \
    const int64_t own = (int64_t)slot[bid] * nv;                                          \
    for (int hz = 0; hz < hs; hz++)                                                       \
      for (int hy = 0; hy < hs; hy++)                                                     \
        for (int hx = 0; hx < hs; hx++) {                                                 \
          int x = x0 + hx - h, y = y0 + hy - h, z = z0 + hz - h;                          \
          double v;                                                                       \
          if (x >= 0 && x < g->sx && y >= 0 && y < g->sy && z >= 0 && z < g->sz) {        \
            const int sl = slot[(z >> s) * nxy + (y >> s) * nx + (x >> s)];               \
            const int vid = ((z & (bs - 1)) << (2 * s)) + ((y & (bs - 1)) << s) +          \
                            (x & (bs - 1));                                               \
            v = sl < 0 ? g->emptyValue : load_val(g, payload, (int64_t)sl * nv + vid);     \
          } else {                                                                        \
            x = imin(imax(x, x0), x0 + bs - 1);                                           \
            y = imin(imax(y, y0), y0 + bs - 1);                                           \
            z = imin(imax(z, z0), z0 + bs - 1);                                           \
            const int vid = ((z - z0) * bs + (y - y0)) * bs + (x - x0);                   \
            v = load_val(g, payload, own + vid);                                          \
          }                                                                               \
          halo[((int64_t)hz * hs + hy) * hs + hx] = (REAL)v;                              \
        }                                                                                 \
  }

DEFINE_HALO(float, halo_f)
DEFINE_HALO(double, halo_d)

typedef struct {
  int laplTyp, constr01;
  float dt, anisAlpha;
} pde_params;

/* Per-voxel update of applyChannelPdeFast (src/msbg4.cpp:559-825), written once
 * for float and once for double math.  F(dx,dy,dz) reads the halo. */
#define DEFINE_UPDATE(REAL, NAME, SQRT, EXP)                                              \
  static inline REAL NAME(const REAL *ph, int hs, const pde_params *pp, int iIter) {      \
    const int hs2 = hs * hs;                                                              \
    const REAL dt = (REAL)pp->dt;                                                         \
    REAL phi = ph[0];                                                                     \
    REAL out = phi;                                                                       \
    (void)iIter;                                                                          \
    if (pp->laplTyp == 4) {                                                               \
      const REAL f0 = ph[0], f1 = ph[-1], f2 = ph[1], f3 = ph[-hs], f4 = ph[hs],          \
                 f5 = ph[-hs2], f6 = ph[hs2];                                             \
      const REAL fx = (REAL)0.5 * (f2 - f1), fy = (REAL)0.5 * (f4 - f3),                  \
                 fz = (REAL)0.5 * (f6 - f5);                                              \
      const REAL fxx = f1 + f2 - 2 * f0, fyy = f3 + f4 - 2 * f0, fzz = f5 + f6 - 2 * f0;  \
      const REAL fy_r = (ph[1 + hs] - ph[1 - hs]) * (REAL)0.5;                            \
      const REAL fy_l = (ph[-1 + hs] - ph[-1 - hs]) * (REAL)0.5;                          \
      const REAL fz_r = (ph[1 + hs2] - ph[1 - hs2]) * (REAL)0.5;                          \
      const REAL fz_l = (ph[-1 + hs2] - ph[-1 - hs2]) * (REAL)0.5;                        \
      const REAL fz_u = (ph[hs + hs2] - ph[hs - hs2]) * (REAL)0.5;                        \
      const REAL fz_d = (ph[-hs + hs2] - ph[-hs - hs2]) * (REAL)0.5;                      \
      const REAL fyx = (fy_r - fy_l) * (REAL)0.5, fzx = (fz_r - fz_l) * (REAL)0.5,        \
                 fzy = (fz_u - fz_d) * (REAL)0.5;                                         \
      REAL H = (fy * fy + fz * fz) * fxx + (fx * fx + fz * fz) * fyy +                    \
               (fx * fx + fy * fy) * fzz -                                                \
               (REAL)2 * (fx * fy * fyx + fx * fz * fzx + fy * fz * fzy);                 \
      const REAL g2 = fx * fx + fy * fy + fz * fz;                                        \
      H = g2 > (REAL)1e-7f ? H / g2 : (REAL)0;                                            \
      REAL D = dt * H;                                                                    \
      D = D < (REAL)-0.1f ? (REAL)-0.1f : D;                                              \
      D = D > (REAL)0.1f ? (REAL)0.1f : D;                                                \
      out = phi + D;                                                                      \
    } else if (pp->laplTyp == 17) {                                                       \
      const REAL s6 = ph[-1] + ph[1] + ph[-hs] + ph[hs] + ph[-hs2] + ph[hs2];             \
      out = (phi + dt * s6) / ((REAL)1 + dt * (REAL)6);                                   \
    } else if (pp->laplTyp == 3) {                                                        \
      const REAL S = ((REAL)1 / (REAL)6) *                                                \
                     (ph[-1] + ph[1] + ph[-hs] + ph[hs] + ph[-hs2] + ph[hs2]);            \
      out = phi + dt * (S - phi);                                                         \
    } else if (pp->laplTyp == 1) {                                                        \
      const REAL F1 = ph[-1], F2 = ph[1], F3 = ph[-hs], F4 = ph[hs], F5 = ph[-hs2],       \
                 F6 = ph[hs2];                                                            \
      const REAL L = F1 + F2 + F3 + F4 + F5 + F6 - (REAL)6 * phi;                         \
      const REAL GX = (REAL)0.5 * (F2 - F1), GY = (REAL)0.5 * (F4 - F3),                  \
                 GZ = (REAL)0.5 * (F6 - F5);                                              \
      const REAL G = SQRT(GX * GX + GY * GY + GZ * GZ);                                   \
      out = phi + dt * L * G;                                                             \
    } else if (pp->laplTyp == 14 || pp->laplTyp == 15) {                                  \
      const REAL a = (REAL)pp->anisAlpha;                                                 \
      const REAL fn[6] = {ph[-1], ph[1], ph[-hs], ph[hs], ph[-hs2], ph[hs2]};             \
      REAL sum = 0, wsum = 0, dsum = 0;                                                   \
      for (int k = 0; k < 6; k++) {                                                       \
        const REAL gk = fn[k] - phi;                                                      \
        const REAL ag = gk < 0 ? -gk : gk;                                                \
        REAL Gk;                                                                          \
        if (a < 0) {                                                                      \
          const REAL t = ag * ((REAL)1 / -a);                                             \
          Gk = EXP(-(t * t));                                                             \
        } else {                                                                          \
          const REAL t = ag / a;                                                          \
          Gk = (REAL)1 / ((REAL)1 + t * t);                                               \
        }                                                                                 \
        sum += Gk * fn[k];                                                                \
        wsum += Gk;                                                                       \
        dsum += Gk * gk;                                                                  \
      }                                                                                   \
      if (pp->laplTyp == 15)                                                              \
        out = (phi + dt * sum) / ((REAL)1 + dt * wsum);                                   \
      else                                                                                \
        out = phi + dt * dsum;                                                            \
    }                                                                                     \
    if (pp->constr01) {                                                                   \
      out = out > (REAL)0 ? out : (REAL)0;                                                \
      out = out < (REAL)1 ? out : (REAL)1;                                                \
    }                                                                                     \
    return out;                                                                           \
  }

DEFINE_UPDATE(float, update_f, sqrtf, expf)
DEFINE_UPDATE(double, update_d, sqrt, exp)

static inline void store_val(const orc_grid *g, void *p, int64_t i, double v) {
  switch (g->storage) {
    case ORC_F32: ((float *)p)[i] = (float)v; break;
    case ORC_U16: ((uint16_t *)p)[i] = u16_rne((float)v); break; /* round_to_int: RNE */
    case ORC_F16: ((uint16_t *)p)[i] = orc_f32_to_f16((float)v); break;
    default: ((double *)p)[i] = v; break;
  }
}

/* One block: halo from src, update into dst (dst may equal src for colored
 * schedules; the halo is a private copy so the block reads only old values). */
static void sweep_block(const orc_grid *g, const int32_t *slot, const void *src, void *dst,
                        int bid, const pde_params *pp, int iIter, void *haloBuf) {
  const int bs = g->bsx, h = 1, hs = bs + 2 * h;
  const int64_t nv = (int64_t)bs * bs * bs, base = (int64_t)slot[bid] * nv;
  if (g->storage == ORC_F64) {
    double *halo = (double *)haloBuf;
    halo_d(g, slot, src, bid, h, halo);
    for (int z = 0; z < bs; z++)
      for (int y = 0; y < bs; y++)
        for (int x = 0; x < bs; x++) {
          const double *ph = halo + ((int64_t)(z + h) * hs + (y + h)) * hs + (x + h);
          store_val(g, dst, base + ((int64_t)z * bs + y) * bs + x, update_d(ph, hs, pp, iIter));
        }
  } else {
    float *halo = (float *)haloBuf;
    halo_f(g, slot, src, bid, h, halo);
    for (int z = 0; z < bs; z++)
      for (int y = 0; y < bs; y++)
        for (int x = 0; x < bs; x++) {
          const float *ph = halo + ((int64_t)(z + h) * hs + (y + h)) * hs + (x + h);
          store_val(g, dst, base + ((int64_t)z * bs + y) * bs + x, update_f(ph, hs, pp, iIter));
        }
  }
}

int orc_pde(const orc_grid *g, const int32_t *slot, const int32_t *activeBids, int32_t nActive,
            void *payload, void *payloadTmp, int laplTyp, int constr01, int numIter, float dt,
            float anisAlpha) {
  int color8 = 0, redBlack = 0;
  if (laplTyp < 0) { /* src/msbg4.cpp:100-114 */
    laplTyp = -laplTyp;
    if (laplTyp & (1 << 29)) {
      laplTyp &= ~(1 << 29);
      color8 = 1;
    } else {
      redBlack = 1;
    }
  }
  if (!(laplTyp == 4 || laplTyp == 17 || laplTyp == 3 || laplTyp == 1 || laplTyp == 14 ||
        laplTyp == 15))
    return -1;
  if (!color8 && !redBlack && !payloadTmp) return -2;
  const int nIter0 = numIter;
  int nIter = numIter;
  if (nIter % 2 == 1) nIter++; /* src/msbg4.cpp:150-152 */
  pde_params pp = {laplTyp, constr01, dt, anisAlpha};
  const int bs = g->bsx, hs = bs + 2;
  const int nx = g->nbx, nxy = g->nbx * g->nby;
  const int64_t nv = (int64_t)bs * bs * bs;
  const size_t eb = elem_bytes(g->storage);
  const size_t haloBytes = (size_t)hs * hs * hs * (g->storage == ORC_F64 ? 8 : 4);
  const int nPass = color8 ? 8 : redBlack ? 2 : 1;

  /* ping-pong: slot layout identical in both slabs */
  void *bufs[2] = {payload, payloadTmp};
  int cur = 0;
  for (int it = 0; it < nIter; it++) {
    void *src = color8 || redBlack ? payload : bufs[cur];
    void *dst = color8 || redBlack ? payload : bufs[cur ^ 1];
    const int copyOnly = !(color8 || redBlack) && it == nIter - 1 && (nIter0 % 2) == 1;
    for (int pass = 0; pass < nPass; pass++) {
#pragma omp parallel
      {
        void *halo = malloc(haloBytes);
#pragma omp for schedule(dynamic, 4)
        for (int32_t t = 0; t < nActive; t++) {
          const int bid = activeBids[t];
          const int bz = bid / nxy, by = (bid % nxy) / nx, bx = bid % nx;
          if (redBlack && ((bx + by + bz) & 1) == pass) continue; /* src/msbg4.cpp:447-454 */
          if (color8 && block_color8(bx, by, bz) != pass) continue;
          if (copyOnly) {
            memcpy((char *)dst + (size_t)slot[bid] * nv * eb,
                   (const char *)src + (size_t)slot[bid] * nv * eb, (size_t)nv * eb);
            continue;
          }
          sweep_block(g, slot, src, dst, bid, &pp, it, halo);
        }
        free(halo);
      }
    }
    cur ^= 1;
  }
  /* ping-pong ends with the result in bufs[cur]; nIter is even so cur == 0 */
  return 0;
}

/* ------------------------------------------------------------------------ */
/* sparse Poisson solve (FP64)                                               */
/* ------------------------------------------------------------------------ */

static inline uint32_t hash32(uint32_t x) {
  x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
  return x;
}

float orc_face_coeff(uint32_t seed, int axis, int gx, int gy, int gz) {
  uint32_t h = hash32(seed ^ hash32((uint32_t)axis + 0x9e3779b9U * 3u));
  h = hash32(h ^ (uint32_t)gx);
  h = hash32(h ^ (uint32_t)gy * 0x85ebca6bU);
  h = hash32(h ^ (uint32_t)gz * 0xc2b2ae35U);
  return 0.5f + 1.5f * (float)(h >> 8) * (1.0f / 16777216.0f);
}

typedef struct {
  int nx, ny, nz;
  uint8_t *act;
  double *cx, *cy, *cz, *d, *x, *b, *r;
  int64_t nAct;
} plev;

#define PIDX(L, x, y, z) (((int64_t)(z) * (L)->ny + (y)) * (L)->nx + (x))

static inline int pin(const plev *L, int x, int y, int z) {
  return x >= 0 && y >= 0 && z >= 0 && x < L->nx && y < L->ny && z < L->nz && L->act[PIDX(L, x, y, z)];
}

static void papply(const plev *L, const double *x, const double *b, double *y, int residual) {
#pragma omp parallel for collapse(2) schedule(static)
  for (int z = 0; z < L->nz; z++)
    for (int yy = 0; yy < L->ny; yy++)
      for (int xx = 0; xx < L->nx; xx++) {
        const int64_t i = PIDX(L, xx, yy, z);
        if (!L->act[i]) { y[i] = 0; continue; }
        double s = L->d[i] * x[i];
        if (pin(L, xx - 1, yy, z)) s -= L->cx[i] * x[i - 1];
        if (pin(L, xx + 1, yy, z)) s -= L->cx[i + 1] * x[i + 1];
        if (pin(L, xx, yy - 1, z)) s -= L->cy[i] * x[i - L->nx];
        if (pin(L, xx, yy + 1, z)) s -= L->cy[i + L->nx] * x[i + L->nx];
        const int64_t sl = (int64_t)L->nx * L->ny;
        if (pin(L, xx, yy, z - 1)) s -= L->cz[i] * x[i - sl];
        if (pin(L, xx, yy, z + 1)) s -= L->cz[i + sl] * x[i + sl];
        y[i] = residual ? b[i] - s : s;
      }
}

static void prbgs(const plev *L, double *x, const double *b, int nSweeps, int redFirst) {
  const int64_t sl = (int64_t)L->nx * L->ny;
  for (int sw = 0; sw < nSweeps; sw++)
    for (int k = 0; k < 2; k++) {
      const int color = redFirst ? k : 1 - k;
#pragma omp parallel for collapse(2) schedule(static)
      for (int z = 0; z < L->nz; z++)
        for (int yy = 0; yy < L->ny; yy++)
          for (int xx = 0; xx < L->nx; xx++) {
            if (((xx + yy + z) & 1) != color) continue;
            const int64_t i = PIDX(L, xx, yy, z);
            if (!L->act[i]) continue;
            double s = b[i];
            if (pin(L, xx - 1, yy, z)) s += L->cx[i] * x[i - 1];
            if (pin(L, xx + 1, yy, z)) s += L->cx[i + 1] * x[i + 1];
            if (pin(L, xx, yy - 1, z)) s += L->cy[i] * x[i - L->nx];
            if (pin(L, xx, yy + 1, z)) s += L->cy[i + L->nx] * x[i + L->nx];
            if (pin(L, xx, yy, z - 1)) s += L->cz[i] * x[i - sl];
            if (pin(L, xx, yy, z + 1)) s += L->cz[i + sl] * x[i + sl];
            x[i] = s / L->d[i];
          }
    }
}

/* Smoother tiles on a level whose blocks have edge bs: 32x16x8 (bs 32), 16^3 (bs 16),
 * 8^3 (bs 8); pointwise red-black below (tile[0] = 0). */
static void ptile(int bsl, int t[3]) {
  if (bsl >= 32) { t[0] = 32; t[1] = 16; t[2] = 8; }
  else if (bsl == 16) { t[0] = t[1] = t[2] = 16; }
  else if (bsl == 8) { t[0] = t[1] = t[2] = 8; }
  else { t[0] = t[1] = t[2] = 0; }
}

/* One smoothing pass.  Pointwise levels: k red-black sweeps.  Tile levels: tiles
 * (TX,TY,TZ) are coloured by (gx/TX + gy/TY + gz/TZ) & 1; for each tile colour,
 * every tile of that colour does k in-tile red-black Gauss-Seidel sweeps with the
 * cells outside the tile held fixed.  Same-colour tiles share no face, so the
 * order among them does not matter.  reverse: tile colours 1,0 and in-tile cell
 * colours black,red (the adjoint order, for the post-smoother). */
static void psmooth_pass(const plev *L, const int *T, double *x, const double *b, int k, int reverse) {
  if (T[0] == 0) {
    prbgs(L, x, b, k, !reverse);
    return;
  }
  const int64_t sl = (int64_t)L->nx * L->ny;
  for (int tci = 0; tci < 2; tci++) {
    const int tc = reverse ? 1 - tci : tci;
    for (int it = 0; it < k; it++)
      for (int cci = 0; cci < 2; cci++) {
        const int cc = reverse ? 1 - cci : cci;
#pragma omp parallel for collapse(2) schedule(static)
        for (int z = 0; z < L->nz; z++)
          for (int yy = 0; yy < L->ny; yy++)
            for (int xx = 0; xx < L->nx; xx++) {
              if (((xx + yy + z) & 1) != cc) continue;
              if (((xx / T[0] + yy / T[1] + z / T[2]) & 1) != tc) continue;
              const int64_t i = PIDX(L, xx, yy, z);
              if (!L->act[i]) continue;
              double s = b[i];
              if (pin(L, xx - 1, yy, z)) s += L->cx[i] * x[i - 1];
              if (pin(L, xx + 1, yy, z)) s += L->cx[i + 1] * x[i + 1];
              if (pin(L, xx, yy - 1, z)) s += L->cy[i] * x[i - L->nx];
              if (pin(L, xx, yy + 1, z)) s += L->cy[i + L->nx] * x[i + L->nx];
              if (pin(L, xx, yy, z - 1)) s += L->cz[i] * x[i - sl];
              if (pin(L, xx, yy, z + 1)) s += L->cz[i + sl] * x[i + sl];
              x[i] = s / L->d[i];
            }
      }
  }
}

static void psmooth(const plev *L, const int *T, double *x, const double *b, int passes, int k, int reverse) {
  for (int p = 0; p < passes; p++) psmooth_pass(L, T, x, b, k, reverse);
}

static plev *pcoarsen(const plev *F) {
  plev *C = (plev *)calloc(1, sizeof(plev));
  C->nx = (F->nx + 1) / 2; C->ny = (F->ny + 1) / 2; C->nz = (F->nz + 1) / 2;
  const int64_t n = (int64_t)C->nx * C->ny * C->nz;
  C->act = (uint8_t *)calloc((size_t)n, 1);
  double **arr[7] = {&C->cx, &C->cy, &C->cz, &C->d, &C->x, &C->b, &C->r};
  for (int k = 0; k < 7; k++) *arr[k] = (double *)calloc((size_t)n, sizeof(double));
  for (int z = 0; z < C->nz; z++)
    for (int y = 0; y < C->ny; y++)
      for (int x = 0; x < C->nx; x++) {
        const int64_t c = PIDX(C, x, y, z);
        double dsum = 0, lx = 0, ly = 0, lz = 0;
        int any = 0;
        for (int k = 0; k < 8; k++) {
          const int ix = k & 1, iy = (k >> 1) & 1, iz = k >> 2;
          const int fx = 2 * x + ix, fy = 2 * y + iy, fz = 2 * z + iz;
          if (!pin(F, fx, fy, fz)) continue;
          any = 1;
          const int64_t f = PIDX(F, fx, fy, fz);
          dsum += F->d[f];
          if (ix == 0) { if (pin(F, fx - 1, fy, fz)) lx += F->cx[f]; }
          else if (pin(F, fx - 1, fy, fz)) dsum -= 2.0 * F->cx[f];
          if (iy == 0) { if (pin(F, fx, fy - 1, fz)) ly += F->cy[f]; }
          else if (pin(F, fx, fy - 1, fz)) dsum -= 2.0 * F->cy[f];
          if (iz == 0) { if (pin(F, fx, fy, fz - 1)) lz += F->cz[f]; }
          else if (pin(F, fx, fy, fz - 1)) dsum -= 2.0 * F->cz[f];
        }
        C->act[c] = (uint8_t)any;
        if (any) {
          C->nAct++;
          C->cx[c] = 0.5 * lx; C->cy[c] = 0.5 * ly; C->cz[c] = 0.5 * lz; C->d[c] = 0.5 * dsum;
        }
      }
  return C;
}

static void pfree(plev *L, int ownsCoeffs) {
  if (!L) return;
  free(L->act);
  if (ownsCoeffs) { free(L->cx); free(L->cy); free(L->cz); free(L->d); }
  free(L->x); free(L->b); free(L->r);
  free(L);
}

typedef struct {
  plev *lv[40];
  int tile[40][3];
  int n;
  int pre, post, k, coarsestIter;
  /* exact coarsest solve (coarsestIter == 0): Cholesky factor over the active cells */
  int nc;
  int64_t *cidx;  /* dense index of each active coarsest cell */
  double *chol;   /* [nc][nc] lower factor */
} phier;

static void pchol_build(phier *H) {
  const plev *C = H->lv[H->n - 1];
  const int64_t nd = (int64_t)C->nx * C->ny * C->nz;
  int64_t *map = (int64_t *)malloc((size_t)nd * sizeof(int64_t));
  int n = 0;
  for (int64_t i = 0; i < nd; i++) map[i] = C->act[i] ? n++ : -1;
  H->nc = n;
  H->cidx = (int64_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
  for (int64_t i = 0; i < nd; i++) if (map[i] >= 0) H->cidx[map[i]] = i;
  double *A = (double *)calloc((size_t)n * n + 1, sizeof(double));
  const int64_t sl = (int64_t)C->nx * C->ny;
  for (int k = 0; k < n; k++) {
    const int64_t i = H->cidx[k];
    const int x = (int)(i % C->nx), y = (int)((i / C->nx) % C->ny), z = (int)(i / sl);
    A[(size_t)k * n + k] = C->d[i];
    if (pin(C, x - 1, y, z)) A[(size_t)k * n + map[i - 1]] = -C->cx[i];
    if (pin(C, x + 1, y, z)) A[(size_t)k * n + map[i + 1]] = -C->cx[i + 1];
    if (pin(C, x, y - 1, z)) A[(size_t)k * n + map[i - C->nx]] = -C->cy[i];
    if (pin(C, x, y + 1, z)) A[(size_t)k * n + map[i + C->nx]] = -C->cy[i + C->nx];
    if (pin(C, x, y, z - 1)) A[(size_t)k * n + map[i - sl]] = -C->cz[i];
    if (pin(C, x, y, z + 1)) A[(size_t)k * n + map[i + sl]] = -C->cz[i + sl];
  }
  for (int j = 0; j < n; j++) {
    double t = A[(size_t)j * n + j];
    for (int k = 0; k < j; k++) t -= A[(size_t)j * n + k] * A[(size_t)j * n + k];
    const double dj = sqrt(t > 0 ? t : 1e-300);
    A[(size_t)j * n + j] = dj;
    for (int i = j + 1; i < n; i++) {
      double u = A[(size_t)i * n + j];
      for (int k = 0; k < j; k++) u -= A[(size_t)i * n + k] * A[(size_t)j * n + k];
      A[(size_t)i * n + j] = u / dj;
    }
  }
  H->chol = A;
  free(map);
}

static void pchol_solve(const phier *H, const double *b, double *x) {
  const int n = H->nc;
  const double *L = H->chol;
  double *y = (double *)malloc((size_t)(n > 0 ? n : 1) * sizeof(double));
  for (int i = 0; i < n; i++) {
    double t = b[H->cidx[i]];
    for (int k = 0; k < i; k++) t -= L[(size_t)i * n + k] * y[k];
    y[i] = t / L[(size_t)i * n + i];
  }
  for (int i = n - 1; i >= 0; i--) {
    double t = y[i];
    for (int k = i + 1; k < n; k++) t -= L[(size_t)k * n + i] * y[k];
    y[i] = t / L[(size_t)i * n + i];
  }
  for (int i = 0; i < n; i++) x[H->cidx[i]] = y[i];
  free(y);
}

static void pbuild(phier *H, const orc_level0 *L0, int log2bs0, int64_t coarsestCells) {
  plev *F = (plev *)calloc(1, sizeof(plev));
  F->nx = L0->nx; F->ny = L0->ny; F->nz = L0->nz;
  const int64_t n = (int64_t)F->nx * F->ny * F->nz;
  F->act = (uint8_t *)malloc((size_t)n);
  memcpy(F->act, L0->act, (size_t)n);
  F->cx = (double *)L0->cx; F->cy = (double *)L0->cy; F->cz = (double *)L0->cz; F->d = (double *)L0->d;
  F->x = (double *)calloc((size_t)n, 8); F->b = (double *)calloc((size_t)n, 8); F->r = (double *)calloc((size_t)n, 8);
  for (int64_t i = 0; i < n; i++) F->nAct += F->act[i];
  H->lv[0] = F;
  ptile(1 << log2bs0, H->tile[0]);
  H->n = 1;
  for (int l = 0; l < log2bs0; l++) {
    plev *c = pcoarsen(H->lv[H->n - 1]);
    H->lv[H->n] = c;
    ptile(1 << (log2bs0 - l - 1), H->tile[H->n]);
    H->n++;
  }
  while (H->n < 40) {
    const plev *f = H->lv[H->n - 1];
    if (f->nAct <= coarsestCells || (f->nx <= 2 && f->ny <= 2 && f->nz <= 2)) break;
    H->lv[H->n] = pcoarsen(f);
    ptile(1, H->tile[H->n]);
    H->n++;
  }
}

static void phfree(phier *H) {
  for (int l = 0; l < H->n; l++) pfree(H->lv[l], l > 0);
  free(H->cidx);
  free(H->chol);
}

static void pvcycle(phier *H, int l, double *x, const double *b, double *r) {
  plev *L = H->lv[l];
  const int64_t n = (int64_t)L->nx * L->ny * L->nz;
  memset(x, 0, (size_t)n * 8);
  if (l == H->n - 1) {
    if (H->coarsestIter > 0) prbgs(L, x, b, H->coarsestIter, 1);
    else pchol_solve(H, b, x);
    return;
  }
  psmooth(L, H->tile[l], x, b, H->pre, H->k, 0);
  papply(L, x, b, r, 1);
  plev *C = H->lv[l + 1];
  for (int z = 0; z < C->nz; z++)
    for (int y = 0; y < C->ny; y++)
      for (int xx = 0; xx < C->nx; xx++) {
        const int64_t c = PIDX(C, xx, y, z);
        double s = 0;
        for (int k = 0; k < 8; k++) {
          const int fx = 2 * xx + (k & 1), fy = 2 * y + ((k >> 1) & 1), fz = 2 * z + (k >> 2);
          if (pin(L, fx, fy, fz)) s += r[PIDX(L, fx, fy, fz)];
        }
        C->b[c] = C->act[c] ? s : 0;
      }
  pvcycle(H, l + 1, C->x, C->b, C->r);
  for (int z = 0; z < L->nz; z++)
    for (int y = 0; y < L->ny; y++)
      for (int xx = 0; xx < L->nx; xx++) {
        const int64_t i = PIDX(L, xx, y, z);
        if (L->act[i]) x[i] += C->x[PIDX(C, xx >> 1, y >> 1, z >> 1)];
      }
  psmooth(L, H->tile[l], x, b, H->post, H->k, 1);
}

static plev view0(const orc_level0 *L0) {
  plev v;
  memset(&v, 0, sizeof(v));
  v.nx = L0->nx; v.ny = L0->ny; v.nz = L0->nz;
  v.act = (uint8_t *)L0->act;
  v.cx = (double *)L0->cx; v.cy = (double *)L0->cy; v.cz = (double *)L0->cz; v.d = (double *)L0->d;
  return v;
}

void orc_poisson_apply(const orc_level0 *L0, const double *x, const double *b, double *y, int residual) {
  plev v = view0(L0);
  papply(&v, x, b, y, residual);
}

void orc_poisson_rbgs(const orc_level0 *L0, double *x, const double *b, int nSweeps, int redFirst) {
  plev v = view0(L0);
  prbgs(&v, x, b, nSweeps, redFirst);
}

void orc_poisson_smooth(const orc_level0 *L0, int log2bs, double *x, const double *b, int passes, int k,
                        int reverse) {
  plev v = view0(L0);
  int t[3];
  ptile(1 << log2bs, t);
  psmooth(&v, t, x, b, passes, k, reverse);
}

int orc_poisson_vcycle(const orc_level0 *L0, int log2bs0, const double *b, double *x, int preSweeps,
                       int postSweeps, int tileIters, int coarsestIter, int64_t coarsestCells) {
  phier H;
  memset(&H, 0, sizeof(H));
  H.pre = preSweeps; H.post = postSweeps; H.k = tileIters; H.coarsestIter = coarsestIter;
  pbuild(&H, L0, log2bs0, coarsestCells);
  if (coarsestIter == 0) pchol_build(&H);
  pvcycle(&H, 0, x, b, H.lv[0]->r);
  const int n = H.n;
  phfree(&H);
  return n;
}

static double pdot(const double *a, const double *b, int64_t n) {
  double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (int64_t i = 0; i < n; i++) s += a[i] * b[i];
  return s;
}

int orc_poisson_mgpcg(const orc_level0 *L0, int log2bs0, const double *b, double *x, double tol,
                      int maxIter, int preSweeps, int postSweeps, int tileIters, int coarsestIter,
                      int64_t coarsestCells, int *iters, double *relres) {
  phier H;
  memset(&H, 0, sizeof(H));
  H.pre = preSweeps; H.post = postSweeps; H.k = tileIters; H.coarsestIter = coarsestIter;
  pbuild(&H, L0, log2bs0, coarsestCells);
  if (coarsestIter == 0) pchol_build(&H);
  plev *L = H.lv[0];
  const int64_t n = (int64_t)L->nx * L->ny * L->nz;
  double *r = (double *)calloc((size_t)n, 8), *z = (double *)calloc((size_t)n, 8),
         *p = (double *)calloc((size_t)n, 8), *q = (double *)calloc((size_t)n, 8);
  papply(L, x, b, r, 1);
  const double bn = sqrt(pdot(b, b, n));
  double rel = bn > 0 ? sqrt(pdot(r, r, n)) / bn : 0;
  int it = 0;
  if (bn > 0 && rel > tol) {
    pvcycle(&H, 0, z, r, L->r);
    memcpy(p, z, (size_t)n * 8);
    double rz = pdot(r, z, n);
    for (it = 1; it <= maxIter; it++) {
      papply(L, p, NULL, q, 0);
      const double alpha = rz / pdot(p, q, n);
      for (int64_t i = 0; i < n; i++) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; }
      rel = sqrt(pdot(r, r, n)) / bn;
      if (rel <= tol) break;
      pvcycle(&H, 0, z, r, L->r);
      const double rz2 = pdot(r, z, n);
      const double beta = rz2 / rz;
      rz = rz2;
      for (int64_t i = 0; i < n; i++) p[i] = z[i] + beta * p[i];
    }
    if (it > maxIter) it = maxIter;
  }
  free(r); free(z); free(p); free(q);
  phfree(&H);
  if (iters) *iters = it;
  if (relres) *relres = rel;
  return 0;
}

void orc_poisson_coeffs_dense(uint32_t seed, int nx, int ny, int nz, const uint8_t *act, double *cx,
                              double *cy, double *cz, double *d) {
#pragma omp parallel for collapse(2) schedule(static)
  for (int z = 0; z < nz; z++)
    for (int y = 0; y < ny; y++)
      for (int x = 0; x < nx; x++) {
        const int64_t i = ((int64_t)z * ny + y) * nx + x;
        if (!act[i]) { cx[i] = cy[i] = cz[i] = d[i] = 0; continue; }
        const float lx = orc_face_coeff(seed, 0, x, y, z), ly = orc_face_coeff(seed, 1, x, y, z),
                    lz = orc_face_coeff(seed, 2, x, y, z);
        const float ux = orc_face_coeff(seed, 0, x + 1, y, z), uy = orc_face_coeff(seed, 1, x, y + 1, z),
                    uz = orc_face_coeff(seed, 2, x, y, z + 1);
        cx[i] = lx; cy[i] = ly; cz[i] = lz;
        d[i] = (float)(((lx + ux) + (ly + uy)) + (lz + uz));
      }
}

/* ------------------------------------------------------------------------- */
/* Restriction to the next coarser multigrid level (src/msbg4.cpp:1035-1379)  */
/* ------------------------------------------------------------------------- */

/* Fine value at global cell (x, y, z) with the OPT_BC_COARSE_LEVEL halo rule. */
static float ds_fetch(const orc_grid *g, const int32_t *slot, const void *payload, int x, int y, int z) {
  const int bs = g->bsx, L = ilog2(bs), m = bs - 1;
  x = imin(imax(x, 0), g->sx - 1);
  y = imin(imax(y, 0), g->sy - 1);
  z = imin(imax(z, 0), g->sz - 1);
  const int64_t bid = (int64_t)(x >> L) + (int64_t)(y >> L) * g->nbx + (int64_t)(z >> L) * g->nbx * g->nby;
  const int32_t s = slot[bid];
  if (s < 0) return (float)g->emptyValue;
  return (float)load_val(g, payload, (int64_t)s * bs * bs * bs + (((z & m) * bs + (y & m)) << L) + (x & m));
}

void orc_downsample(const orc_grid *g, const int32_t *slot, const int32_t *activeBids, int32_t nActive,
                    const void *payload, int simpleAverage, float *out) {
  const int bs = g->bsx, cb = bs / 2;
  const float k1[4] = {1.f, 3.f, 3.f, 1.f};
  float w[4][4][4];
  for (int k = 0; k < 4; k++)
    for (int j = 0; j < 4; j++)
      for (int i = 0; i < 4; i++) w[k][j][i] = k1[k] * k1[j] * k1[i] / 512.f;
#pragma omp parallel for schedule(static)
  for (int32_t t = 0; t < nActive; t++) {
    const int32_t bid = activeBids[t];
    const int bx = bid % g->nbx, by = (bid / g->nbx) % g->nby, bz = bid / (g->nbx * g->nby);
    for (int vz = 0; vz < cb; vz++)
      for (int vy = 0; vy < cb; vy++)
        for (int vx = 0; vx < cb; vx++) {
          const int x0 = bx * bs + 2 * vx, y0 = by * bs + 2 * vy, z0 = bz * bs + 2 * vz;
          float val;
          if (simpleAverage) {
            float sum = 0.f;
            for (int c = 0; c < 8; c++) {  /* iv0..iv7: x fastest, then y, then z */
              const float f = ds_fetch(g, slot, payload, x0 + (c & 1), y0 + ((c >> 1) & 1), z0 + (c >> 2));
              sum = c == 0 ? f : sum + f;
            }
            val = sum * (1.f / 8.f);
          } else {
            float S[4][4] = {{0.f}};
            for (int k = 0; k < 4; k++)
              for (int j = 0; j < 4; j++)
                for (int i = 0; i < 4; i++)
                  S[j][i] = fmaf(w[k][j][i], ds_fetch(g, slot, payload, x0 - 1 + i, y0 - 1 + j, z0 - 1 + k),
                                 S[j][i]);
            float T[4];
            for (int i = 0; i < 4; i++) T[i] = ((S[0][i] + S[1][i]) + S[2][i]) + S[3][i];
            val = (T[0] + T[1]) + (T[2] + T[3]);
          }
          out[(int64_t)t * cb * cb * cb + ((int64_t)vz * cb + vy) * cb + vx] = val;
        }
  }
}

/* ---- grid-to-particle interpolation ---------------------------------------------- */

/* The stored value at a voxel as a float, without the uint16 density scale. */
static float ip_raw(const orc_grid *g, const int32_t *slot, const void *payload, int x, int y, int z) {
  const int bs = g->bsx, L = ilog2(bs), m = bs - 1;
  const int64_t bid = (int64_t)(x >> L) + (int64_t)(y >> L) * g->nbx + (int64_t)(z >> L) * g->nbx * g->nby;
  const int32_t s = slot[bid];
  if (s < 0) return (float)g->emptyValue;
  const int64_t i = (int64_t)s * bs * bs * bs + (((z & m) * bs + (y & m)) << L) + (x & m);
  switch (g->storage) {
    case ORC_F32: return ((const float *)payload)[i];
    case ORC_U16: return (float)((const uint16_t *)payload)[i];
    case ORC_F16: return orc_f16_to_f32(((const uint16_t *)payload)[i]);
    default: return (float)((const double *)payload)[i];
  }
}

static inline float ip_lerp(float t, float a, float b) { return fmaf(b - a, t, a); }
static inline float ip_lin(float p0, float p1, float t) { return fmaf(p1, t, p0 * (1.0f - t)); }

/* One point of orc_interpolate. */
static float ip_point(const orc_grid *g, const int32_t *slot, const void *payload, const float p[3], int opt) {
  const float po = (opt & ORC_IP_CORNER) ? 0.0f : 0.5f;
  const int dom[3] = {g->sx, g->sy, g->sz};
  float pos[3], t[3];
  int ip[3], inside = 1;
  for (int a = 0; a < 3; a++) {
    pos[a] = p[a] - po;
    const float pf = floorf(pos[a]);
    ip[a] = (int)pf;
    t[a] = pos[a] - pf;
    if (!(ip[a] >= 0 && ip[a] < dom[a] - 1)) inside = 0;
  }
  float c[8];
  float val;
  if (inside) {
    for (int i = 0; i < 8; i++) c[i] = ip_raw(g, slot, payload, ip[0] + (i & 1), ip[1] + ((i >> 1) & 1), ip[2] + (i >> 2));
    const float a0 = ip_lerp(t[0], c[0], c[1]), a1 = ip_lerp(t[0], c[2], c[3]);
    const float a2 = ip_lerp(t[0], c[4], c[5]), a3 = ip_lerp(t[0], c[6], c[7]);
    const float b0 = ip_lerp(t[1], a0, a1), b1 = ip_lerp(t[1], a2, a3);
    val = ip_lerp(t[2], b0, b1);
  } else if (opt & ORC_IP_BC_DIRICHLET_OLD) {
    val = (float)g->emptyValue;
  } else {
    for (int i = 0; i < 8; i++) {
      int cc[3] = {ip[0] + (i & 1), ip[1] + ((i >> 1) & 1), ip[2] + (i >> 2)}, clipped = 0;
      for (int a = 0; a < 3; a++) {
        if (cc[a] < 0) { cc[a] = 0; clipped = 1; }
        if (cc[a] >= dom[a]) { cc[a] = dom[a] - 1; clipped = 1; }
      }
      c[i] = ((opt & ORC_IP_BC_DIRICHLET) && clipped) ? (float)g->emptyValue
                                                      : ip_raw(g, slot, payload, cc[0], cc[1], cc[2]);
    }
    const float a0 = ip_lin(c[0], c[1], t[0]), a1 = ip_lin(c[2], c[3], t[0]);
    const float a2 = ip_lin(c[4], c[5], t[0]), a3 = ip_lin(c[6], c[7], t[0]);
    const float b0 = ip_lin(a0, a1, t[1]), b1 = ip_lin(a2, a3, t[1]);
    val = ip_lin(b0, b1, t[2]);
  }
  if ((opt & ORC_IP_RENDER_DENS) && g->storage == ORC_U16) val *= kU16ToF;
  return val;
}

void orc_interpolate(const orc_grid *g, const int32_t *slot, const void *payload, const float *pts,
                     int64_t n, int opt, float *out) {
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < n; k++) out[k] = ip_point(g, slot, payload, pts + 3 * k, opt);
}

/* ---- ray-march render (src/render.h:52-160, src/render.cpp:20-101) ---- */

typedef struct { double x, y, z; } rv3;
static inline rv3 rv(double x, double y, double z) { rv3 r = {x, y, z}; return r; }
static inline rv3 rsub(rv3 a, rv3 b) { return rv(a.x - b.x, a.y - b.y, a.z - b.z); }
/* dot(a, b) = a.x*b.x + a.y*b.y + a.z*b.z, contracted left to right */
static inline double rdot(rv3 a, rv3 b) { return fma(a.z, b.z, fma(a.y, b.y, a.x * b.x)); }
static inline rv3 rnormalize(rv3 v, int opt) {
  const double len = sqrt(rdot(v, v));
  if (!(len > (double)1e-20f)) return rv(0, 1, 0);
  if (opt & ORC_RENDER_RECIP) {
    const double r = 1.0 / len;
    return rv(v.x * r, v.y * r, v.z * r);
  }
  return rv(v.x / len, v.y / len, v.z / len);
}
/* cross(a, b): a.y*b.z - a.z*b.y, ... contracted as fma(a.y, b.z, -(a.z*b.y)) */
static inline rv3 rcross(rv3 a, rv3 b) {
  return rv(fma(a.y, b.z, -(a.z * b.y)), fma(a.z, b.x, -(a.x * b.z)), fma(a.x, b.y, -(a.y * b.x)));
}

typedef struct {
  const orc_grid *g;
  const int32_t *slot;
  const void *payload;
  float res;
  float domMin[3], domMax[3];
} rnd_ctx;

/* sampleDensity (src/render.h:89-117) */
static double rnd_density(const rnd_ctx *c, rv3 p) {
  const float q[3] = {c->res * (float)p.x, c->res * (float)p.y, c->res * (float)p.z};
  const int dom[3] = {c->g->sx, c->g->sy, c->g->sz};
  int ip[3];
  for (int a = 0; a < 3; a++) {
    ip[a] = (int)floorf(q[a]);
    if (ip[a] < 0 || ip[a] > dom[a] - 1) return 0.0;
  }
  const int bs = c->g->bsx;
  const int64_t bid = (int64_t)(ip[0] / bs) + (int64_t)(ip[1] / bs) * c->g->nbx +
                      (int64_t)(ip[2] / bs) * c->g->nbx * c->g->nby;
  if (c->slot[bid] < 0) return 0.0;  /* skip fast over empty blocks */
  return (double)ip_point(c->g, c->slot, c->payload, q, ORC_IP_RENDER_DENS);
}

/* MtCubicBSplineWeights1D (src/mtool.h:344-362) */
static void bspline3(float t, float w[4], float d[4]) {
  const float s = 1.0f - t;
  w[0] = (1.0f / 6.0f) * s * s * s;
  w[1] = (2.0f / 3.0f) - 0.5f * t * t * (2.0f - t);
  w[2] = (2.0f / 3.0f) - 0.5f * s * s * (1.0f + t);
  w[3] = (1.0f / 6.0f) * t * t * t;
  d[0] = -s * s / 2.0f;
  d[1] = 0.5f * t * t - 1.0f * (2.0f - t) * t;
  d[2] = 1.0f * s * (t + 1.0f) - 0.5f * s * s;
  d[3] = t * t / 2.0f;
}

/* sampleDensityGradient (src/render.h:119-132): minus the gradient of the cubic
 * B-spline interpolant, interpolateWithDerivs0<IP_BSPLINE_CUBIC> (src/sbg.h:3903-4133)
 * with options 0: a window voxel outside the domain is clamped to it, a block without
 * payload reads emptyValue; uint16 scaled by 1/65535. */
static rv3 rnd_gradient(const rnd_ctx *c, rv3 p) {
  const float q[3] = {c->res * (float)p.x, c->res * (float)p.y, c->res * (float)p.z};
  for (int a = 0; a < 3; a++)
    if (q[a] < c->domMin[a] || q[a] > c->domMax[a]) return rv(-0.0, -0.0, -0.0);
  const int dom[3] = {c->g->sx, c->g->sy, c->g->sz};
  float t[3], w[3][4], d[3][4];
  int i0[3];
  for (int a = 0; a < 3; a++) {
    const float pos = q[a] - 0.5f, pf = floorf(pos);
    t[a] = pos - pf;
    i0[a] = (int)pf - 1;
    bspline3(t[a], w[a], d[a]);
  }
  float gx = 0, gy = 0, gz = 0;
  for (int dz = 0; dz < 4; dz++)
    for (int dy = 0; dy < 4; dy++)
      for (int dx = 0; dx < 4; dx++) {
        int cc[3] = {i0[0] + dx, i0[1] + dy, i0[2] + dz};
        for (int a = 0; a < 3; a++) cc[a] = cc[a] < 0 ? 0 : cc[a] >= dom[a] ? dom[a] - 1 : cc[a];
        const float f = ip_raw(c->g, c->slot, c->payload, cc[0], cc[1], cc[2]);
        const float wyz = w[2][dz] * w[1][dy];
        gx = fmaf(wyz * d[0][dx], f, gx);
        gy = fmaf(w[2][dz] * d[1][dy] * w[0][dx], f, gy);
        gz = fmaf(d[2][dz] * w[1][dy] * w[0][dx], f, gz);
      }
  if (c->g->storage == ORC_U16) {
    gx *= kU16ToF;
    gy *= kU16ToF;
    gz *= kU16ToF;
  }
  return rv(-1.0 * (double)gx, -1.0 * (double)gy, -1.0 * (double)gz);
}

void orc_render(const orc_grid *g, const int32_t *slot, const void *payload, int width, int height,
                const orc_camera *cam, int opt, int32_t *pixels) {
  rnd_ctx c;
  c.g = g;
  c.slot = slot;
  c.payload = payload;
  domain_limits(g, c.domMin, c.domMax);
  const int res = g->sx > g->sy ? (g->sx > g->sz ? g->sx : g->sz) : (g->sy > g->sz ? g->sy : g->sz);
  c.res = (float)res;
  const double hstep = 1.0 / (double)res;
  const int maxSteps = (int)(2.0 / hstep);
  const double invW = 1.0 / (double)width, invH = 1.0 / (double)height;
  const double aspect = (double)width / (double)height;
  const rv3 camPos = rv(cam->pos[0], cam->pos[1], cam->pos[2]);
  const rv3 fwd = rnormalize(rsub(rv(cam->lookAt[0], cam->lookAt[1], cam->lookAt[2]), camPos), opt);
  const rv3 right = rnormalize(rcross(fwd, rv(0, 1, 0)), opt);
  const rv3 up = rcross(right, fwd);
  const rv3 sun = rv(cam->sun[0], cam->sun[1], cam->sun[2]);
  const double zoom = cam->zoom;
#pragma omp parallel for schedule(dynamic, 1)
  for (int y = 0; y < height; y++) {
    for (int x = 0; x < width; x++) {
      const double ndcX = fma((double)((float)x + 0.5f), invW, -0.5) * 2.0 * aspect;
      const double ndcY = fma(-(double)((float)y + 0.5f), invH, 0.5) * 2.0;
      const rv3 dir = rnormalize(rv(fma(up.x, ndcY, fma(right.x, ndcX, fwd.x * zoom)),
                                    fma(up.y, ndcY, fma(right.y, ndcX, fwd.y * zoom)),
                                    fma(up.z, ndcY, fma(right.z, ndcX, fwd.z * zoom))), opt);
      const rv3 inc = rv(dir.x * hstep, dir.y * hstep, dir.z * hstep);
      rv3 pos = camPos, prevPos = camPos, hitPos = camPos;
      double prev = rnd_density(&c, pos);
      int hit = 0;
      for (int step = 0; step < maxSteps; step++) {
        pos = rv(pos.x + inc.x, pos.y + inc.y, pos.z + inc.z);
        const double d = rnd_density(&c, pos);
        if (prev < 0.5 && d >= 0.5) {
          const double t = (0.5 - prev) / (d - prev);
          hitPos = rv(fma(pos.x - prevPos.x, t, prevPos.x), fma(pos.y - prevPos.y, t, prevPos.y),
                      fma(pos.z - prevPos.z, t, prevPos.z));
          hit = 1;
          break;
        }
        prev = d;
        prevPos = pos;
      }
      int32_t col = 0x02000000;
      if (hit) {
        const rv3 nrm = rnormalize(rnd_gradient(&c, hitPos), opt);
        const rv3 ld = rnormalize(rsub(sun, hitPos), opt);
        double diff = rdot(nrm, ld);
        diff = diff > 0.0 ? diff : 0.0;
        int ch[3];
        for (int k = 0; k < 3; k++) {
          double v = cam->color[k] * diff;
          v = v < 0.0 ? 0.0 : v > 1.0 ? 1.0 : v;
          ch[k] = (int)(uint8_t)(int)fma(v, 255.0, 0.5);
        }
        col = 0x02000000 | (ch[2] << 16) | (ch[1] << 8) | ch[0];
      }
      pixels[(int64_t)y * width + x] = col;
    }
  }
}

/* ---- cross-resolution halo fill (src/halo.cpp:266-479, src/halo.h:270-330) ---- */

/* A constant block's voxel value as stored, read back as a float. */
static float lg_const(const orc_grid *g, float v) {
  switch (g->storage) {
    case ORC_U16: return (float)u16_rha(v) * kU16ToF;
    case ORC_F16: return orc_f16_to_f32(orc_f32_to_f16(v));
    default: return v;
  }
}

/* Value of voxel (x, y, z) of level l, or 0 in *found when that block does not exist
 * at level l.  (x, y, z) must lie inside the level's domain. */
static float lg_value(const orc_grid *g, const orc_level_grid *lg, int l, int x, int y, int z,
                      int *found) {
  const int bs = g->bsx >> l;
  const int64_t bid = (int64_t)(x / bs) + (int64_t)(y / bs) * g->nbx + (int64_t)(z / bs) * g->nbx * g->nby;
  const int32_t st = lg[l].state[bid];
  *found = st != ORC_LBLK_NONE;
  if (st == ORC_LBLK_NONE) return 0.0f;
  if (st == ORC_LBLK_EMPTY) return lg_const(g, lg[l].emptyValue);
  if (st == ORC_LBLK_FULL) return lg_const(g, lg[l].fullValue);
  const int64_t i = (int64_t)st * bs * bs * bs + ((int64_t)(z % bs) * bs + (y % bs)) * bs + (x % bs);
  switch (g->storage) {
    case ORC_F32: return ((const float *)lg[l].payload)[i];
    case ORC_U16: return (float)((const uint16_t *)lg[l].payload)[i] * kU16ToF;
    case ORC_F16: return orc_f16_to_f32(((const uint16_t *)lg[l].payload)[i]);
    default: return (float)((const double *)lg[l].payload)[i];
  }
}

static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : v > hi ? hi : v; }

int64_t orc_fill_halo(const orc_grid *g, int nLevels, const int32_t *levels,
                      const orc_level_grid *lg, int level, const int32_t *bids, int64_t nBids,
                      int haloSize, unsigned opt, float *out) {
  const int bs = g->bsx >> level, h = haloSize, hs = bs + 2 * h;
  const int s[3] = {g->sx >> level, g->sy >> level, g->sz >> level};
  const int64_t per = (int64_t)hs * hs * hs;
  int64_t skipped = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : skipped)
  for (int64_t k = 0; k < nBids; k++) {
    const int32_t bid = bids[k];
    float *dst = out + k * per;
    if (levels[bid] != level || lg[level].state[bid] == ORC_LBLK_NONE) {
      skipped++;
      continue;
    }
    const int b[3] = {bid % g->nbx, (bid / g->nbx) % g->nby, bid / (g->nbx * g->nby)};
    const int o[3] = {b[0] * bs, b[1] * bs, b[2] * bs};
    for (int hz = 0; hz < hs; hz++)
      for (int hy = 0; hy < hs; hy++)
        for (int hx = 0; hx < hs; hx++) {
          int p[3] = {o[0] + hx - h, o[1] + hy - h, o[2] + hz - h};
          const int inRange = p[0] >= 0 && p[0] < s[0] && p[1] >= 0 && p[1] < s[1] && p[2] >= 0 && p[2] < s[2];
          int found = 0;
          float v = 0.0f;
          if (inRange) v = lg_value(g, lg, level, p[0], p[1], p[2], &found);
          if (!found) {
            if (opt & ORC_BC_NEUMANN) {
              v = lg_value(g, lg, level, clampi(p[0], o[0], o[0] + bs - 1), clampi(p[1], o[1], o[1] + bs - 1),
                           clampi(p[2], o[2], o[2] + bs - 1), &found);
            } else if (opt & ORC_BC_COARSE_LEVEL) {
              if (!inRange) {
                for (int a = 0; a < 3; a++) p[a] = clampi(p[a], 0, s[a] - 1);
                v = lg_value(g, lg, level, p[0], p[1], p[2], &found);
              }
              if (!found) {
                v = lg_const(g, lg[level].emptyValue);
                if (level + 1 < nLevels) {
                  int c[3];
                  for (int a = 0; a < 3; a++) c[a] = clampi(p[a] / 2, 0, (s[a] >> 1) - 1);
                  const float vc = lg_value(g, lg, level + 1, c[0], c[1], c[2], &found);
                  if (found) v = vc;
                }
              }
            } else {
              v = lg_const(g, lg[level].emptyValue);
            }
          }
          dst[((int64_t)hz * hs + hy) * hs + hx] = v;
        }
  }
  return skipped;
}

/* ---- Morton order (src/msbg2.cpp:46-58, src/fastmath.h:290-316) ---- */

static uint64_t split3(uint64_t x) {
  x &= 0x1fffff;
  x = (x | x << 32) & 0x1f00000000ffffull;
  x = (x | x << 16) & 0x1f0000ff0000ffull;
  x = (x | x << 8) & 0x100f00f00f00f00full;
  x = (x | x << 4) & 0x10c30c30c30c30c3ull;
  x = (x | x << 2) & 0x1249249249249249ull;
  return x;
}

uint64_t orc_morton64(uint32_t x, uint32_t y, uint32_t z) {
  return split3(x) | (split3(y) << 1) | (split3(z) << 2);
}

typedef struct { uint64_t key; int32_t bid; } mkey;

static int mkey_cmp(const void *a, const void *b) {
  const uint64_t ka = ((const mkey *)a)->key, kb = ((const mkey *)b)->key;
  return ka < kb ? -1 : ka > kb ? 1 : 0;
}

void orc_sort_blocks_morton(int nbx, int nby, int nbz, int32_t *bids, int64_t n) {
  (void)nbz;
  mkey *k = (mkey *)malloc(sizeof(mkey) * (size_t)(n > 0 ? n : 1));
  for (int64_t i = 0; i < n; i++) {
    const int32_t b = bids[i];
    k[i].key = orc_morton64((uint32_t)(b % nbx), (uint32_t)((b / nbx) % nby), (uint32_t)(b / (nbx * nby)));
    k[i].bid = b;
  }
  qsort(k, (size_t)n, sizeof(mkey), mkey_cmp);
  for (int64_t i = 0; i < n; i++) bids[i] = k[i].bid;
  free(k);
}

/* ---- restriction of multi-level blocks (src/msbg4.cpp:1035-1379) ---- */

int64_t orc_restrict_level(const orc_grid *g, int nLevels, const int32_t *levels,
                           const orc_level_grid *lg, int level, const int32_t *bids, int64_t nBids,
                           int simpleAverage, float *out) {
  const int bs = g->bsx >> level, cb = bs / 2, hs = bs + 2;
  const int64_t box = (int64_t)hs * hs * hs, per = (int64_t)cb * cb * cb;
  float *boxes = (float *)malloc(sizeof(float) * (size_t)(nBids > 0 ? nBids : 1) * (size_t)box);
  const int64_t skipped = orc_fill_halo(g, nLevels, levels, lg, level, bids, nBids, 1, ORC_BC_COARSE_LEVEL, boxes);
  const float k1[4] = {1.f, 3.f, 3.f, 1.f};
  float w[4][4][4];
  for (int k = 0; k < 4; k++)
    for (int j = 0; j < 4; j++)
      for (int i = 0; i < 4; i++) w[k][j][i] = k1[k] * k1[j] * k1[i] / 512.f;
#pragma omp parallel for schedule(static)
  for (int64_t t = 0; t < nBids; t++) {
    const int32_t bid = bids[t];
    if (levels[bid] != level || lg[level].state[bid] == ORC_LBLK_NONE) continue;
    const float *b = boxes + t * box;
    /* fine cell (x, y, z) of the block, -1 .. bs */
#define BOX(x, y, z) b[((int64_t)((z) + 1) * hs + ((y) + 1)) * hs + ((x) + 1)]
    for (int vz = 0; vz < cb; vz++)
      for (int vy = 0; vy < cb; vy++)
        for (int vx = 0; vx < cb; vx++) {
          const int x0 = 2 * vx, y0 = 2 * vy, z0 = 2 * vz;
          float val;
          if (simpleAverage) {
            float sum = 0.f;
            for (int c = 0; c < 8; c++) {
              const float f = BOX(x0 + (c & 1), y0 + ((c >> 1) & 1), z0 + (c >> 2));
              sum = c == 0 ? f : sum + f;
            }
            val = sum * (1.f / 8.f);
          } else {
            float S[4][4] = {{0.f}};
            for (int k = 0; k < 4; k++)
              for (int j = 0; j < 4; j++)
                for (int i = 0; i < 4; i++) S[j][i] = fmaf(w[k][j][i], BOX(x0 - 1 + i, y0 - 1 + j, z0 - 1 + k), S[j][i]);
            float T[4];
            for (int i = 0; i < 4; i++) T[i] = ((S[0][i] + S[1][i]) + S[2][i]) + S[3][i];
            val = (T[0] + T[1]) + (T[2] + T[3]);
          }
          out[t * per + ((int64_t)vz * cb + vy) * cb + vx] = val;
        }
#undef BOX
  }
  free(boxes);
  return skipped;
}

/* ---- the reference's block smoother (src/msbg3.cpp:1108-1332, 2170-2369) ---------- */

/* One block: halo buffer hb [(bs+2)^3], x-fastest, position (i+1, j+1, k+1) for cell
 * (i, j, k) of the block; then blockIter in-place iterations; the last one into x. */
static void relax_ref_block(int nx, int ny, int nz, int bs, float *x, const float *b, const float *cx,
                            const float *cy, const float *cz, const float *dinv, int bx, int by, int bz,
                            int reverse, int blockIter, float omega, float *hb) {
  const int hs = bs + 2, hs2 = hs * hs;
  const int64_t sxy = (int64_t)nx * ny;
  const int ox = bx * bs, oy = by * bs, oz = bz * bs;
  for (int k = -1; k <= bs; k++)
    for (int j = -1; j <= bs; j++)
      for (int i = -1; i <= bs; i++) {
        const int gx = ox + i, gy = oy + j, gz = oz + k;
        const int out = (i < 0) + (i >= bs) + (j < 0) + (j >= bs) + (k < 0) + (k >= bs);
        float v = 0.0f;
        /* own cells and the face-neighbour layers; edges and corners are never read */
        if (out <= 1 && gx >= 0 && gy >= 0 && gz >= 0 && gx < nx && gy < ny && gz < nz)
          v = x[gz * sxy + (int64_t)gy * nx + gx];
        hb[(k + 1) * hs2 + (j + 1) * hs + (i + 1)] = v;
      }
  /* upper-face coefficient of a cell: the lower face of the next cell (0 past the
     domain, as the reference's zero block there) */
  const float oneMinusOmega = 1.0f - omega;
  /* the reference's SIMD width for the block edge (src/msbg3.cpp:1688-1745): 8 for edges
     16 and 8, the edge itself below; edge 32 (which the reference does not handle)
     takes 8 */
  const int gw = bs >= 8 ? 8 : bs;
  const int G = bs / gw;
  float y[8];
  for (int it = 0; it < blockIter; it++) {
    const int backward = (it & 1) == (reverse ? 1 : 0);
    const int last = it == blockIter - 1;
    for (int s = 0; s < bs * bs * G; s++) {
      const int q = backward ? bs * bs * G - 1 - s : s;
      const int g = q % G, j = (q / G) % bs, k = q / (G * bs);
      for (int l = 0; l < gw; l++) {
        const int i = gw * g + l;
        const int gx = ox + i, gy = oy + j, gz = oz + k;
        const int64_t c = gz * sxy + (int64_t)gy * nx + gx;
        const float *p = hb + (k + 1) * hs2 + (j + 1) * hs + (i + 1);
        const float F0 = p[0], F1 = p[-1], F2 = p[1], F3 = p[-hs], F4 = p[hs], F5 = p[-hs2], F6 = p[hs2];
        const float W1 = cx[c], W2 = gx + 1 < nx ? cx[c + 1] : 0.0f;
        const float W3 = cy[c], W4 = gy + 1 < ny ? cy[c + nx] : 0.0f;
        const float W5 = cz[c], W6 = gz + 1 < nz ? cz[c + sxy] : 0.0f;
        float S = 0.0f;
        S = fmaf(F1, W1, S);
        S = fmaf(F2, W2, S);
        S = fmaf(F3, W3, S);
        S = fmaf(F4, W4, S);
        S = fmaf(F5, W5, S);
        S = fmaf(F6, W6, S);
        /* omega (B + S) D + (1 - omega) F0 as the reference's build (-O3 -ffast-math
           -march=native) evaluates it in its 8-wide path: t = S + B, then one fused
           multiply-add with (omega D) t; this matches its output bit for bit */
        const float t = S + b[c];
        y[l] = fmaf(oneMinusOmega, F0, (omega * dinv[c]) * t);
      }
      for (int l = 0; l < gw; l++) {
        const int i = gw * g + l;
        if (last)
          x[(oz + k) * sxy + (int64_t)(oy + j) * nx + ox + i] = y[l];
        else
          hb[(k + 1) * hs2 + (j + 1) * hs + (i + 1)] = y[l];
      }
    }
  }
}

void orc_relax_ref(int nx, int ny, int nz, int bs, float *x, const float *b, const float *cx,
                   const float *cy, const float *cz, const float *dinv, const int32_t *bids, int64_t n,
                   int passes, int reverse, int blockIter, float omega) {
  const int nbx = nx / bs, nby = ny / bs;
  const int hs = bs + 2;
  for (int pass = 0; pass < passes; pass++)
    for (int rb = 0; rb < 2; rb++) {
#pragma omp parallel
      {
        float *hb = (float *)malloc(sizeof(float) * hs * hs * hs);
#pragma omp for schedule(dynamic, 4)
        for (int64_t t = 0; t < n; t++) {
          const int bid = bids[t];
          const int bx = bid % nbx, by = (bid / nbx) % nby, bz = bid / (nbx * nby);
          int skip = ((bx + by + bz) & 1) == rb;
          if (reverse) skip = !skip;
          if (skip) continue;
          relax_ref_block(nx, ny, nz, bs, x, b, cx, cy, cz, dinv, bx, by, bz, reverse, blockIter, omega, hb);
        }
        free(hb);
      }
    }
}

/* ---- the solver's halo (src/halo.cpp:536-738) ------------------------------------- */

static uint16_t lf_value(const orc_grid *g, const orc_flag_grid *lf, int l, int x, int y, int z) {
  const int bs = g->bsx >> l;
  const int64_t bid = (int64_t)(x / bs) + (int64_t)(y / bs) * g->nbx + (int64_t)(z / bs) * g->nbx * g->nby;
  const int32_t st = lf[l].state[bid];
  if (st == ORC_LBLK_EMPTY) return lf[l].emptyFlags;
  if (st == ORC_LBLK_FULL) return lf[l].fullFlags;
  if (st < 0) return 0;
  return lf[l].payload[(int64_t)st * bs * bs * bs + ((int64_t)(z % bs) * bs + (y % bs)) * bs + (x % bs)];
}

int64_t orc_fill_halo3(const orc_grid *g, int nLevels, const int32_t *levels, const orc_level_grid *lg,
                       const orc_flag_grid *lf, const int32_t *bids, int64_t nBids, const int32_t *dbc,
                       float *out) {
  const float kDirichlet = 1e20f, kNeumann = -1e20f; /* SPEC_FLOAT_*, src/msbgcell.h:199-200 */
  const int bs = g->bsx, hs = bs + 2;
  const int s[3] = {g->sx, g->sy, g->sz};
  const int64_t per = (int64_t)hs * hs * hs;
  int64_t skipped = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : skipped)
  for (int64_t k = 0; k < nBids; k++) {
    const int32_t bid = bids[k];
    float *dst = out + k * per;
    if (levels[bid] != 0 || nLevels < 2) {
      skipped++;
      continue;
    }
    const int o[3] = {(bid % g->nbx) * bs, ((bid / g->nbx) % g->nby) * bs, (bid / (g->nbx * g->nby)) * bs};
    for (int hz = 0; hz < hs; hz++)
      for (int hy = 0; hy < hs; hy++)
        for (int hx = 0; hx < hs; hx++) {
          const int p[3] = {o[0] + hx - 1, o[1] + hy - 1, o[2] + hz - 1};
          float v;
          int side = -1; /* the face p leaves through: x decides before y before z */
          for (int a = 2; a >= 0; a--)
            if (p[a] < 0 || p[a] >= s[a]) side = 2 * a + (p[a] >= s[a]);
          if (side < 0) {
            const int64_t b2 = (int64_t)(p[0] / bs) + (int64_t)(p[1] / bs) * g->nbx +
                               (int64_t)(p[2] / bs) * g->nbx * g->nby;
            const int l = levels[b2] == 0 ? 0 : 1;
            const int q[3] = {p[0] >> l, p[1] >> l, p[2] >> l};
            const uint16_t f = lf_value(g, lf, l, q[0], q[1], q[2]);
            int found;
            v = (f & ORC_CELL_VOID) ? kDirichlet
                : (f & ORC_CELL_SOLID) ? kNeumann
                                        : lg_value(g, lg, l, q[0], q[1], q[2], &found);
          } else {
            v = dbc[side] == 0 ? kDirichlet : kNeumann;
          }
          dst[((int64_t)hz * hs + hy) * hs + hx] = v;
        }
  }
  return skipped;
}

/* ---- setRefinementMap: the fine-coarse distance channel (src/msbg.cpp:1887-2033) ---- */

int64_t orc_dist_fine_coarse(const int32_t *levels, const uint16_t *flags, int nbx, int nby, int nbz, int bsx,
                             int level, int dTransRes, int32_t *state, uint16_t *data) {
  const int64_t nB = (int64_t)nbx * nby * nbz;
  const int bs = bsx >> level;
  const uint16_t kFineCoarse = 1u << 3; /* BLK_FINE_COARSE, src/msbg.h:561-573 */
  int64_t n = 0;
  for (int64_t b = 0; b < nB; b++) {
    state[b] = ORC_LBLK_EMPTY;
    if (levels[b] == level && (flags[b] & kFineCoarse)) state[b] = (int32_t)n++;
  }
  for (int64_t b = 0; b < nB; b++) {
    const int bx = (int)(b % nbx), by = (int)((b / nbx) % nby), bz = (int)(b / ((int64_t)nbx * nby));
    if (state[b] >= 0) {
      float box[26][3];
      int nbox = 0;
      for (int dz = -1; dz <= 1; dz++)
        for (int dy = -1; dy <= 1; dy++)
          for (int dx = -1; dx <= 1; dx++) {
            const int x = bx + dx, y = by + dy, z = bz + dz;
            if ((!dx && !dy && !dz) || x < 0 || y < 0 || z < 0 || x >= nbx || y >= nby || z >= nbz) continue;
            if (levels[((int64_t)z * nby + y) * nbx + x] <= level) continue;
            box[nbox][0] = (float)x; box[nbox][1] = (float)y; box[nbox][2] = (float)z;
            nbox++;
          }
      uint16_t *d = data + state[b] * (int64_t)bs * bs * bs;
      int vid = 0;
      for (int z1 = bz * bs; z1 < (bz + 1) * bs; z1++)
        for (int y1 = by * bs; y1 < (by + 1) * bs; y1++)
          for (int x1 = bx * bs; x1 < (bx + 1) * bs; x1++, vid++) {
            const float p[3] = {x1 + 0.5f, y1 + 0.5f, z1 + 0.5f};
            float d2 = 1e20f;
            for (int i = 0; i < nbox; i++) { /* distToBoxSq, src/msbg.h:3874-3886 */
              float s2 = 0.0f;
              for (int a = 0; a < 3; a++) {
                const float lo = box[i][a] * (float)bs - p[a], hi = p[a] - (box[i][a] + 1.0f) * (float)bs;
                float m = lo > 0.0f ? lo : 0.0f;
                m = m > hi ? m : hi;
                s2 += m * m;
              }
              d2 = d2 < s2 ? d2 : s2;
            }
            float dist = sqrtf(d2);
            if (dist < 0.0f || dist > (float)dTransRes) dist = (float)dTransRes;
            d[vid] = (uint16_t)(dist * 1024.0f);
          }
    } else if (levels[b] <= level && levels[b] >= level - 1) {
      for (int dz = -1; dz <= 1 && state[b] == ORC_LBLK_EMPTY; dz++)
        for (int dy = -1; dy <= 1; dy++)
          for (int dx = -1; dx <= 1; dx++) {
            const int x = bx + dx, y = by + dy, z = bz + dz;
            if ((!dx && !dy && !dz) || x < 0 || y < 0 || z < 0 || x >= nbx || y >= nby || z >= nbz) continue;
            const int64_t b2 = ((int64_t)z * nby + y) * nbx + x;
            if (levels[b2] == level && (flags[b2] & kFineCoarse)) state[b] = ORC_LBLK_FULL;
          }
    }
  }
  return n;
}
