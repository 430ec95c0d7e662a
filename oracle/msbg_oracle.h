/*
 * CPU restatement of the MSBG hot path (test infrastructure only).
 *
 * This is the checker the GPU library is compared against: plain C (+OpenMP),
 * portable to x86-64 and aarch64, and itself pinned against the reference
 * library built from its own sources (oracle/_ref, x86 only) by the tests.
 * Nothing in the GPU product links or calls it.
 *
 * Data layout (the same one the GPU library uses, so results compare directly):
 *   block id     bid = bx + by*nbx + bz*nbx*nby            (src/sbg.h:1744-1749)
 *   voxel index  vid = x + y*bs + z*bs*bs inside a block   (src/sbg.h:1816-1820)
 *   slot[bid]    >= 0: index of the block's payload in a dense slab of
 *                [nActive][bs^3] values; -1: the shared constant "empty" block
 *                whose every voxel reads emptyValue (src/sbg.h:2042-2047).
 */
#ifndef MSBG_ORACLE_H
#define MSBG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Storage types of a payload slab. */
enum { ORC_F32 = 0, ORC_U16 = 1, ORC_F16 = 2, ORC_F64 = 3 };

/* Block flags, same bit values as src/msbg.h:561-573. */
enum {
  ORC_BLK_DOM_BORDER = 1 << 1,
  ORC_BLK_COARSE_FINE = 1 << 2,
  ORC_BLK_FINE_COARSE = 1 << 3,
  ORC_BLK_EXISTS = 1 << 12,
  ORC_BLK_UNIFORM_EMPTY = 1 << 13
};

typedef struct {
  int32_t sx, sy, sz;   /* voxels at the finest level */
  int32_t bsx;          /* block edge (power of two)  */
  int32_t nbx, nby, nbz;
  int32_t storage;      /* ORC_* */
  double emptyValue;    /* value of every voxel of a constant empty block */
} orc_grid;

void orc_grid_init(orc_grid *g, int sx, int sy, int sz, int bsx, int storage);

/* ---- active-block marking and per-block particle buckets ------------------
 * src/msbg_demo.cpp:339-397.  valid[i]=1 for points that pass the domain tests;
 * blockCount[bid] += 1 for every block of the point's rScan box.  Points are then
 * bucketed by the block that contains them: bucketStart[nBlocks+1] (prefix sums)
 * and bucketIdx[nValid] (point indices).  Returns the number of valid points. */
int64_t orc_mark_blocks(const orc_grid *g, const float *pts, int64_t n, float rScan,
                        int32_t *blockCount, uint8_t *valid);
void orc_bucket_points(const orc_grid *g, const float *pts, int64_t n, const uint8_t *valid,
                       int64_t *bucketStart, int64_t *bucketIdx);

/* Multi-band level assignment: level 0 for blocks in the rBand[0] box of any
 * point, level l for the rBand[l] box, nLevels-1 elsewhere (nBands <= nLevels-1). */
void orc_band_levels(const orc_grid *g, const float *pts, int64_t n, const uint8_t *valid,
                     const float *rBand, int nBands, int nLevels, int32_t *levels);

/* ---- refinement map --------------------------------------------------------
 * regularizeRefinementMap (src/msbg.cpp:1202-1423): at most one level jump
 * between 26-neighbours.  levelsOut may alias levelsIn.  perLevel[8] counts. */
void orc_regularize(const int32_t *levelsIn, int32_t *levelsOut, int nbx, int nby, int nbz,
                    int nLevels, int64_t *perLevel);
/* BlockInfo flags of setRefinementMap (src/msbg.cpp:1632-1720) for levelMg 0;
 * existsFlags may be NULL (no BLK_EXISTS). */
void orc_block_flags(const int32_t *levels, const uint16_t *existsFlags, uint16_t *flags,
                     int nbx, int nby, int nbz);

/* Level-0 blocks get slots in ascending bid order (src/msbg_demo.cpp:455-511).
 * Returns nActive; activeBids[nActive]. */
int32_t orc_build_slots(const int32_t *levels, int nBlocks, int32_t *slot, int32_t *activeBids);

/* Fill every active payload voxel with v. */
void orc_fill(const orc_grid *g, void *payload, int64_t nActive, double v);

/* ---- splat and finalize ----------------------------------------------------
 * 8-color splat of min(distSq/distSqMax) (src/msbg_demo.cpp:527-636) and the
 * distance-to-density finalize (src/msbg_demo.cpp:655-680).  A particle is
 * abandoned at its first in-sphere voxel that lies in a non-value block. */
int64_t orc_splat(const orc_grid *g, const float *pts, const int64_t *bucketStart,
                  const int64_t *bucketIdx, const int32_t *slot, const int32_t *activeBids,
                  int32_t nActive, void *payload, float rParticle, float nbDist);
void orc_finalize(const orc_grid *g, void *payload, int64_t nActive, float rParticle,
                  float nbDist);

/* ---- stencil sweeps: applyChannelPdeFast (src/msbg4.cpp:60-957) -----------
 * laplTyp as the reference takes it: negative = in-place colored schedule (with
 * OPT_8_COLOR_SCHEME = 1<<29: 8 colors, else red-black), positive = ping-pong.
 * Kernels: 4 MCF, 17 Jacobi diffusion, 15 Perona-Malik Jacobi, 14 Perona-Malik,
 * 3 simple diffusion, 1 Laplacian smoothing.  numIter is rounded up to even as
 * the reference does.  Math runs in float, or in double when storage==ORC_F64.
 * payloadTmp is needed for the ping-pong schedule only. */
int orc_pde(const orc_grid *g, const int32_t *slot, const int32_t *activeBids, int32_t nActive,
            void *payload, void *payloadTmp, int laplTyp, int constr01, int numIter, float dt,
            float anisAlpha);

/* ---- restriction to the next coarser multigrid level -------------------------
 * downsampleFloatChannelNew (src/msbg4.cpp:1035-1379) for the value blocks: coarse
 * cell v of a block (edge bs/2) = sum over the fine cells 2v-1 .. 2v+2 with weights
 * (1,3,3,1)^3/512 (src/grid.c:30-70); simpleAverage: the mean of the 8 children.
 * Fine halo as fillHaloBlock_ with OPT_BC_COARSE_LEVEL (src/halo.h:288-300): clamp to
 * the domain, empty blocks read emptyValue.  out: [nActive][(bs/2)^3] floats.
 * Summation order (FP32, one rounding per operation): per x offset i and row j,
 * S[j][i] = fma(w, f, S[j][i]) over the 4 planes; T[i] = ((S0+S1)+S2)+S3 over the
 * rows; value = (T0+T1)+(T2+T3) -- the reference's 4-wide accumulators and its
 * horizontal add.  The 8-child mean sums in the reference's order, then * 1/8. */
void orc_downsample(const orc_grid *g, const int32_t *slot, const int32_t *activeBids, int32_t nActive,
                    const void *payload, int simpleAverage, float *out);

/* ---- grid-to-particle interpolation (trilinear) ----------------------------
 * SparseGrid<float>::interpolateFloatFast (src/sbg.h:4623-4792) and
 * SparseGrid<uint16_t>::interpolateUint16ToFloatFast (src/sbg.h:4920-5032) at n points
 * pts[3i..3i+2] (voxel units; the voxel centre of cell i is i + 0.5).
 *  - pos = p - 0.5 (not with ORC_IP_CORNER); i = floor(pos); t = pos - i.
 *  - Corner values are the stored values as floats: FP32 as is, uint16 unscaled, FP16
 *    widened; a block without payload reads emptyValue.
 *  - Inside (0 <= i <= s-2 on every axis): lerp(t, a, b) = fma(b - a, t, a)
 *    (vlerp_ps, src/vectorclass_util.h:143-146) along x for the 4 corner pairs, then y,
 *    then z.
 *  - Otherwise the generic path interpolateGen0<IP_LINEAR> (src/sbg.h:3109-3246): corner
 *    coordinates clamped to the domain (ORC_IP_BC_DIRICHLET: a corner with a clamped
 *    coordinate reads emptyValue; ORC_IP_BC_DIRICHLET_OLD: the result is emptyValue),
 *    lerps in the same order as Interpolate1D (src/sbg.h:2934-2940), p1*t + p0*(1-t),
 *    which the reference's own flags (-O3 -ffast-math, FMA hardware) compile to
 *    fma(p1, t, p0*(1-t)).  That form is pinned against the compiled reference.
 *  - ORC_IP_RENDER_DENS (uint16 only): the value times 1/65535
 *    (interpolateRenderDensity, src/msbg.h:478-484).
 *  - ORC_IP_NO_BORDER_CHECK changes nothing for points inside the domain; the border
 *    test is always made. */
enum {
  ORC_IP_CORNER = 1 << 0,
  ORC_IP_BC_DIRICHLET = 1 << 13,
  ORC_IP_BC_DIRICHLET_OLD = 1 << 14,
  ORC_IP_NO_BORDER_CHECK = 1 << 15,
  ORC_IP_RENDER_DENS = 1 << 18
};
void orc_interpolate(const orc_grid *g, const int32_t *slot, const void *payload, const float *pts,
                     int64_t n, int opt, float *out);

/* ---- cross-resolution halo fill ------------------------------------------------
 * HaloBlockSet::fillHaloBlock_<T> (src/halo.cpp:266-479) with getOutOfBlockValue
 * (src/halo.h:270-330) on a multi-level channel.  Level l of the channel is the
 * reference's SparseGrid of resolution level l: block edge bsx>>l, domain sx>>l, the
 * same block grid (src/msbg.cpp:800-812).  lg[l].state[bid]: >= 0 index of the block's
 * payload in lg[l].payload ([n][(bsx>>l)^3] of g->storage); ORC_LBLK_EMPTY the
 * constant empty block, ORC_LBLK_FULL the constant full block (every voxel reads
 * emptyValue / fullValue); ORC_LBLK_NONE no block at this level (a NULL block map
 * entry).  For every listed block (its level levels[bid] must be `level`, and it must
 * have a block at that level) out receives the (bs+2h)^3 floats [z][y][x] of
 * positions origin-h .. origin+bs+h-1 in level coordinates:
 *  - a position inside the domain whose block exists at this level: that value;
 *  - otherwise, with ORC_BC_NEUMANN: the own block's value at the position clamped to
 *    the block;
 *  - otherwise, with ORC_BC_COARSE_LEVEL: a position outside the domain is clamped
 *    to it and read at this level if that block exists; else the position is halved
 *    (after the clamp) and read at level+1 (clamped to that level's domain);
 *  - otherwise the level's empty value.
 * A level+1 read with no block there, or from the coarsest level, gives the empty
 * value (the reference requires data there).  uint16 reads as v/65535, FP16 widened.
 * Returns the number of listed blocks that were skipped (wrong level, no own block). */
enum { ORC_LBLK_EMPTY = -1, ORC_LBLK_FULL = -2, ORC_LBLK_NONE = -3 };
enum { ORC_BC_NEUMANN = 1 << 10, ORC_BC_COARSE_LEVEL = 1 << 26 };
typedef struct {
  const int32_t *state;   /* [nBlocks] */
  const void *payload;    /* [n][(bsx>>l)^3] */
  float emptyValue, fullValue;
} orc_level_grid;
int64_t orc_fill_halo(const orc_grid *g, int nLevels, const int32_t *levels,
                      const orc_level_grid *lg, int level, const int32_t *bids, int64_t nBids,
                      int haloSize, unsigned opt, float *out);

/* Cell flags of one resolution level (the reference's CH_CELL_FLAGS grids): per-block
 * states as orc_level_grid, uint16 payload, and the constant blocks' flags. */
typedef struct {
  const int32_t *state;
  const uint16_t *payload; /* [n][(bsx>>l)^3] */
  uint16_t emptyFlags, fullFlags;
} orc_flag_grid;
enum { ORC_CELL_SOLID = 1 << 0, ORC_CELL_VOID = 1 << 12 }; /* src/msbg.h:602-614 */
/* HaloBlockSet::fillHaloBlock3 (src/halo.cpp:536-738) at multigrid level 0, halo 1, for the
 * listed blocks of layout level 0 (others skipped and counted): per position p of the
 * (bs+2)^3 box, in level-0 coordinates,
 *   p in the domain, its block at layout level 0: flags(0, p) & CELL_VOID -> +1e20
 *     (SPEC_FLOAT_DIRICHLET), & CELL_SOLID -> -1e20 (SPEC_FLOAT_NEUMANN), else value(0, p);
 *   p in the domain, its block coarser: the same with flags and value of level 1 at p/2
 *     (getOutOfBlockValue3, src/halo.cpp:536-562);
 *   p outside the domain: +1e20 when the face it leaves through is open (DBC_OPEN = 0),
 *     else -1e20; the x face decides before y before z (the 3x3x3 table,
 *     src/msbg.cpp:2527-2548).
 * dbc[6]: the domain boundary types of faces -x, +x, -y, +y, -z, +z. */
int64_t orc_fill_halo3(const orc_grid *g, int nLevels, const int32_t *levels, const orc_level_grid *lg,
                       const orc_flag_grid *lf, const int32_t *bids, int64_t nBids, const int32_t *dbc,
                       float *out);

/* ---- ray-march render of the iso-0.5 surface ----------------------------------
 * RDR::RaymarchRenderer (src/render.h:52-160, src/render.cpp:20-101): per pixel a
 * primary ray from the camera (FP64), stepped by 1/res (res = max(sx,sy,sz)) for at
 * most 2 units; the density at a point p is 0 outside the domain or in a block without
 * payload, else the trilinear interpolant at res*p (FP32; uint16 times 1/65535).  The
 * first step whose density crosses 0.5 upwards gives the hit, placed by linear
 * interpolation; its normal is minus the cubic B-spline gradient
 * (interpolateWithDerivs0<IP_BSPLINE_CUBIC>, src/sbg.h:3903-4133); Lambert shading
 * with the sun, colour channels rounded to 8 bits.  pixels[y*width+x] = BMP_MKRGB
 * (0x02000000 | b<<16 | g<<8 | r), 0x02000000 for a miss.  The gradient is taken
 * inside the grid's float domain box of SparseGrid::inRange(Vec4f) (src/sbg.cpp:262-316)
 * only; elsewhere the normal is (0, 1, 0).
 * opt bits select the floating-point forms the reference's -ffast-math build may
 * produce (ORC_RENDER_RECIP: v/len as v*(1/len)); 0 is the reference's as written,
 * with fused multiply-adds where the compiler contracts. */
typedef struct {
  double pos[3], lookAt[3], sun[3], color[3];
  double zoom;
} orc_camera;
enum { ORC_RENDER_RECIP = 1 };
void orc_render(const orc_grid *g, const int32_t *slot, const void *payload, int width, int height,
                const orc_camera *cam, int opt, int32_t *pixels);

/* ---- Morton order of block lists ---------------------------------------------------
 * MultiresSparseGrid::sortBlockListMorton (src/msbg2.cpp:46-58): ascending
 * FMA::morton64_encode of the block coordinates (src/fastmath.h:290-316: the bits of x,
 * y, z interleaved, x lowest).  Sorts bids[n] in place. */
uint64_t orc_morton64(uint32_t x, uint32_t y, uint32_t z);
void orc_sort_blocks_morton(int nbx, int nby, int nbz, int32_t *bids, int64_t n);

/* Restriction of blocks of a multi-level channel: downsampleFloatChannelNew
 * (src/msbg4.cpp:1035-1379) for each listed block at `level`: the (bs/2)^3 coarse values
 * of the block, from its fine halo box of orc_fill_halo with halo 1 and
 * ORC_BC_COARSE_LEVEL (the cross-resolution rule), with orc_downsample's weights and
 * summation order (or the 8-child mean).  out: [nBids][(bs/2)^3].  Returns the number of
 * skipped blocks (their output is left as is). */
int64_t orc_restrict_level(const orc_grid *g, int nLevels, const int32_t *levels,
                           const orc_level_grid *lg, int level, const int32_t *bids, int64_t nBids,
                           int simpleAverage, float *out);

/* ---- conversions (exposed for tests) ---- */
uint16_t orc_f32_to_f16(float f);
float orc_f16_to_f32(uint16_t h);

/* ---- sparse Poisson solve (FP64 restatement) ---------------------------------
 * Same operator, hierarchy, transfers, smoother and CG as the GPU solver, on dense
 * per-level arrays with an activity mask (x = 0 outside, Dirichlet):
 *   (A x)_i = d_i x_i - sum_f c_f x_nb(f)            (src/msbg3.cpp:1281-1296)
 * cx/cy/cz hold each cell's lower-face coefficient, d the diagonal.  Level l+1 has
 * ceil(n/2) cells per axis; a coarse cell is active when any child is; coarse
 * operator = P^T A P / 2 with piecewise-constant P.  Smoothing pass on a level of
 * block edge bs: tiles (TX,TY,TZ) = 32x16x8 (bs 32), 16^3 (bs 16) or 8^3 (bs 8)
 * coloured by (gx/TX+gy/TY+gz/TZ)&1, each tile colour in turn doing k in-tile
 * red-black Gauss-Seidel sweeps with the outside held fixed; pointwise red-black
 * GS (k sweeps) on levels with bs < 8.  Pre-smoothing: tile colours 0,1 and cells red
 * first; post-smoothing the adjoint order (1,0; black first).  Coarsest level:
 * exact solve (Cholesky) when coarsestIter == 0, else coarsestIter RB sweeps
 * from zero.  Levels: log2(bs0) halvings, then more while
 * the coarse level has more than coarsestCells active cells and a side longer
 * than 2. */
typedef struct {
  int nx, ny, nz;
  const uint8_t *act;  /* [nz][ny][nx] */
  const double *cx, *cy, *cz, *d;
} orc_level0;

/* Seeded face coefficients of level 0 in [0.5,2] (identical bits to the GPU). */
float orc_face_coeff(uint32_t seed, int axis, int gx, int gy, int gz);
void orc_poisson_apply(const orc_level0 *L, const double *x, const double *b, double *y, int residual);
void orc_poisson_rbgs(const orc_level0 *L, double *x, const double *b, int nSweeps, int redFirst);
/* passes smoothing passes of level 0 (block edge 1<<log2bs), k in-tile sweeps. */
void orc_poisson_smooth(const orc_level0 *L, int log2bs, double *x, const double *b, int passes, int k,
                        int reverse);
int orc_poisson_vcycle(const orc_level0 *L, int log2bs0, const double *b, double *x, int preSweeps,
                       int postSweeps, int tileIters, int coarsestIter, int64_t coarsestCells);
int orc_poisson_mgpcg(const orc_level0 *L, int log2bs0, const double *b, double *x, double tol,
                      int maxIter, int preSweeps, int postSweeps, int tileIters, int coarsestIter,
                      int64_t coarsestCells, int *iters, double *relres);
/* The reference's block smoother, FP32 on dense [nz][ny][nx] arrays (cells outside the
 * value blocks hold 0 in x): relax() (src/msbg3.cpp:2244-2369) calling relaxBlockList
 * (src/msbg3.cpp:2170-2239) `passes` times.  Each pass runs two half-passes over the
 * listed blocks (bids on the nx/bs x ny/bs x nz/bs block grid): blocks whose
 * (bx+by+bz)&1 differs from the half-pass index (the other parity first with reverse),
 * each with its face-neighbour halo taken at its start and blockIter block-local
 * iterations in place (IprocessBlockLaplacian, src/msbg3.cpp:1108-1332): groups of gw
 * x-consecutive cells updated together (gw = the reference's SIMD width, 8 for block
 * edges 8 and 16, the edge itself for 4 and 2, src/msbg3.cpp:1688-1745; 8 for edge 32,
 * which the reference does not handle),
 *   S = fma(F6,W6, ... fma(F1,W1, 0)),  Y = omega (B + S) D + (1 - omega) F0,
 * D = 1/diagonal (dinv), W the face coefficients (lower faces cx/cy/cz, upper faces the
 * next cell's); iteration i sweeps the groups backward when (i&1) == reverse, forward
 * otherwise; the last iteration writes to x instead of the block buffer, so it is a
 * Jacobi step. */
void orc_relax_ref(int nx, int ny, int nz, int bs, float *x, const float *b, const float *cx,
                   const float *cy, const float *cz, const float *dinv, const int32_t *bids, int64_t n,
                   int passes, int reverse, int blockIter, float omega);
/* setRefinementMap's fine-coarse distance channel CH_DIST_FINECOARSE at resolution level l
 * (src/msbg.cpp:1887-1960, 1994-2033) from the regularised level map and the BlockInfo
 * flags: every block of level l flagged BLK_FINE_COARSE is a value block (ascending id,
 * state[b] = its index) whose cell (x,y,z) (level-l coordinates) holds
 * uint16(1024 * min(dTransRes, sqrt(min over its 26-neighbours of level > l of
 * distToBoxSq(box, cell centre)))); a block of level l-1 or l that is no value block but has
 * a BLK_FINE_COARSE 26-neighbour of level l is full (state -2, value dTransRes*1024); other
 * blocks are empty (-1).  data: [n][(bsx>>l)^3]; returns n. */
int64_t orc_dist_fine_coarse(const int32_t *levels, const uint16_t *flags, int nbx, int nby, int nbz, int bsx,
                             int level, int dTransRes, int32_t *state, uint16_t *data);
/* The GPU's seeded coefficients (float values) on a dense grid: lower faces + diagonal. */
void orc_poisson_coeffs_dense(uint32_t seed, int nx, int ny, int nz, const uint8_t *act, double *cx,
                              double *cy, double *cz, double *d);

#ifdef __cplusplus
}
#endif
#endif

