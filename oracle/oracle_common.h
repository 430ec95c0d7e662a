/*
 * Shared binary job/result layout between the test harness (Python), the
 * reference-library driver (ref_driver.cpp, x86 only) and the project's C
 * restatement (msbg_oracle.c).  Test infrastructure only.
 *
 * A "surface job" reproduces the reference demo pipeline of
 * src/msbg_demo.cpp:228-727 on a caller-supplied point cloud:
 *   mark active blocks -> level map -> regularizeRefinementMap ->
 *   setRefinementMap -> allocate level-0 blocks (value 1.0) -> 8-color splat ->
 *   finalize -> applyChannelPdeFast (in-place 8-color or plain schedules).
 * A "levels job" runs regularizeRefinementMap + setRefinementMap on a given
 * per-block level map with the multi-level grid (src/msbg.cpp:1202-2165).
 * An "interp job" loads a given payload into the value blocks of a single-level
 * grid (every other block is the constant empty block, value 0) and interpolates
 * it at query points: SparseGrid<float>::interpolateFloatFast (src/sbg.h:4623-4792),
 * SparseGrid<uint16_t>::interpolateUint16ToFloatFast (src/sbg.h:4920-5032), or, with
 * ORACLE_IP_RENDER_DENS, MultiresSparseGrid::interpolateRenderDensity
 * (src/msbg.h:478-484, a free function: the uint16 value times 1/65535).
 * A "halo job" builds a multi-level grid on a given (regular) level map, loads every
 * resolution level of one channel with caller-given block states (payload block,
 * constant empty, constant full, or no block) and payloads, and dumps
 * HaloBlockSet::fillHaloBlock_<T> (src/halo.cpp:266-479) of every block at one level.
 * A "render job" loads a uint16 payload like the interp job and renders it with
 * RDR::RaymarchRenderer (src/render.h:52-160, src/render.cpp:20-101): the points are
 * camera position, look-at point, sun position, surface colour and (zoom, 0, 0);
 * nIter x laplTyp is the image size.
 * A "morton job" sorts a list of block ids with MultiresSparseGrid::sortBlockListMorton
 * (src/msbg2.cpp:46-58): int32 bids[nBlocksIn] in, the sorted list out.
 * A "solver job" runs the solver building blocks (multiplyLaplacianMatrixOpt,
 * dotProdChannel, AXPBYChannelCombined, relaxBlockList) on the value blocks of a
 * single-resolution layout: int32 bids[nBlocksIn], then float32 [nBlocksIn][bsx^3]
 * arrays X, B, Q, P, CX, CY, CZ, DINV in; dt / rParticle = AXPBY a / b, nIter = relax
 * passes, constr01 = reverse order.  Out: double dot(AX, X), dot(X, B), then A X,
 * B - A X, X + aP, Q + bP and the relaxed X, each [nBlocksIn][bsx^3].
 * A "downsample job" takes the halo job's input (FP32 only) and dumps
 * downsampleFloatChannelNew to multigrid level 1 for every level-0 block (constr01 = 1:
 * OPT_SIMPLE_AVERAGE): int32 bids[nActive], float32 [nActive][(bsx/2)^3].
 * A "halo3 job" takes the halo job's FP32 input plus the cell flags of every level (int32
 * states [nLevels][nBlocks], then per level uint16 [max+1][(bsx>>l)^3]) and int32 domain
 * boundary types [6] (-x,+x,-y,+y,-z,+z), the constant blocks' flags in `reserved`
 * (empty | full << 16), and dumps HaloBlockSet::fillHaloBlock3 at multigrid level 0 of
 * every level-0 block: int32 bids[nActive], float32 [nActive][(bsx+2)^3].
 * A "layout job" takes the levels job's input and dumps, after the header, lists (int32
 * count, then the sorted ids): _blocksExisting, _blocksFineCoarsePerLevel[l] for every
 * level, then per level the CH_DIST_FINECOARSE grid: its value blocks (list, then uint16
 * [n][(bsx>>l)^3]), its full blocks (list) and the full value (uint16).
 */
#ifndef MSBG_ORACLE_COMMON_H
#define MSBG_ORACLE_COMMON_H

#include <stdint.h>

#define ORACLE_JOB_MAGIC "MSBGJOB2"
#define ORACLE_OUT_MAGIC "MSBGOUT2"

enum { ORACLE_CHAN_F32 = 0, ORACLE_CHAN_U16 = 1 };
enum { ORACLE_JOB_SURFACE = 1, ORACLE_JOB_LEVELS = 2, ORACLE_JOB_INTERP = 3, ORACLE_JOB_HALO = 4,
       ORACLE_JOB_RENDER = 5, ORACLE_JOB_MORTON = 6, ORACLE_JOB_SOLVER = 7, ORACLE_JOB_DOWNSAMPLE = 8,
       ORACLE_JOB_HALO3 = 9, ORACLE_JOB_LAYOUT = 10, ORACLE_JOB_MULTIRES = 11, ORACLE_JOB_DENSE = 12 };

/* Interp job option bits: the reference's own interpolation options (src/sbg.h:140-170)
 * plus one bit that the reference's enum leaves unused, for the render-density scale. */
enum {
  ORACLE_IP_CORNER = 1 << 0,           /* OPT_IPCORNER: no half-voxel shift */
  ORACLE_IP_BC_DIRICHLET = 1 << 13,    /* OPT_IPBC_DIRICHLET: clipped corners read empty */
  ORACLE_IP_BC_DIRICHLET_OLD = 1 << 14,/* OPT_IPBC_DIRICHLET_OLD: border points give empty */
  ORACLE_IP_NO_BORDER_CHECK = 1 << 15, /* OPT_IP_NO_BORDER_CHECK */
  ORACLE_IP_RENDER_DENS = 1 << 18      /* uint16: interpolateRenderDensity */
};

typedef struct {
  char magic[8];
  int32_t jobType;  /* ORACLE_JOB_* */
  int32_t sx, sy, sz, bsx;
  int32_t nLevels;  /* resolution levels of the grid (3 in the demo) */
  int32_t chanType; /* ORACLE_CHAN_* */
  int32_t nIter;    /* applyChannelPdeFast numIter (rounded up to even inside) */
  int32_t laplTyp;  /* applyChannelPdeFast laplTyp, signed as the reference wants */
  int32_t constr01; /* doConstrZeroOne; interp job: ORACLE_IP_* option bits */
  int32_t nThreads; /* OpenMP threads for the reference's parallel loops */
  float dt;         /* applyChannelPdeFast timeStep */
  float rParticle;  /* splat kernel radius (demo: 2) */
  float nbDist;     /* narrow band added to the scan radius (demo: 2) */
  float anisAlpha;  /* applyChannelPdeFast anisDiffAlpha (Perona-Malik) */
  int32_t reserved; /* keeps the int64 fields 8-byte aligned */
  int64_t nPoints;  /* surface / interp job: float32 xyz follow; levels job: 0 */
  int64_t nBlocksIn;/* levels job: int32 levels[nBlocksIn] follow;
                       interp job: int32 activeBids[nBlocksIn] follow, then the
                       payload [nBlocksIn][bsx^3] of the channel type;
                       halo job (nBlocksIn = nBlocks; nIter = halo size, laplTyp = the
                       level whose blocks are filled, constr01 = option bits, dt / rParticle
                       = empty / full value): int32 levels[nBlocks], int32
                       state[nLevels][nBlocks] (>= 0 payload index, -1 empty, -2 full,
                       -3 no block), then per level l the payload [max(state_l)+1][(bsx>>l)^3] */
} OracleJobHeader;

typedef struct {
  char magic[8];
  int32_t nBlocks;      /* nbx*nby*nbz */
  int32_t nActive;      /* level-0 blocks (surface job) */
  int64_t nActParticles;/* points that passed the domain checks */
  int64_t nBlocksPerLevel[8];
  double tMarkSec, tLevelsSec, tAllocSec, tSplatSec, tFinalSec, tPdeSec;
  int32_t elemBytes;    /* 4 (float) or 2 (uint16) */
  int32_t nThreadsUsed;
  /* then: int8 levels[nBlocks]; uint16 flags[nBlocks];
   *       int32 activeBids[nActive];
   *       payloadAfterFinalize[nActive*bsx^3]; payloadAfterPde[nActive*bsx^3]
   * interp job: tPdeSec = interpolation time; then float32 values[nPoints]
   * halo job: nActive = filled blocks, tPdeSec = fill time; then int32 bids[nActive],
   *           float32 halo[nActive][(bs_l+2h)^3]
   * render job: tPdeSec = render time; then int32 pixels[height][width] (BMP_MKRGB)
   * morton job: nActive = list length; then int32 sorted bids[nActive] */
} OracleOutHeader;

#endif
