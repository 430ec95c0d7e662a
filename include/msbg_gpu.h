/*
 * msbg_gpu.h -- C ABI of the GB300 (sm_103a) implementation of the MSBG
 * (Multiresolution Sparse Block Grids, tum-pbs/MSBG) data-parallel hot path.
 *
 * The reference exposes this path as C++ methods of MSBG::MultiresSparseGrid
 * and SBG::SparseGrid<T> (src/msbg.h, src/sbg.h).  Each entry point below
 * names the reference interface it replaces.  All functions:
 *   - return 0 (MSBG_GPU_OK) or a negative MSBG_GPU_ERR_* code; the last error
 *     message of a context is available from msbg_gpu_last_error();
 *   - launch on the context's stream (msbg_gpu_set_stream) and are
 *     asynchronous unless stated otherwise; pointers named d* are device
 *     pointers, h* host pointers;
 *   - take plain C types only.
 * A context is not thread-safe (like the reference, whose per-thread scratch is
 * indexed by TBB thread id, src/halo.cpp:72-92); use one context per host thread.
 *
 * Data layout on the device:
 *   block id     bid = bx + by*nbx + bz*nbx*nby          (src/sbg.h:1744-1749)
 *   voxel index  vid = x + y*bs + z*bs*bs inside a block (src/sbg.h:1816-1820)
 *   slot[bid]    payload index of a level-0 ("value") block, or -1 for the
 *                shared constant empty block              (src/sbg.h:2042-2047)
 *   payload      one slab per channel: [nActive][bs^3] elements of the
 *                channel's storage type, slots in ascending bid order.
 */
#ifndef MSBG_GPU_H
#define MSBG_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MSBG_GPU_ABI_VERSION 2

/* ---- status codes ---------------------------------------------------------- */
enum {
  MSBG_GPU_OK = 0,
  MSBG_GPU_ERR_ARG = -1,         /* invalid argument (size, pointer, option)     */
  MSBG_GPU_ERR_CUDA = -2,        /* a CUDA runtime call failed                  */
  MSBG_GPU_ERR_NOMEM = -3,       /* device or pinned host allocation failed     */
  MSBG_GPU_ERR_STATE = -4,       /* call out of order (e.g. no layout yet)      */
  MSBG_GPU_ERR_CAPACITY = -5,    /* block pool exhausted                        */
  MSBG_GPU_ERR_NONFINITE = -6,   /* a reduction met NaN/Inf (src/msbg.cpp:4635) */
  MSBG_GPU_ERR_DIVERGED = -7,    /* solver residual non-finite or increasing    */
  MSBG_GPU_ERR_UNSUPPORTED = -8, /* option the GPU path does not implement      */
  MSBG_GPU_ERR_TIMEOUT = -9,     /* a bounded device-side wait gave up          */
  MSBG_GPU_ERR_IO = -10          /* a checkpoint file could not be written or read, or
                                    its contents fail their checks              */
};

/* ---- storage types of a channel ------------------------------------------ */
enum {
  MSBG_GPU_F32 = 0, /* float                                                   */
  MSBG_GPU_U16 = 1, /* uint16 density, v/65535 (src/sbg.h:225-351)              */
  MSBG_GPU_F16 = 2, /* IEEE half, FP32 arithmetic                              */
  MSBG_GPU_F64 = 3  /* double (the FP64 check path)                            */
};

/* ---- applyChannelPdeFast laplTyp values (src/msbg.h:132-141) -------------- */
#define MSBG_GPU_OPT_8_COLOR_SCHEME (1 << 29)
#define MSBG_GPU_PDE_MEAN_CURVATURE 4

/* ---- block flags (same bits as src/msbg.h:561-573) ------------------------ */
#define MSBG_GPU_BLK_DOM_BORDER (1 << 1)
#define MSBG_GPU_BLK_COARSE_FINE (1 << 2)
#define MSBG_GPU_BLK_FINE_COARSE (1 << 3)
#define MSBG_GPU_BLK_EXISTS (1 << 12)
#define MSBG_GPU_BLK_UNIFORM_EMPTY (1 << 13)

/* ---- sweep kernel variants ------------------------------------------------- */
enum {
  MSBG_GPU_SWEEP_EXACT = 0, /* reference expression order, every float op
                               individually rounded: bit-identical to the CPU
                               restatement                                       */
  MSBG_GPU_SWEEP_FAST = 1   /* same PDE, re-associated with fused multiply-adds;
                               agrees within rel-L2 1e-5                          */
};

typedef struct msbg_gpu_ctx msbg_gpu_ctx;

typedef struct {
  int32_t sx, sy, sz;       /* finest-level voxels                          */
  int32_t bsx;              /* finest-level block edge                      */
  int32_t nbx, nby, nbz;    /* blocks per axis                              */
  int32_t nLevels;          /* resolution levels                            */
  int64_t nBlocks;          /* nbx*nby*nbz                                  */
  int64_t nActive;          /* level-0 (value) blocks after the last layout */
  int64_t capacityBlocks;   /* block-pool capacity (value blocks)           */
  int64_t blocksPerLevel[8];
  int32_t colorCount[8];    /* value blocks per 8-color class               */
  int64_t nActParticles;    /* points that passed the domain checks         */
  int64_t nAborted;         /* particles abandoned at a non-value block     */
} msbg_gpu_info;

/* ---- lifecycle --------------------------------------------------------------
 * Replaces MultiresSparseGrid::create / destroy (src/msbg.h:834-852).
 * Creates the block index for an sx*sy*sz grid with base block bsx (a power of
 * two, 8..32, dividing each side) and nLevels resolution levels (block size
 * halves per level, src/msbg.cpp:808-811).  Channel 0 (the density channel of
 * the demo, CH_UINT16_1 / CH_FLOAT_1) is created with storage `storage`.
 * capacityBlocks bounds the value blocks of the block pool (0 = all blocks). */
int msbg_gpu_create(msbg_gpu_ctx **ctx, int sx, int sy, int sz, int bsx, int nLevels,
                    int storage, int64_t capacityBlocks);
int msbg_gpu_destroy(msbg_gpu_ctx *ctx);
const char *msbg_gpu_last_error(const msbg_gpu_ctx *ctx);
int msbg_gpu_set_stream(msbg_gpu_ctx *ctx, void *cudaStream);
int msbg_gpu_get_info(msbg_gpu_ctx *ctx, msbg_gpu_info *info); /* synchronizes */
int msbg_gpu_synchronize(msbg_gpu_ctx *ctx);

/* Creates another payload channel over the same block layout (reference:
 * MultiresSparseGrid channels by id, src/msbg.h:274-343, src/msbgaux.cpp:26-96). */
int msbg_gpu_channel_create(msbg_gpu_ctx *ctx, int chan, int storage);

/* ---- layout ----------------------------------------------------------------
 * Active-block marking of the demo (src/msbg_demo.cpp:339-397): every block of
 * each in-domain point's rScan box is marked; dPts is float xyz[n] on the device. */
int msbg_gpu_mark_points(msbg_gpu_ctx *ctx, const float *dPts, int64_t n, float rScan);
/* Level map from the marks: marked -> 0, else nLevels-1 (src/msbg_demo.cpp:413-425). */
int msbg_gpu_levels_from_marks(msbg_gpu_ctx *ctx);
/* Distance-band level map: level l for blocks in the rBand[l] box of a point,
 * nLevels-1 elsewhere (nBands <= nLevels-1). */
int msbg_gpu_levels_from_bands(msbg_gpu_ctx *ctx, const float *dPts, int64_t n,
                               const float *hBands, int nBands);
/* Caller-supplied level map, int32 per block, host memory. */
int msbg_gpu_set_levels(msbg_gpu_ctx *ctx, const int32_t *hLevels);
/* regularizeRefinementMap (src/msbg.h:897-901, src/msbg.cpp:1202-1423). */
int msbg_gpu_regularize_refinement_map(msbg_gpu_ctx *ctx);
/* setRefinementMap for levelMg 0 (src/msbg.h:903-908, src/msbg.cpp:1428-2165) plus
 * the demo's allocation loop (src/msbg_demo.cpp:455-511): BlockInfo flags,
 * value blocks for level 0 in ascending bid order, 8-color lists, every
 * channel's payload filled with fillValue. */
int msbg_gpu_set_refinement_map(msbg_gpu_ctx *ctx, double fillValue);
/* setRefinementMap's block lists (src/msbg.cpp:1682-1727): MSBG_GPU_LIST_EXISTING = the
 * reference's _blocksExisting (blocks flagged BLK_EXISTS), MSBG_GPU_LIST_FINE_COARSE =
 * _blocksFineCoarsePerLevel[level] (blocks of that level flagged BLK_FINE_COARSE), in
 * ascending block id (the release fills them in no fixed order).  dBids: device, nBlocks
 * entries; *hCount: the list's length.  Synchronizes. */
enum { MSBG_GPU_LIST_EXISTING = 0, MSBG_GPU_LIST_FINE_COARSE = 1 };
int msbg_gpu_get_block_list(msbg_gpu_ctx *ctx, int which, int level, int32_t *dBids, int64_t *hCount);
/* setRefinementMap's fine-coarse distance channel CH_DIST_FINECOARSE at resolution level
 * `level` (src/msbg.cpp:1887-1960, 1994-2033), as a level grid: dState (device, nBlocks):
 * the data index of every block of that level flagged BLK_FINE_COARSE (ascending id), whose
 * cells (level coordinates, x fastest) hold uint16(1024 * min(6, distance from the cell
 * centre to the nearest coarser 26-neighbour block)) in dData (device, capBlocks blocks of
 * (bsx>>level)^3); MSBG_GPU_LBLK_FULL (value 6 * 1024) for blocks of level-1 or level that
 * touch such a block; MSBG_GPU_LBLK_EMPTY otherwise.  *hCount: the data blocks;
 * MSBG_GPU_ERR_CAPACITY when they exceed capBlocks.  Synchronizes. */
int msbg_gpu_dist_fine_coarse(msbg_gpu_ctx *ctx, int level, int32_t *dState, uint16_t *dData, int64_t capBlocks,
                              int64_t *hCount);
/* Read back the layout (synchronize): levels int8[nBlocks], flags uint16[nBlocks],
 * active block ids int32[nActive], slots int32[nBlocks]. */
int msbg_gpu_get_levels(msbg_gpu_ctx *ctx, int8_t *hLevels);
int msbg_gpu_get_flags(msbg_gpu_ctx *ctx, uint16_t *hFlags);
int msbg_gpu_get_active_blocks(msbg_gpu_ctx *ctx, int32_t *hBids, int64_t cap, int64_t *n);
int msbg_gpu_get_slots(msbg_gpu_ctx *ctx, int32_t *hSlots);

/* ---- channel data ------------------------------------------------------------
 * Payload of all value blocks, [nActive][bs^3] of the channel's storage type
 * (SparseGrid::getBlockDataPtr for every block of the active list). */
int msbg_gpu_upload_payload(msbg_gpu_ctx *ctx, int chan, const void *hData);
int msbg_gpu_download_payload(msbg_gpu_ctx *ctx, int chan, void *hData);
/* Device pointer of a channel's payload slab (valid until the next layout). */
int msbg_gpu_payload_ptr(msbg_gpu_ctx *ctx, int chan, void **dPtr);
int msbg_gpu_fill(msbg_gpu_ctx *ctx, int chan, double value);

/* ---- splat --------------------------------------------------------------------
 * Splat of min(distSq/distSqMax) into channel 0 (src/msbg_demo.cpp:527-636):
 * a particle is abandoned at its first (z,y,x scan order) in-sphere voxel that
 * lies in a non-value block, as the demo does.  The particles are sorted into
 * lists of the value blocks their boxes touch, and each value block takes the
 * minimum over its list; min is order-independent, so this replaces the demo's
 * 8 color passes over its per-block lists.  Then the distance-to-density
 * finalize (src/msbg_demo.cpp:655-680). */
int msbg_gpu_splat(msbg_gpu_ctx *ctx, const float *dPts, int64_t n, float rParticle,
                   float nbDist);
/* The demo's per-block particle lists particlesPerBlock (src/msbg_demo.cpp:349-390):
 * every point that passes the marking loop's domain tests, in the list of the
 * block that contains it.  CSR form in caller device arrays: dOffsets[nBlocks+1]
 * (int64; block b's list is dIndex[dOffsets[b] .. dOffsets[b+1]-1]) and dIndex
 * (int32 point indices, capacity n).  *hCount = the listed points (the demo's
 * nActParticles).  The order inside a list is unspecified, as in the reference,
 * whose lists are lock-free stacks filled by a parallel loop. */
int msbg_gpu_particles_per_block(msbg_gpu_ctx *ctx, const float *dPts, int64_t n, int64_t *dOffsets,
                                 int32_t *dIndex, int64_t *hCount);
int msbg_gpu_splat_finalize(msbg_gpu_ctx *ctx, float rParticle, float nbDist);

/* ---- block lists ------------------------------------------------------------------
 * The reference's solver and sweep calls take `std::vector<int> *blockList` (NULL = all
 * blocks).  Here a block list is dBlockList (device, nBlockList block ids; NULL = all
 * value blocks).  Listed blocks without payload are skipped, as the reference skips
 * BLK_NO_FLUID blocks; an id outside the block grid returns MSBG_GPU_ERR_ARG.  A call
 * with a list synchronizes once to size its launches. */

/* ---- stencil sweeps -------------------------------------------------------------
 * applyChannelPdeFast<T>(chPhi, chTmp, chTmp2, blockList, laplTyp, doConstrZeroOne,
 * densThr, densThrTol1, densThrTol2, numIter, gridSpacing, timeStep, velMagThr, msbgVel,
 * lambda, lambdaSDF, taubinStrength, redist, anisDiffAlpha, veldep_on, veldep_fit, visOpt)
 * (src/msbg.h:2150-2172, src/msbg4.cpp:60-957), argument for argument, plus the kernel
 * variant.  Updates channel chPhi on the listed value blocks (all with a NULL list):
 * laplTyp < 0 in place with 8 colors (with MSBG_GPU_OPT_8_COLOR_SCHEME) or red-black,
 * laplTyp > 0 ping-pong through the library's own scratch (chTmp, chTmp2 are accepted and
 * not used; unlisted blocks keep their values).  Kernels 4 (mean curvature), 17 (Jacobi
 * diffusion), 15/14 (Perona-Malik, anisDiffAlpha > 0), 3 (simple diffusion), 1
 * (Laplacian).  numIter is rounded up to even, as the reference does.  Halo:
 * OPT_BC_NEUMANN.  gridSpacing must be 1 (the reference asserts it); lambda and lambdaSDF
 * have no effect (the reference sets lambda to 0 itself); visOpt and veldepFit are
 * ignored.  MSBG_GPU_ERR_UNSUPPORTED: negative numIter (the compressed-range mode), densThr
 * or its tolerances > 0, velMagThr != 0, msbgVel != NULL, veldepOn, taubinStrength != 0,
 * redist > 0. */
int msbg_gpu_apply_channel_pde_fast(msbg_gpu_ctx *ctx, int chPhi, int chTmp, int chTmp2,
                                    const int32_t *dBlockList, int64_t nBlockList, int laplTyp,
                                    int doConstrZeroOne, float densThr, float densThrTol1,
                                    float densThrTol2, int numIter, float gridSpacing, float timeStep,
                                    float velMagThr, const void *msbgVel, float lambda, float lambdaSDF,
                                    float taubinStrength, float redist, float anisDiffAlpha, int veldepOn,
                                    const float *veldepFit, int visOpt, int variant);

/* ---- whole surface job with host buffers (end-to-end entry point) --------------
 * Upload n points (host, float xyz), build the layout (marks with rScan =
 * rParticle + nbDist, or distance bands when nBands > 0), splat, finalize,
 * numIter sweeps of laplTyp, and download channel 0's payload into hOut
 * (capacity hOutCap bytes).  *nActiveOut receives the value-block count. */
int msbg_gpu_surface_job(msbg_gpu_ctx *ctx, const float *hPts, int64_t n, float rParticle,
                         float nbDist, const float *hBands, int nBands, int laplTyp, int numIter,
                         float timeStep, int variant, void *hOut, size_t hOutCap,
                         int64_t *nActiveOut);
/* The streaming form of msbg_gpu_surface_job for a sequence of jobs on one context: the same
 * arguments and result, queued.  The call returns after the job's last host read-back (the
 * sweeps' status check): nActiveOut is known then and the points have been uploaded, so hPts
 * may be reused; hOut is complete only after msbg_gpu_surface_job_wait.  This job's result comes
 * down (through a device staging copy of the payload) while the next job's points go up and it
 * computes, so a sequence runs at the rate of its compute.  The library's small read-backs go
 * through pinned memory written by a kernel, so they do not wait behind the download on a copy
 * engine.  hPts and hOut should be pinned (msbg_gpu_host_alloc). */
int msbg_gpu_surface_job_submit(msbg_gpu_ctx *ctx, const float *hPts, int64_t n, float rParticle, float nbDist,
                                const float *hBands, int nBands, int laplTyp, int numIter, float timeStep,
                                int variant, void *hOut, size_t hOutCap, int64_t *nActiveOut);
/* Waits for every submitted job, uploads and downloads included. */
int msbg_gpu_surface_job_wait(msbg_gpu_ctx *ctx);
/* Stream time (ms) of the stages of the last msbg_gpu_surface_job, from CUDA events at their
 * boundaries: points uploaded, layout built (levels, regularisation, refinement map, slab
 * fill), splat, finalize, sweeps, payload downloaded.  msOut receives min(cap, *nOut)
 * values; host time spent inside a stage (the layout's read-back of the block counts)
 * counts towards it. */
int msbg_gpu_surface_job_stages(msbg_gpu_ctx *ctx, float *msOut, int cap, int *nOut);

/* ---- sparse Poisson solve -------------------------------------------------------------
 * Operator on the value-block cells (src/msbg3.cpp:1281-1296):
 *   (A x)_i = d_i x_i - sum_f c_f x_nb(f),   x = 0 outside the value blocks (Dirichlet)
 * Coefficients are FP32 channels of the current layout: the lower-face coefficient of
 * every cell in x, y, z and the diagonal d (which includes faces towards inactive
 * cells).  The upper face of a cell is the lower face of the cell above.  Setting the
 * coefficients (re)builds the multigrid hierarchy: block edge halving down to one cell
 * per block, then 2x2x2 aggregation of the block grid (the dense coarse levels of
 * src/msbg.cpp:854-998), coarse operators P^T A P / 2 with piecewise-constant transfers. */
int msbg_gpu_poisson_set_coefficients(msbg_gpu_ctx *ctx, int chanCx, int chanCy, int chanCz,
                                      int chanDiag);
/* Seeded coefficients uniform in [0.5, 2] per face (hash of the face position and
 * seed); copies them into the given FP32 channels when they are >= 0. */
int msbg_gpu_poisson_procedural_coefficients(msbg_gpu_ctx *ctx, uint32_t seed, int chanCx,
                                             int chanCy, int chanCz, int chanDiag);
/* multiplyLaplacianMatrixOpt(options, levelMg, chanX, chanB, kap, chanDstY, pDotprod,
 * blockList) (src/msbg.h:3167-3176, src/msbg3.cpp:1756-1912): Y = A X on the listed value
 * blocks, or with MSBG_GPU_OPT_CALC_RESIDUAL Y = B - A X.  pDotprod (host, may be NULL;
 * not with the residual, as the reference asserts) receives sum(Y X) in FP64 and makes the
 * call synchronize.  levelMg must be 0 (the value blocks); kap is unused, as in the
 * reference's sparse-level path.  The reference's operator is h ((1/D) X - sum W X_nb) with
 * D = 1/diagonal stored in CH_DIAGONAL, the face areas W and h = 1 at level 0; here the
 * diagonal itself is stored, and the call forms 1/(1/d) in FP32 from it and evaluates the
 * rest in the reference's compiled order, so Y equals the reference's bit for bit.  Without a
 * list the call covers every value block. */
#define MSBG_GPU_OPT_CALC_RESIDUAL (1u << 12) /* OPT_CALC_RESIDUAL (src/msbg.h:115) */
int msbg_gpu_multiply_laplacian(msbg_gpu_ctx *ctx, unsigned options, int levelMg, int chanX, int chanB,
                                float kap, int chanDstY, double *pDotprod, const int32_t *dBlockList,
                                int64_t nBlockList);
/* multiplyLaplacianMatrixOpt(options, levelMg, chanX, chanB, kap, chanDstY) at a dense
 * multigrid level (levelMg >= the number of resolution levels; src/msbg3.cpp:1756-1812, the
 * operator ImultiplyLaplacianMatrixProcessSliceDenseLevel, src/msbg3.cpp:166-403) on device
 * arrays of one such level: sx*sy*sz cells, x fastest, with the cell flags (uint16, the
 * reference's CellFlags bits), X, B (residual only), the diagonal channel as the reference
 * holds it (1/diagonal) and the lower-face areas.  Outside the box X and the face areas are 0
 * and the cells are void, as the reference's zero border with void flags gives.  Each row goes
 * in groups of 4 cells from x = 0: a group without a fluid cell is skipped and its outputs are
 * not written; a group with a solid or partially solid cell weighs every neighbour by its face
 * area.  Fluid cells get Y = h ((1/D) X - sum F), h = 2^levelMg, other cells of a processed
 * group 0; with MSBG_GPU_OPT_CALC_RESIDUAL Y = B - A X.  Bit for bit with the reference's
 * compiled operator.  Asynchronous on the context's stream. */
int msbg_gpu_multiply_laplacian_dense(msbg_gpu_ctx *ctx, unsigned options, int levelMg, int sx, int sy, int sz,
                                      const uint16_t *dFlags, const float *dX, const float *dB, const float *dDiag,
                                      const float *dAreaX, const float *dAreaY, const float *dAreaZ, float *dY);
/* relax(0, reverseOrder, levelMg, chanX, chanB, chanTmp, nIter, 0) at a dense multigrid level
 * (src/msbg3.cpp:2244-2310 -> ImultiplyLaplacianMatrixDenseLevel, src/msbg3.cpp:1917-2165):
 * nIter omega-Jacobi iterations (omega from msbg_gpu_set_relax_params) of the operator above,
 * alternating between dX and dTmp (the reference's chanTmp; cells of skipped groups keep what
 * it holds), the whole of dTmp copied to dX after an odd count.  Fluid cells get
 * omega (B + h S) D / h + (1 - omega) X in the reference's compiled order, other cells of a
 * processed group 0.  Bit for bit with the reference.  Asynchronous on the context's stream. */
int msbg_gpu_relax_dense(msbg_gpu_ctx *ctx, int levelMg, int sx, int sy, int sz, int nIter, const uint16_t *dFlags,
                         float *dX, const float *dB, const float *dDiag, const float *dAreaX, const float *dAreaY,
                         const float *dAreaZ, float *dTmp);
/* relax(boundaryZoneOnly, reverseOrder, levelMg, chanX, chanB, chanTmp, nIter, options)
 * (src/msbg.h:3269-3277, src/msbg3.cpp:2244-2369): nIter passes of the reference's block
 * smoother on A X = B, in place: each pass relaxes the blocks of parity (bx+by+bz)&1 = 1,
 * then 0 (0 then 1 with reverseOrder), each block with its face-neighbour halo taken at its
 * start and _mgSmBlockIter block-local weighted Gauss-Seidel iterations
 *   X = omega (B + sum W X_nb) / d + (1 - omega) X
 * over groups of 8 x-consecutive cells (the reference's SIMD width), alternating sweep
 * direction, the last iteration a Jacobi step (src/msbg3.cpp:1108-1332).  omega = 6/7 and
 * 5 block iterations (src/msbg.cpp:814-843) unless msbg_gpu_set_relax_params changes them.
 * The reference relaxes its member list _blocksRelax[levelMg], which nothing in the
 * release fills; dBlockList stands in for it.  With options MSBG_GPU_RELAX_TILES the call
 * runs the multigrid's own smoother instead (red-black over tiles with in-tile red-black
 * Gauss-Seidel, all value blocks, no list; reverseOrder = the adjoint order); when chanX and
 * chanB are both FP16 channels it runs the mixed solve's FP16-storage form of that smoother
 * (FP32 arithmetic, the coefficients rounded to FP16 once).  levelMg must
 * be 0; boundaryZoneOnly != 0 is MSBG_GPU_ERR_UNSUPPORTED; chanTmp is unused, as in the
 * reference's in-place block order. */
#define MSBG_GPU_RELAX_TILES (1u << 31) /* a bit the reference's option enum leaves unused */
int msbg_gpu_relax(msbg_gpu_ctx *ctx, int boundaryZoneOnly, int reverseOrder, int levelMg, int chanX, int chanB,
                   int chanTmp, int nIter, unsigned options, const int32_t *dBlockList, int64_t nBlockList);
/* The block smoother's weight and block-local iterations (_mgSmOmega, _mgSmBlockIter,
 * src/msbg.cpp:814-843; the reference reads the latter from psConf->ps_mg_sm_block_iter). */
int msbg_gpu_set_relax_params(msbg_gpu_ctx *ctx, float omega, int blockIter);
/* Diagnostics of the failure path: one CTA waits on an mbarrier that nothing completes,
 * with the same bounded try-wait loop as the library's kernels but a limit of `polls`
 * (1..1<<20).  The kernel records the expired wait in the device status word and returns;
 * the call returns MSBG_GPU_ERR_TIMEOUT, clears the word, and leaves the context usable.
 * No GPU fault is involved. */
int msbg_gpu_diag_wait_timeout(msbg_gpu_ctx *ctx, int polls);
/* downsampleFloatChannelNew (src/msbg4.cpp:1035-1379, levelMg = 1, OPT_ALL_CELLS): the
 * restriction of channel chSrc (FP32, FP16 or uint16 storage) to the next coarser
 * multigrid level, for every value block.  dDst (device, FP32) receives
 * nActive * (bs/2)^3 values, block by block in slot order, x fastest.  A coarse cell v
 * is the sum over the fine cells 2v-1 .. 2v+2 (4 per axis) with weights
 * (1,3,3,1)x(1,3,3,1)x(1,3,3,1)/512 (G3D_GetGausslikeKernel4x4x4, src/grid.c:30-70); with
 * simpleAverage != 0 (OPT_SIMPLE_AVERAGE) the mean of its 8 children.  Fine cells
 * outside the block come from the halo fill with OPT_BC_COARSE_LEVEL (src/halo.h:288-300):
 * outside the domain, the value at the clamped position; in a block without payload, the
 * channel's empty value. */
int msbg_gpu_downsample_channel(msbg_gpu_ctx *ctx, int chSrc, float *dDst, int simpleAverage);
/* Grid-to-particle interpolation: dOut[i] (device, FP32) = the trilinear interpolant of
 * channel chan (FP32, FP16 or uint16 storage) at dPts[3i..3i+2] (device, voxel units,
 * voxel centres at i + 0.5), for i < n.
 * Replaces SparseGrid<float>::interpolateFloatFast (src/sbg.h:1443-1444, body
 * src/sbg.h:4623-4792) and SparseGrid<uint16_t>::interpolateUint16ToFloatFast
 * (src/sbg.h:1445, body src/sbg.h:4920-5032), called per point; with
 * MSBG_GPU_IP_RENDER_DENS, MSBG::interpolateRenderDensity (src/msbg.h:478-484).
 *  - uint16 values are interpolated unscaled unless MSBG_GPU_IP_RENDER_DENS is given
 *    (then times 1/65535); FP16 values are widened to FP32.
 *  - A block without payload reads the empty value 0.
 *  - Points whose lower corner is outside [0, s-2] on an axis take the reference's
 *    generic path (interpolateGen0<IP_LINEAR>, src/sbg.h:3109-3246): corners clamped
 *    to the domain, or the Dirichlet variants below.
 *  - opt: the reference's bits MSBG_GPU_IP_CORNER (no half-voxel shift),
 *    MSBG_GPU_IP_BC_DIRICHLET, MSBG_GPU_IP_BC_DIRICHLET_OLD, MSBG_GPU_IP_NO_BORDER_CHECK
 *    (the border test is always made; results inside the domain are unchanged),
 *    MSBG_GPU_IP_CHKBLK (no effect), plus MSBG_GPU_IP_RENDER_DENS.  Other bits:
 *    MSBG_GPU_ERR_UNSUPPORTED.
 * Asynchronous on the context's stream. */
enum {
  MSBG_GPU_IP_CORNER = 1 << 0,            /* OPT_IPCORNER           (src/sbg.h:142) */
  MSBG_GPU_IP_CHKBLK = 1 << 5,            /* OPT_IPCHKBLK           (src/sbg.h:147) */
  MSBG_GPU_IP_BC_DIRICHLET = 1 << 13,     /* OPT_IPBC_DIRICHLET     (src/sbg.h:155) */
  MSBG_GPU_IP_BC_DIRICHLET_OLD = 1 << 14, /* OPT_IPBC_DIRICHLET_OLD (src/sbg.h:156) */
  MSBG_GPU_IP_NO_BORDER_CHECK = 1 << 15,  /* OPT_IP_NO_BORDER_CHECK (src/sbg.h:157) */
  MSBG_GPU_IP_RENDER_DENS = 1 << 18       /* uint16 render density; a bit the reference's
                                             option enum leaves unused */
};
int msbg_gpu_interpolate(msbg_gpu_ctx *ctx, int chan, const float *dPts, int64_t n, float *dOut,
                         int opt);
/* ---- multi-level channels and the cross-resolution halo fill ----------------------
 * A level grid is resolution level l of one channel of the reference's
 * MultiresSparseGrid: the SparseGrid that getChannel<T>(msbg, chan, l) returns
 * (src/msbg.h:720, src/msbg.h:3056-3076), with block edge bsx>>l, domain (sx>>l,
 * sy>>l, sz>>l) and the block grid of level 0 (src/msbg.cpp:800-812).  A block has
 * one state per level: payload (>= 0, the index of its data in hPayload), the
 * constant empty block (MSBG_GPU_LBLK_EMPTY, SparseGrid::setEmptyBlock), the constant
 * full block (MSBG_GPU_LBLK_FULL, setFullBlock) or no block (MSBG_GPU_LBLK_NONE, a
 * NULL block-map entry).
 * msbg_gpu_level_grid_set copies level `level` of level channel lchan (0..7, a
 * namespace of its own, apart from the value-block channels) to the device: hState
 * (host, nBlocks entries) and hPayload (host, nData blocks of (bsx>>level)^3 values of
 * `storage`, x fastest).  emptyValue / fullValue are the constant blocks' values
 * (setEmptyValue / setFullValue), stored in the storage type (uint16: v*65535 rounded
 * half away from zero).  Every level of a level channel has the same storage (FP32,
 * FP16 or uint16); setting a level with another storage clears the other levels. */
enum { MSBG_GPU_LBLK_EMPTY = -1, MSBG_GPU_LBLK_FULL = -2, MSBG_GPU_LBLK_NONE = -3 };
int msbg_gpu_level_grid_set(msbg_gpu_ctx *ctx, int lchan, int level, int storage, const int32_t *hState,
                            const void *hPayload, int64_t nData, float emptyValue, float fullValue);
/* The same for data already on the device: binds the caller's device arrays (dState:
 * nBlocks states; dPayload: the payload blocks, 16-byte aligned) without copying.  They
 * must stay valid, and unchanged while a fill reads them, until the level is set or
 * bound again or the context is destroyed.  A level-0 value-block channel binds as its slab
 * (msbg_gpu_payload_ptr) with states = its slots, -3 for blocks that are not at level 0. */
int msbg_gpu_level_grid_bind(msbg_gpu_ctx *ctx, int lchan, int level, int storage, const int32_t *dState,
                             const void *dPayload, float emptyValue, float fullValue);
/* HaloBlockSet::fillHaloBlock_<T>(iChan, bid, levelMg = 0, tid, options)
 * (src/halo.h:385-391, body src/halo.cpp:266-479, out-of-block rule
 * getOutOfBlockValue src/halo.h:270-330) for n blocks in one call.
 * dBids (device, n entries): blocks whose level in the current layout is `level` and
 * that have a block at that level of lchan.  dOut (device, 16-byte aligned): per listed block k,
 * (bs+2h)^3 floats at dOut + k*(bs+2h)^3, [z][y][x] over the positions origin-h ..
 * origin+bs+h-1 of level `level` (bs = bsx>>level, h = haloSize, 1..4).  A position
 * inside the domain whose block exists at that level reads it; otherwise
 *  - MSBG_GPU_BC_NEUMANN (OPT_BC_NEUMANN): the own block at the position clamped to it;
 *  - MSBG_GPU_BC_COARSE_LEVEL (OPT_BC_COARSE_LEVEL): outside the domain the position is
 *    clamped to it and read at this level if that block exists; else the position,
 *    halved, is read at level+1 (clamped to its domain) -- the cross-resolution fill;
 *  - neither: the level's empty value.
 * The reference needs a block at level+1 there; without one (or at the coarsest
 * level) the empty value is used.  uint16 reads as v/65535, FP16 widened.
 * OPT_INTERPOLATE (interpolateGhost) is not supported (MSBG_GPU_ERR_UNSUPPORTED).
 * Blocks that do not satisfy the conditions are skipped (output not written); when
 * hSkipped is not NULL the call synchronizes and stores their number there, else it
 * is asynchronous on the context's stream. */
enum { MSBG_GPU_BC_NEUMANN = 1 << 10, MSBG_GPU_BC_COARSE_LEVEL = 1 << 26 };
int msbg_gpu_fill_halo_blocks(msbg_gpu_ctx *ctx, int lchan, int level, const int32_t *dBids, int64_t n,
                              int haloSize, int opt, float *dOut, int64_t *hSkipped);
/* The solver's halo: HaloBlockSet::fillHaloBlock3(iChan, bid, bx, by, bz, levelMg, tid)
 * (src/halo.h:396-401, body src/halo.cpp:536-738) for n listed blocks at levelMg 0, halo 1.
 * The cell flags (the reference's CH_CELL_FLAGS grids) come from flags channel fchan, set
 * per level with msbg_gpu_level_flags_set (states as for level grids, raw uint16 flags, the
 * constant blocks' flags).  Per position p of the (bs+2)^3 box (floats [z][y][x] at
 * dOut + k*(bs+2)^3): p inside the domain in a block of layout level 0 -> CELL_VOID:
 * +1e20 (SPEC_FLOAT_DIRICHLET), CELL_SOLID: -1e20 (SPEC_FLOAT_NEUMANN), else the value of
 * level 0 of lchan; in a coarser block -> the same from level 1 at p/2; outside the domain
 * -> +1e20 if the face it leaves through is open (hDomainBc[face] == 0, DBC_OPEN), else
 * -1e20, the x face deciding before y before z.  hDomainBc (host, 6): the boundary types of
 * faces -x, +x, -y, +y, -z, +z (src/msbg.h:910-915).  Listed blocks not at layout level 0,
 * or without a level-0 block of lchan, are skipped (counted in *hSkipped, which makes the
 * call synchronize). */
#define MSBG_GPU_CELL_SOLID (1u << 0)  /* CELL_SOLID (src/msbg.h:602) */
#define MSBG_GPU_CELL_VOID (1u << 12)  /* CELL_VOID (src/msbg.h:614) */
int msbg_gpu_level_flags_set(msbg_gpu_ctx *ctx, int fchan, int level, const int32_t *hState,
                             const uint16_t *hFlags, int64_t nData, uint16_t emptyFlags, uint16_t fullFlags);
int msbg_gpu_fill_halo_blocks3(msbg_gpu_ctx *ctx, int lchan, int fchan, int levelMg, const int32_t *dBids,
                               int64_t n, const int32_t *hDomainBc, float *dOut, int64_t *hSkipped);
/* downsampleFloatChannelNew (src/msbg4.cpp:1035-1379) for blocks of a multi-level channel,
 * the step that restricts a block's data to the next coarser level (its ghost block,
 * src/msbg.cpp:3110-3150): for each listed block (as for msbg_gpu_fill_halo_blocks, any
 * level whose block edge is >= 2) dOut receives (bs/2)^3 floats [z][y][x], the 4^3
 * Gauss-like weights (1,3,3,1)^3/512 (src/grid.c:30-70) over the fine cells 2v-1 .. 2v+2
 * with the fine halo of fillHaloBlock_ with OPT_BC_COARSE_LEVEL, or with simpleAverage
 * (OPT_SIMPLE_AVERAGE) the mean of the 8 children; summed in the reference's order as
 * msbg_gpu_downsample_channel, which it equals on single-level layouts.  Skipped blocks
 * leave their output as is.  Allocates scratch for the halo boxes and synchronizes. */
int msbg_gpu_restrict_level_blocks(msbg_gpu_ctx *ctx, int lchan, int level, const int32_t *dBids, int64_t n,
                                   int simpleAverage, float *dOut, int64_t *hSkipped);
/* multiplyLaplacianMatrixOpt (src/msbg3.cpp:1756-1912) on a multi-resolution layout, for
 * the listed blocks of layout level `level` (the reference's call covers every level; one
 * call per level here): Y = A X, or with MSBG_GPU_OPT_CALC_RESIDUAL Y = B - A X.  Operands
 * are FP32 level channels: X (lchanX) at levels level-1, level, level+1 as the neighbours
 * need them, the diagonal channel (lchanD, what the reference's CH_DIAGONAL holds: the
 * operator multiplies by its reciprocal) and B (lchanB, residual only) at `level`.  Every
 * block is a fluid block at its level with unit face areas (no block cuts a solid); cells
 * of neighbouring levels meet through procNeighMixedRes2 (src/msbg3.cpp:46-161): a fine cell
 * takes 2/3 of the coarse cell across the face, a coarse cell 1/3 of each of the four fine
 * cells, scaled by h = 2^level; zero outside the domain.  dOut (device): n * (bsx>>level)^3
 * floats, block k's at dOut + k*(bsx>>level)^3.  pDotprod (host, may be NULL; not with the
 * residual) receives sum(Y X) in FP64.  A listed block is skipped (counted in *hSkipped)
 * when it is not at `level`, has no X payload or diagonal there, or a face neighbour has no
 * block at its level in X.  Synchronizes when pDotprod or hSkipped is given. */
int msbg_gpu_multiply_laplacian_levels(msbg_gpu_ctx *ctx, unsigned options, int level, int lchanX, int lchanB,
                                       int lchanD, const int32_t *dBids, int64_t n, float *dOut,
                                       double *pDotprod, int64_t *hSkipped);
/* relaxBlockList(blocks, levelMg = 0, iIter, chanX, chanB, options, chanX) (src/msbg.h:3279-3285,
 * src/msbg3.cpp:2170-2239) on a multi-resolution layout: one pass of the reference's block
 * smoother over the listed blocks of any level, red-black over blocks ((bx+by+bz)&1 = 1
 * first, 0 first with reverseOrder), each block relaxed in place in level `its level` of the
 * X level channel from the operator's halo of msbg_gpu_multiply_laplacian_levels
 * (mixed-resolution faces included) by _mgSmBlockIter block-local weighted Gauss-Seidel
 * iterations with omega = _mgSmOmega (msbg_gpu_set_relax_params; 5 and 6/7 by default),
 * as msbg_gpu_relax describes.  X (written: a bound payload receives the result), B and the
 * diagonal channel are FP32 level channels.  Listed blocks without data at their level, or
 * out of range, are skipped (counted in *hSkipped, which makes the call synchronize). */
int msbg_gpu_relax_levels(msbg_gpu_ctx *ctx, int reverseOrder, int lchanX, int lchanB, int lchanD,
                          const int32_t *dBids, int64_t n, int64_t *hSkipped);
/* ---- ray-march render of the iso-0.5 surface -----------------------------------------
 * RDR::RaymarchRenderer (src/render.h:52-160): setCamera(pos, lookAt, zoom),
 * setSunLight(sun), setSurfaceColor(color), then render() (src/render.cpp:20-101), which the
 * demo calls after the splat and after the sweeps (src/msbg_demo.cpp:129-175).  Renders
 * channel chan (uint16 as the reference; FP32 and FP16 read as values, no reference
 * counterpart) into dRGB (device, width*height*3 bytes, RGB, row-major, top row first;
 * the reference's BMP_MKRGB pixel (r, g, b) is bytes r, g, b here; a miss is black).
 * Camera coordinates are in units of the largest grid side (the domain is [0,1]^3 for a
 * cubic grid).  Asynchronous on the context's stream. */
typedef struct {
  double pos[3], lookAt[3], sun[3], color[3];
  double zoom;
} msbg_gpu_camera;
int msbg_gpu_render(msbg_gpu_ctx *ctx, int chan, int width, int height, const msbg_gpu_camera *cam,
                    uint8_t *dRGB);
/* ---- Morton order of block lists ---------------------------------------------------
 * MultiresSparseGrid::sortBlockListMorton (src/msbg2.cpp:46-58, declared src/msbg.h:3423):
 * sorts the n block ids of the device list dBids in place by the Morton code of their
 * block coordinates (FMA::morton64_encode, src/fastmath.h:290-316: x, y, z bits
 * interleaved, x lowest).  Each block may appear once (the reference's block lists hold
 * each block once); a repeated or out-of-range id returns MSBG_GPU_ERR_ARG and leaves the
 * list unchanged.  The work is one pass over all 8^K codes (2^K = the next power of two
 * at or above the longest block-grid side); grids so elongated that this exceeds both
 * 2^27 and 8x the block count return MSBG_GPU_ERR_UNSUPPORTED.  Allocates scratch and
 * synchronizes. */
int msbg_gpu_sort_block_list_morton(msbg_gpu_ctx *ctx, int32_t *dBids, int64_t n);
/* ---- checkpoint files ------------------------------------------------------------
 * The reference has no on-disk format for a MultiresSparseGrid (its VDB writers are
 * declarations only, src/sbg.h:599-605); this is a raw dump for checkpoint and restart.
 * msbg_gpu_save writes the grid geometry, the level map (int8 per block) and the
 * payload of nChans channels (chans[]; all value blocks in slot order, that is ascending
 * block id), each with an FNV-1a 64-bit checksum, little-endian:
 *   "MSBGCKP1", uint32 version 1, uint32 header bytes (64), int32 sx sy sz bsx nLevels
 *   nChans, int64 nBlocks nActive, uint64 checksum of the level map;
 *   int8 levels[nBlocks];
 *   per channel: int32 chan, int32 storage, int64 bytes, uint64 checksum, payload bytes.
 * msbg_gpu_load creates a context from such a file (*ctx), rebuilds the layout with
 * msbg_gpu_set_levels + msbg_gpu_set_refinement_map and restores the channels.  Both
 * stream through a pinned staging buffer and synchronize.  Errors: MSBG_GPU_ERR_IO for
 * a file that cannot be opened, written or read, is truncated, has another magic or
 * version, or fails a checksum (a failed load leaves *ctx NULL). */
int msbg_gpu_save(msbg_gpu_ctx *ctx, const char *path, const int *chans, int nChans);
int msbg_gpu_load(msbg_gpu_ctx **ctx, const char *path);
/* One multigrid V-cycle X = M^{-1} B from X = 0 (the CG preconditioner). */
int msbg_gpu_vcycle(msbg_gpu_ctx *ctx, int chanX, int chanB);
/* dotProdChannel(ch1, ch2, levelMg, blockList, pErrCode) (src/msbg.h:3331-3341): the
 * FP64-accumulated sum over the listed value blocks into *out; the reference's pErrCode is
 * the return code, MSBG_GPU_ERR_NONFINITE when the sum is not finite
 * (src/msbg.cpp:4635-4642).  levelMg must be 0.  Synchronizes. */
int msbg_gpu_dot(msbg_gpu_ctx *ctx, int chanA, int chanB, int levelMg, const int32_t *dBlockList,
                 int64_t nBlockList, double *out);
/* AXPBYChannel(a, iChanX, b, iChanDstY, levelMax, levelMg, blockList) (src/msbg.h:3356-3362):
 * Y = a X + b Y on the listed value blocks (all of them are level 0, so levelMax < 0 selects
 * none); levelMg must be 0. */
int msbg_gpu_axpby(msbg_gpu_ctx *ctx, double a, int chanX, double b, int chanY, int levelMax, int levelMg,
                   const int32_t *dBlockList, int64_t nBlockList);
/* AXPBYChannelCombined(a, b, iChanQ, iChanX, iChanP, blockList) (src/msbg.h:3364-3368):
 * X += a P; P = Q + b P on the listed value blocks. */
int msbg_gpu_axpby_combined(msbg_gpu_ctx *ctx, double a, double b, int chanQ, int chanX, int chanP,
                            const int32_t *dBlockList, int64_t nBlockList);
/* Multigrid-preconditioned CG: solves A X = B from the given X until the FP64-checked
 * relative residual ||B - A X|| / ||B|| <= tol or maxIter iterations.  Returns
 * MSBG_GPU_ERR_DIVERGED when the residual becomes non-finite or keeps growing. */
int msbg_gpu_mgpcg_solve(msbg_gpu_ctx *ctx, int chanX, int chanB, double tol, int maxIter,
                         int *itersOut, double *relResOut);
/* Mixed precision: FP32 iterative refinement around an FP16-storage MG-PCG.  Each
 * outer step forms r = B - A X with the FP32 operator, solves A e = r / rms(r) with
 * FP16 vectors and FP16 coefficients (FP32 arithmetic, FP64 dots) to innerTol or
 * maxInner iterations, and adds rms(r) e to X; stops at the FP64-checked relative
 * residual tol or after maxOuter steps. */
int msbg_gpu_mgpcg_solve_mixed(msbg_gpu_ctx *ctx, int chanX, int chanB, double tol, int maxOuter,
                               double innerTol, int maxInner, int *outerOut, int *innerTotalOut,
                               double *relResOut);
/* Multigrid parameters (defaults 2, 2, 3, 0): smoothing passes before and
 * after the coarse correction, in-tile red-black sweeps per pass (levels with
 * block edge >= 8 smooth 16^3 / 8^3 tiles in two tile colours; smaller levels
 * do that many pointwise red-black sweeps), and the coarsest level's solver:
 * 0 = exact (dense inverse from an FP64 Cholesky factor), > 0 = that many
 * red-black sweeps from zero.  Pre-smoothing orders tile colours 0,1 and cells red first;
 * post-smoothing uses the reverse (adjoint) order, which keeps the V-cycle a
 * symmetric preconditioner. */
int msbg_gpu_poisson_set_params(msbg_gpu_ctx *ctx, int preSweeps, int postSweeps, int tileIters,
                                int coarsestIter);
/* Frees the solver's level-0 work vectors (FP32: r, p, z, s, 16 B per cell; FP16: 12 B per
 * cell) and the FP16 coefficient copies of the mixed solve; the next solve allocates what it
 * needs again.  Lets a caller run the FP32 and the mixed solve on one large layout in turn. */
int msbg_gpu_poisson_release_work(msbg_gpu_ctx *ctx);
/* Multigrid levels of the current hierarchy and their cell counts. */
int msbg_gpu_mg_info(msbg_gpu_ctx *ctx, int *nLevels, int64_t *cellsPerLevel, int cap);
/* The launch-shape autotuner of the operator kernel: on the first operator call of a
 * (level, precision, mode) on a level of at least 2^21 cells, the candidate shapes (cells
 * per thread 4 or 8, grids of 608 / 1216 / 2432 CTAs) are timed on that call's data and
 * the fastest is kept for the layout.  enable: 1 on (the default), 0 off (static shapes),
 * -1 unchanged.  hOut (may be NULL): up to cap entries of 5 int32 each (level, bytes per
 * value, mode, cells per thread, grid) for the shapes picked so far; *nOut their count. */
int msbg_gpu_poisson_tuning(msbg_gpu_ctx *ctx, int enable, int32_t *hOut, int cap, int *nOut);

/* ---- batched solves ------------------------------------------------------------------
 * Many independent volumes on one layout: every value block belongs to one volume
 * (hVolOfBlock[nBlocks], -1 for blocks without data; volumes must not share a
 * block face, and each volume must lie in its own aligned region of the block grid
 * so that the multigrid aggregation never merges two volumes).  The solve runs a
 * segmented MG-PCG: CG scalars per volume, a volume freezes once its recurrence
 * residual is <= tol * ||B_v||.  useGraph: one captured CUDA graph per iteration,
 * replayed.  Outputs per volume (host arrays of nVol, may be NULL): iterations
 * (-1 not converged, 0 converged at the start), milliseconds from the start to the
 * iteration it converged in, FP64-checked relative residual; *hTotalMs = the whole
 * batch.  No reference counterpart (the reference solves one grid at a time). */
int msbg_gpu_batch_set_volumes(msbg_gpu_ctx *ctx, const int32_t *hVolOfBlock, int nVol);
int msbg_gpu_batch_mgpcg_solve(msbg_gpu_ctx *ctx, int chanX, int chanB, double tol, int maxIter,
                               int useGraph, int32_t *hIters, float *hMsToTol, double *hRelRes,
                               float *hTotalMs);

/* ---- learned warm start ------------------------------------------------------------
 * A 4-layer 3D convolutional network (channels 2-16-16-16-2, 3x3x3 kernels, BF16
 * weights, FP32 activations and accumulation) on the level-1 cells of the Poisson
 * hierarchy (value blocks with their edge halved).  Inputs: the restricted
 * right-hand side (scaled by its rms) and the level-1 diagonal (scaled by its
 * mean); outputs: a level-1 solution plus a level-2-averaged correction, injected
 * to level 0 as the solve's starting point.  Trained on (B, X*) pairs from the
 * plain solver with Adam; loss 0 (default) = ||X1 - avg(X*)||^2 / ||avg(X*)||^2 on
 * level 1 (avg: mean of the 8 level-0 children), loss 1 = ||A (X0 - X*)||^2 / ||B||^2.
 * No reference counterpart: the reference has no learned component.
 * Weight layout: per layer l, W[27][Cin][Cout] (tap = (dx+1) + 3(dy+1) + 9(dz+1)),
 * layers concatenated; biases per layer concatenated. */
int msbg_gpu_warmnet_param_count(int *nWeights, int *nBiases);
int msbg_gpu_warmnet_set_weights(msbg_gpu_ctx *ctx, const float *hW, const float *hB, int resetOptimizer);
int msbg_gpu_warmnet_get_weights(msbg_gpu_ctx *ctx, float *hW, float *hB);
int msbg_gpu_warmnet_set_loss(msbg_gpu_ctx *ctx, int lossMode);
/* X0 = the network's starting point for A X = B (FP32 channels). */
int msbg_gpu_warmnet_predict(msbg_gpu_ctx *ctx, int chanB, int chanX0);
/* Loss and gradients (host arrays in the weight layout, may be NULL) for one pair. */
int msbg_gpu_warmnet_loss_grad(msbg_gpu_ctx *ctx, int chanB, int chanXstar, double *loss, float *hGradW,
                               float *hGradB);
/* One Adam step (lr; betas 0.9, 0.999) on a pair given as device arrays laid out
 * like a level-0 payload [nActive][bs^3]; *loss is the loss before the step. */
int msbg_gpu_warmnet_train_step(msbg_gpu_ctx *ctx, const float *dB, const float *dXstar, float lr,
                                double *loss);

/* ---- value-block slots without allocating ----------------------------------------
 * This entry point has no counterpart in the reference.  It computes what
 * msbg_gpu_set_refinement_map's block-pool step computes -- slot[bid] = rank of bid
 * among the blocks whose level is 0 (ascending bid), -1 for all others,
 * activeBids[rank] = bid, *dCount = number of level-0 blocks -- for callers that
 * must not allocate device memory: a runtime that owns all device memory, a
 * memory budget fixed before the solve, code that may not call cudaMalloc or
 * cudaFree.  It needs no context and allocates nothing; all five pointers are the
 * caller's device buffers (dSlot: nBlocks entries, dActiveBids: nBlocks entries,
 * dCount: one int64), launched on cudaStream.
 * Its scan scratch is a fixed array inside the library (32 KiB on every device
 * that loads it, kept until the process exits), so nBlocks is limited to
 * MSBG_GPU_NOALLOC_MAX_BLOCKS; larger maps return MSBG_GPU_ERR_CAPACITY.
 * The first call on a device looks the array's address up: make that call
 * before any stream capture.  All calls share the array, so calls whose kernels
 * may overlap on the GPU (unordered streams) race; order them on one stream.
 * The call does not synchronize: its status covers the arguments and the launches
 * only (MSBG_GPU_ERR_CUDA also when the runtime already holds an error from earlier
 * work, which it then leaves unread); a fault while the kernels run shows up on the
 * caller's stream, so check that stream (cudaStreamSynchronize) before using dSlot. */
#define MSBG_GPU_NOALLOC_MAX_BLOCKS ((int64_t)1 << 24)
int msbg_gpu_assign_slots_noalloc(const int32_t *dLevels, int64_t nBlocks, int32_t *dSlot,
                                  int32_t *dActiveBids, int64_t *dCount, void *cudaStream);

/* ---- timing and accounting -------------------------------------------------------
 * CUDA events on the context's stream (slot 0..15); elapsed in milliseconds. */
int msbg_gpu_event_record(msbg_gpu_ctx *ctx, int slot);
int msbg_gpu_event_elapsed(msbg_gpu_ctx *ctx, int slotA, int slotB, float *ms);
/* Kernels this context has launched since creation. */
int64_t msbg_gpu_launch_count(const msbg_gpu_ctx *ctx);
/* Pinned host memory for staging (cudaMallocHost / cudaFreeHost). */
int msbg_gpu_host_alloc(void **hPtr, size_t bytes);
int msbg_gpu_host_free(void *hPtr);
/* Device memory helpers for callers without a CUDA runtime of their own. */
int msbg_gpu_device_alloc(void **dPtr, size_t bytes);
int msbg_gpu_device_free(void *dPtr);
int msbg_gpu_copy_d2d(msbg_gpu_ctx *ctx, void *dDst, const void *dSrc, size_t bytes);
int msbg_gpu_copy_h2d(msbg_gpu_ctx *ctx, void *dDst, const void *hSrc, size_t bytes);
int msbg_gpu_copy_d2h(msbg_gpu_ctx *ctx, void *hDst, const void *dSrc, size_t bytes);

#ifdef __cplusplus
}
#endif
#endif /* MSBG_GPU_H */
