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
 */
#ifndef MSBG_ORACLE_COMMON_H
#define MSBG_ORACLE_COMMON_H

#include <stdint.h>

#define ORACLE_JOB_MAGIC "MSBGJOB2"
#define ORACLE_OUT_MAGIC "MSBGOUT2"

enum { ORACLE_CHAN_F32 = 0, ORACLE_CHAN_U16 = 1 };
enum { ORACLE_JOB_SURFACE = 1, ORACLE_JOB_LEVELS = 2 };

typedef struct {
  char magic[8];
  int32_t jobType;  /* ORACLE_JOB_* */
  int32_t sx, sy, sz, bsx;
  int32_t nLevels;  /* resolution levels of the grid (3 in the demo) */
  int32_t chanType; /* ORACLE_CHAN_* */
  int32_t nIter;    /* applyChannelPdeFast numIter (rounded up to even inside) */
  int32_t laplTyp;  /* applyChannelPdeFast laplTyp, signed as the reference wants */
  int32_t constr01; /* doConstrZeroOne */
  int32_t nThreads; /* OpenMP threads for the reference's parallel loops */
  float dt;         /* applyChannelPdeFast timeStep */
  float rParticle;  /* splat kernel radius (demo: 2) */
  float nbDist;     /* narrow band added to the scan radius (demo: 2) */
  float anisAlpha;  /* applyChannelPdeFast anisDiffAlpha (Perona-Malik) */
  int32_t reserved; /* keeps the int64 fields 8-byte aligned */
  int64_t nPoints;  /* surface job: float32 xyz follow; levels job: 0 */
  int64_t nBlocksIn;/* levels job: int32 levels[nBlocksIn] follow */
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
   *       payloadAfterFinalize[nActive*bsx^3]; payloadAfterPde[nActive*bsx^3] */
} OracleOutHeader;

#endif
