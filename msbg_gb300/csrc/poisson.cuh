// Internal declarations of the sparse Poisson solver (poisson.cu).
#pragma once

#include <vector>

#include "internal.cuh"

namespace msbg {

// Geometry of one multigrid level, passed by value to kernels.
struct LvGeom {
  int bs, log2bs, nbx, nby, nbz;
  int64_t nCell;
  const int32_t *slot;    // [nbx*nby*nbz] slot or -1
  const int32_t *active;  // [nAct] block ids
};

struct MgLevel {
  int bs = 0, log2bs = 0, nbx = 0, nby = 0, nbz = 0;
  int64_t nAct = 0, nCell = 0;
  int32_t *slot = nullptr, *active = nullptr;
  bool ownsIndex = false;
  float *x = nullptr, *b = nullptr, *r = nullptr;             // levels >= 1
  float *cx = nullptr, *cy = nullptr, *cz = nullptr, *d = nullptr;  // lower faces, diagonal
};

struct PoissonState {
  int64_t layoutStamp = -1;
  std::vector<MgLevel> levels;
  bool coeffsValid = false;
  float *r = nullptr, *p = nullptr, *z = nullptr, *s = nullptr;  // CG vectors on level 0
  double *dPartial = nullptr;
  int nPartial = 0;
  double *dScal = nullptr, *hScal = nullptr;
  int preSweeps = 2, postSweeps = 2;
  int coarsestIter = 200;
  int64_t coarsestCells = 512;
};

void poissonFree(PoissonState *ps);
int poissonEnsure(msbg_gpu_ctx *ctx);
LvGeom geomOf(const MgLevel &L);

}  // namespace msbg
