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

struct MgLevel {  // geometry of one level (arrays live in PrecSet)
  int bs = 0, log2bs = 0, nbx = 0, nby = 0, nbz = 0;
  int64_t nAct = 0, nCell = 0;
  int32_t *slot = nullptr, *active = nullptr;
  bool ownsIndex = false;
};

// Arrays of one storage precision: per level x, b, r (levels >= 1) and the
// coefficients (lower faces cx, cy, cz and diagonal d); level-0 work vectors.
struct PrecSet {
  std::vector<void *> x, b, r, cx, cy, cz, d;
  void *vr = nullptr, *vp = nullptr, *vz = nullptr, *vs = nullptr, *ve = nullptr, *vb = nullptr;
};

struct PoissonState {
  int64_t layoutStamp = -1;
  std::vector<MgLevel> levels;
  bool coeffsValid = false, f16Valid = false;
  PrecSet f32, f16;
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
