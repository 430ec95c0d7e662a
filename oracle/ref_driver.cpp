/*
 * Oracle driver linked against the MSBG reference library (compiled from the
 * reference's own sources by oracle/Makefile).  Test infrastructure only.
 *
 * Usage:  msbg_ref_driver <job.bin> <out.bin>
 *
 * The demo's marking / splat / finalize loops live in the application, not in
 * the library (src/msbg_demo.cpp:326-680), so this driver restates them with the
 * library's own types and index helpers, keeping every step of their
 * arithmetic and their control flow (including the "abort this particle on a
 * non-value block" rule at src/msbg_demo.cpp:613-618).  Everything else is the
 * library itself: MultiresSparseGrid::create, regularizeRefinementMap,
 * setRefinementMap, SparseGrid block management, applyChannelPdeFast<T>, the
 * trilinear interpolation functions (interp job), HaloBlockSet::fillHaloBlock_<T>
 * (halo job), the ray-march renderer RDR::RaymarchRenderer (render job),
 * sortBlockListMorton (morton job), the solver building blocks
 * multiplyLaplacianMatrixOpt / dotProdChannel / AXPBYChannelCombined / relaxBlockList
 * (solver job), the same operator on a multi-resolution layout (multires job) and at a
 * dense multigrid level (dense job), and
 * downsampleFloatChannelNew (downsample job).
 *
 * Differences from the demo, both forced by the workload definition:
 *  - points come from the job file (already in voxel coordinates) instead of
 *    the bunny instancing of src/msbg_demo.cpp:349-356;
 *  - an FP32 channel (CH_FLOAT_1) stores floats directly, because the demo's
 *    renderDensFromFloat_<float> scales by FLT_MAX (src/sbg.h:302-314).
 */
#include <omp.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <type_traits>
#include <vector>

#include "msbg.h"
#include "halo.h"
#include "render.h"
#include "oracle_common.h"

extern int nMaxThreads;

namespace {

using MSBG::MultiresSparseGrid;
using SBG::SparseGrid;

double nowSec() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

// Storage conversions that mirror src/sbg.h:236-296 for uint16 and are the identity for
// float (the FP32 harness stores values directly).
template <typename T> struct Quant;
template <> struct Quant<float> {
  static float fromFloat(float f) { return f; }
  static float toFloat(float v) { return v; }
  static float one() { return 1.0f; }
  static float zero() { return 0.0f; }
};
template <> struct Quant<uint16_t> {
  static uint16_t fromFloat(float f) { return SBG::renderDensFromFloat_<uint16_t>(f); }
  static float toFloat(uint16_t v) { return SBG::renderDensToFloat_<uint16_t>(v); }
  static uint16_t one() { return fromFloat(1.0f); }
  static uint16_t zero() { return fromFloat(0.0f); }
};

struct Particle {
  float x, y, z;
  uint32_t next;  // 0 = end of list; particle i is stored at slot i+1
};

template <typename T>
int runSurfaceJob(const OracleJobHeader &job, const float *pts, const int32_t *levelsIn, FILE *fout) {
  OracleOutHeader out;
  memset(&out, 0, sizeof(out));
  memcpy(out.magic, ORACLE_OUT_MAGIC, 8);

  const int chan = (sizeof(T) == 4) ? MSBG::CH_FLOAT_1 : MSBG::CH_UINT16_1;
  MultiresSparseGrid *msbg = MultiresSparseGrid::create(
      "TEST", job.sx, job.sy, job.sz, job.bsx, -1, 0, -1,
      MSBG::OPT_SINGLE_LEVEL | MSBG::OPT_SINGLE_CHANNEL_FLOAT);
  if (!msbg) return 2;
  SparseGrid<T> *sg0 = MSBG::getChannel<T>(msbg, chan, 0);
  if (!sg0) return 3;

  const int nBlocks = msbg->nBlocks();
  const float rParticle = job.rParticle, nbDist = job.nbDist;
  const float rScan = rParticle + nbDist;

  std::vector<long> blockActive(nBlocks, 0);
  std::vector<uint32_t> listHead(nBlocks, 0);
  std::vector<Particle> parts((size_t)job.nPoints + 1);
  int64_t nAct = 0;

  // ---- active-block marking + per-block particle lists (demo 339-397) ----
  double t0 = nowSec();
  {
    const int bxMax = sg0->nbx() - 1, byMax = sg0->nby() - 1, bzMax = sg0->nbz() - 1;
    const float scale2Blk = 1.0f / (float)sg0->bsx();
    const float rScanBsx = rScan / (float)sg0->bsx();
    const int nxBlk = sg0->nbx(), nxyBlk = sg0->nbxy();
    const int bsxLog2 = sg0->bsxLog2();
#pragma omp parallel for schedule(static) reduction(+ : nAct)
    for (int64_t i = 0; i < job.nPoints; i++) {
      const float px = pts[3 * i], py = pts[3 * i + 1], pz = pts[3 * i + 2];
      Vec4f pos(px, py, pz, 0.f);
      if (!msbg->isInDomainRange(pos)) continue;
      const int ix = (int)px, iy = (int)py, iz = (int)pz;
      if (!sg0->inRange(Vec4i(ix, iy, iz, 0))) continue;
      Particle &p = parts[i + 1];
      p.x = px; p.y = py; p.z = pz;
      const float bx = px * scale2Blk, by = py * scale2Blk, bz = pz * scale2Blk;
      const int bx1 = std::max((int)(bx - rScanBsx), 0), bx2 = std::min((int)(bx + rScanBsx), bxMax);
      const int by1 = std::max((int)(by - rScanBsx), 0), by2 = std::min((int)(by + rScanBsx), byMax);
      const int bz1 = std::max((int)(bz - rScanBsx), 0), bz2 = std::min((int)(bz + rScanBsx), bzMax);
      for (int k = bz1; k <= bz2; k++)
        for (int j = by1; j <= by2; j++)
          for (int l = bx1; l <= bx2; l++) {
            const int bid = sg0->getBlockIndex(l, j, k);
            __atomic_fetch_add(&blockActive[bid], 1, __ATOMIC_RELAXED);
          }
      const int bidOwn = (iz >> bsxLog2) * nxyBlk + (iy >> bsxLog2) * nxBlk + (ix >> bsxLog2);
      p.next = __atomic_exchange_n(&listHead[bidOwn], (uint32_t)(i + 1), __ATOMIC_RELAXED);
      nAct++;
    }
  }
  out.tMarkSec = nowSec() - t0;
  out.nActParticles = nAct;

  // ---- level map + regularize + setRefinementMap (demo 413-436) ----
  t0 = nowSec();
  std::vector<int> levels(nBlocks);
  for (int b = 0; b < nBlocks; b++) levels[b] = blockActive[b] ? 0 : msbg->getNumLevels() - 1;
  if (job.nBlocksIn == nBlocks && levelsIn) {
    // caller-supplied level map (used to provoke the splat's abort rule)
    for (int b = 0; b < nBlocks; b++) levels[b] = levelsIn[b];
  }
  msbg->regularizeRefinementMap(levels.data());
  msbg->setRefinementMap(levels.data(), NULL, -1, NULL, false);
  out.tLevelsSec = nowSec() - t0;

  // ---- allocate level-0 blocks, value 1.0; others become the const empty block (demo 455-511) ----
  t0 = nowSec();
  std::vector<int> activeBlocks;
  sg0->reset();
  sg0->prepareDataAccess();
  sg0->setEmptyValue(Quant<T>::zero());
  sg0->setFullValue(Quant<T>::one());
  for (int bid = 0; bid < nBlocks; bid++) {
    MSBG::BlockInfo *bi = msbg->getBlockInfo(bid);
    bi->flags &= ~MSBG::BLK_EXISTS;
    if (bi->level > 0) {
      sg0->setEmptyBlock(bid);
      continue;
    }
    activeBlocks.push_back(bid);
    bi->flags |= MSBG::BLK_EXISTS;
    T *data = sg0->getBlockDataPtr(bid, 1, 0);
    for (int v = 0; v < sg0->nVoxelsInBlock(); v++) data[v] = Quant<T>::one();
  }
  out.tAllocSec = nowSec() - t0;
  out.nActive = (int)activeBlocks.size();

  // ---- 8-color splat of min(distSq/distSqMax) (demo 527-636) ----
  t0 = nowSec();
  {
    const float distSqMax = rScan * rScan, distSqMaxInv = 1.0f / distSqMax;
    std::vector<int> perColor[8];
    for (int bid : activeBlocks) {
      int bx, by, bz;
      sg0->getBlockCoordsById(bid, bx, by, bz);
      perColor[MSBG::getBlockColor8(bx, by, bz)].push_back(bid);
    }
    const int bsxLog2 = sg0->bsxLog2(), bsx2Log2 = sg0->bsx2Log2(), bsxMask = sg0->bsx() - 1;
    const int nx = sg0->nbx(), nxy = sg0->nbxy();
    const int xMax = job.sx - 1, yMax = job.sy - 1, zMax = job.sz - 1;
    for (int c = 0; c < 8; c++) {
      const std::vector<int> &lst = perColor[c];
#pragma omp parallel for schedule(dynamic, 1)
      for (size_t t = 0; t < lst.size(); t++) {
        const int bid = lst[t];
        for (uint32_t ixp = listHead[bid]; ixp; ixp = parts[ixp].next) {
          const Particle &p = parts[ixp];
          const int ix1 = std::max((int)std::ceil(p.x - rScan - 0.5f), 0);
          const int iy1 = std::max((int)std::ceil(p.y - rScan - 0.5f), 0);
          const int iz1 = std::max((int)std::ceil(p.z - rScan - 0.5f), 0);
          const int ix2 = std::min((int)std::floor(p.x + rScan - 0.5f), xMax);
          const int iy2 = std::min((int)std::floor(p.y + rScan - 0.5f), yMax);
          const int iz2 = std::min((int)std::floor(p.z + rScan - 0.5f), zMax);
          const float x0 = p.x - 0.5f, y0 = p.y - 0.5f, z0 = p.z - 0.5f;
          bool aborted = false;
          for (int iz = iz1; iz <= iz2 && !aborted; iz++) {
            const float dz = iz - z0;
            const int ibz = (iz >> bsxLog2) * nxy, ivz = (iz & bsxMask) << bsx2Log2;
            for (int iy = iy1; iy <= iy2 && !aborted; iy++) {
              const float dy = iy - y0;
              const float dzy = dz * dz + dy * dy;
              const int ibzy = ibz + (iy >> bsxLog2) * nx, ivzy = ivz + ((iy & bsxMask) << bsxLog2);
              for (int ix = ix1; ix <= ix2; ix++) {
                const float dx = ix - x0;
                const float d2 = dzy + dx * dx;
                if (d2 > distSqMax) continue;
                SBG::Block<T> *blk = sg0->getBlock(ibzy + (ix >> bsxLog2));
                if (!sg0->isValueBlock(blk)) { aborted = true; break; }
                const int iv = ivzy + (ix & bsxMask);
                const T val = Quant<T>::fromFloat(d2 * distSqMaxInv);
                if (val < blk->_data[iv]) blk->_data[iv] = val;
              }
            }
          }
        }
      }
    }
  }
  out.tSplatSec = nowSec() - t0;

  // ---- finalize: distance -> density with iso 0.5 (demo 655-680) ----
  t0 = nowSec();
  {
    const float distSqMax = rScan * rScan;
#pragma omp parallel for schedule(static)
    for (size_t t = 0; t < activeBlocks.size(); t++) {
      T *data = sg0->getBlockDataPtr(activeBlocks[t]);
      for (int v = 0; v < sg0->nVoxelsInBlock(); v++) {
        float d = Quant<T>::toFloat(data[v]);
        T q = Quant<T>::fromFloat(0.0f);
        if (d < 0.999f) {
          d *= distSqMax;
          const float dist = sqrtf(d) - rParticle;
          const float f = 1.0f - MT_LINSTEPF(-rParticle, rParticle + nbDist, dist);
          q = Quant<T>::fromFloat(f);
        }
        data[v] = q;
      }
    }
  }
  out.tFinalSec = nowSec() - t0;

  const size_t nv = (size_t)sg0->nVoxelsInBlock();
  std::vector<T> afterFinal(activeBlocks.size() * nv);
  for (size_t t = 0; t < activeBlocks.size(); t++)
    memcpy(&afterFinal[t * nv], sg0->getBlockDataPtr(activeBlocks[t]), nv * sizeof(T));

  // ---- the library's sweep (demo 716-727) ----
  t0 = nowSec();
  if (job.nIter > 0) {
    // Colored schedules update in place; the plain ping-pong schedule needs a
    // temporary channel of the same type.
    const int chTmp = job.laplTyp < 0 ? (int)MSBG::CH_NULL
                                      : (sizeof(T) == 4 ? (int)MSBG::CH_FLOAT_2 : (int)MSBG::CH_UINT16_2);
    msbg->applyChannelPdeFast<T>(chan, chTmp, MSBG::CH_NULL, &activeBlocks, job.laplTyp,
                                 job.constr01, 0, 0, 0, job.nIter, 1.0f, job.dt, 0, NULL, 0, 0, 0,
                                 0, job.anisAlpha, 0, 0, 0);
  }
  out.tPdeSec = nowSec() - t0;

  std::vector<int8_t> lev8(nBlocks);
  std::vector<uint16_t> flags(nBlocks);
  for (int b = 0; b < nBlocks; b++) {
    lev8[b] = (int8_t)msbg->getBlockInfo(b)->level;
    flags[b] = msbg->getBlockInfo(b)->flags;
    if (lev8[b] >= 0 && lev8[b] < 8) out.nBlocksPerLevel[lev8[b]]++;
  }
  out.nBlocks = nBlocks;
  out.elemBytes = (int)sizeof(T);
  out.nThreadsUsed = omp_get_max_threads();

  fwrite(&out, sizeof(out), 1, fout);
  fwrite(lev8.data(), 1, nBlocks, fout);
  fwrite(flags.data(), 2, nBlocks, fout);
  fwrite(activeBlocks.data(), 4, activeBlocks.size(), fout);
  fwrite(afterFinal.data(), sizeof(T), afterFinal.size(), fout);
  for (size_t t = 0; t < activeBlocks.size(); t++)
    fwrite(sg0->getBlockDataPtr(activeBlocks[t]), sizeof(T), nv, fout);

  MultiresSparseGrid::destroy(msbg);
  return 0;
}

// Multi-level layout: regularizeRefinementMap then setRefinementMap on the full
// (non-single-level) grid; dumps the per-block level and BlockInfo flags.
int runLevelsJob(const OracleJobHeader &job, const int32_t *levelsIn, FILE *fout) {
  OracleOutHeader out;
  memset(&out, 0, sizeof(out));
  memcpy(out.magic, ORACLE_OUT_MAGIC, 8);
  MultiresSparseGrid *msbg = MultiresSparseGrid::create(
      "TEST", job.sx, job.sy, job.sz, job.bsx, -1, 0, -1, 0, NULL, NULL, job.nLevels);
  if (!msbg) return 2;
  const int nBlocks = msbg->nBlocks();
  if ((int64_t)nBlocks != job.nBlocksIn) return 4;
  std::vector<int> levels(levelsIn, levelsIn + nBlocks);
  double t0 = nowSec();
  msbg->regularizeRefinementMap(levels.data());
  msbg->setRefinementMap(levels.data(), NULL, 0, NULL, false, false);
  out.tLevelsSec = nowSec() - t0;
  std::vector<int8_t> lev8(nBlocks);
  std::vector<uint16_t> flags(nBlocks);
  for (int b = 0; b < nBlocks; b++) {
    lev8[b] = (int8_t)levels[b];
    flags[b] = msbg->getBlockInfo(b, 0)->flags;
    if (levels[b] >= 0 && levels[b] < 8) out.nBlocksPerLevel[levels[b]]++;
  }
  out.nBlocks = nBlocks;
  out.nThreadsUsed = omp_get_max_threads();
  fwrite(&out, sizeof(out), 1, fout);
  fwrite(lev8.data(), 1, nBlocks, fout);
  fwrite(flags.data(), 2, nBlocks, fout);
  MultiresSparseGrid::destroy(msbg);
  return 0;
}

// Interpolation of a given payload at query points by the reference's own functions
// (src/sbg.h:4623-4792, src/sbg.h:4920-5032, src/msbg.h:478-484).  The grid is the
// single-level one of the surface job; value blocks get the caller's payload and every
// other block is the constant empty block (empty value 0).
template <typename T>
int runInterpJob(const OracleJobHeader &job, const float *pts, const int32_t *bids,
                 const T *payload, FILE *fout) {
  OracleOutHeader out;
  memset(&out, 0, sizeof(out));
  memcpy(out.magic, ORACLE_OUT_MAGIC, 8);
  const int chan = (sizeof(T) == 4) ? MSBG::CH_FLOAT_1 : MSBG::CH_UINT16_1;
  MultiresSparseGrid *msbg = MultiresSparseGrid::create(
      "TEST", job.sx, job.sy, job.sz, job.bsx, -1, 0, -1,
      MSBG::OPT_SINGLE_LEVEL | MSBG::OPT_SINGLE_CHANNEL_FLOAT);
  if (!msbg) return 2;
  SparseGrid<T> *sg0 = MSBG::getChannel<T>(msbg, chan, 0);
  if (!sg0) return 3;
  const int nBlocks = msbg->nBlocks();
  std::vector<int> levels(nBlocks, msbg->getNumLevels() - 1);
  for (int64_t t = 0; t < job.nBlocksIn; t++) {
    if (bids[t] < 0 || bids[t] >= nBlocks) return 4;
    levels[bids[t]] = 0;
  }
  msbg->regularizeRefinementMap(levels.data());
  msbg->setRefinementMap(levels.data(), NULL, -1, NULL, false);
  sg0->reset();
  sg0->prepareDataAccess();
  sg0->setEmptyValue(Quant<T>::zero());
  sg0->setFullValue(Quant<T>::one());
  for (int bid = 0; bid < nBlocks; bid++) sg0->setEmptyBlock(bid);
  const size_t nv = (size_t)sg0->nVoxelsInBlock();
  for (int64_t t = 0; t < job.nBlocksIn; t++) {
    T *data = sg0->getBlockDataPtr(bids[t], 1, 0);
    memcpy(data, payload + (size_t)t * nv, nv * sizeof(T));
  }
  const int opt = job.constr01;
  std::vector<float> vals((size_t)job.nPoints);
  const double t0 = nowSec();
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < job.nPoints; i++) {
    const Vec4f pos(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2], 0.f);
    float f;
    if constexpr (sizeof(T) == 4) {
      f = sg0->interpolateFloatFast(pos, opt & ~ORACLE_IP_RENDER_DENS);
    } else {
      if (opt & ORACLE_IP_RENDER_DENS)
        f = MSBG::interpolateRenderDensity(sg0, pos, opt & ~ORACLE_IP_RENDER_DENS);
      else
        f = sg0->interpolateUint16ToFloatFast(pos, opt);
    }
    vals[i] = f;
  }
  out.tPdeSec = nowSec() - t0;
  out.nBlocks = nBlocks;
  out.nActive = (int)job.nBlocksIn;
  out.elemBytes = (int)sizeof(T);
  out.nThreadsUsed = omp_get_max_threads();
  fwrite(&out, sizeof(out), 1, fout);
  fwrite(vals.data(), 4, vals.size(), fout);
  MultiresSparseGrid::destroy(msbg);
  return 0;
}

// Cross-resolution halo fill by the reference's own HaloBlockSet::fillHaloBlock_<T>
// (src/halo.cpp:266-479).  A multi-level grid on the job's level map; every resolution
// level l of the channel gets the job's block states (payload / constant empty /
// constant full / no block) and payloads; then every block at level job.laplTyp that
// has a block at that level is filled with halo size job.nIter and options job.constr01.
template <typename T>
int runHaloJob(const OracleJobHeader &job, const int32_t *levelsIn, const int32_t *state,
               const std::vector<std::vector<uint8_t>> &pay, FILE *fout) {
  OracleOutHeader out;
  memset(&out, 0, sizeof(out));
  memcpy(out.magic, ORACLE_OUT_MAGIC, 8);
  const int chan = (sizeof(T) == 4) ? MSBG::CH_FLOAT_1 : MSBG::CH_UINT16_1;
  MultiresSparseGrid *msbg = MultiresSparseGrid::create(
      "TEST", job.sx, job.sy, job.sz, job.bsx, -1, 0, -1, 0, NULL, NULL, job.nLevels);
  if (!msbg) return 2;
  const int nBlocks = msbg->nBlocks();
  if ((int64_t)nBlocks != job.nBlocksIn) return 4;
  std::vector<int> levels(levelsIn, levelsIn + nBlocks);
  msbg->regularizeRefinementMap(levels.data());
  for (int b = 0; b < nBlocks; b++)
    if (levels[b] != levelsIn[b]) return 5;  // the job's map must already be regular
  msbg->setRefinementMap(levels.data(), NULL, 0, NULL, false, false);
  for (int l = 0; l < job.nLevels; l++) {
    SparseGrid<T> *sg = MSBG::getChannel<T>(msbg, chan, l);
    if (!sg) return 3;
    sg->reset();
    sg->prepareDataAccess();
    sg->setEmptyValue(Quant<T>::fromFloat(job.dt));
    sg->setFullValue(Quant<T>::fromFloat(job.rParticle));
    const size_t nv = (size_t)sg->nVoxelsInBlock();
    const int32_t *st = state + (size_t)l * nBlocks;
    const T *src = reinterpret_cast<const T *>(pay[l].data());
    for (int b = 0; b < nBlocks; b++) {
      if (st[b] >= 0) {
        T *data = sg->getBlockDataPtr(b, 1, 0);
        memcpy(data, src + (size_t)st[b] * nv, nv * sizeof(T));
      } else if (st[b] == -1) {
        sg->setEmptyBlock(b);
      } else if (st[b] == -2) {
        sg->setFullBlock(b);
      }
    }
  }
  const int L = job.laplTyp, h = job.nIter;
  const int bs = job.bsx >> L, hs = bs + 2 * h;
  std::vector<int32_t> bids;
  for (int b = 0; b < nBlocks; b++)
    if (levels[b] == L && state[(size_t)L * nBlocks + b] != -3) bids.push_back(b);
  std::vector<float> halo(bids.size() * (size_t)hs * hs * hs);
  MSBG::HaloBlockSet hb(msbg, h, 1);
  const double t0 = nowSec();
  for (size_t k = 0; k < bids.size(); k++) {
    float **p = hb.fillHaloBlock_<T>(chan, bids[k], 0, 0, (unsigned)job.constr01);
    memcpy(halo.data() + k * (size_t)hs * hs * hs, p[0], sizeof(float) * hs * hs * hs);
  }
  out.tPdeSec = nowSec() - t0;
  out.nBlocks = nBlocks;
  out.nActive = (int)bids.size();
  out.elemBytes = (int)sizeof(T);
  out.nThreadsUsed = 1;
  fwrite(&out, sizeof(out), 1, fout);
  fwrite(bids.data(), 4, bids.size(), fout);
  fwrite(halo.data(), 4, halo.size(), fout);
  MultiresSparseGrid::destroy(msbg);
  return 0;
}

// The demo's ray-march renderer (src/render.h:52-160, src/render.cpp:20-101) on a uint16
// payload loaded into the value blocks of a single-level grid, as the interp job does.
int runRenderJob(const OracleJobHeader &job, const float *cam, const int32_t *bids,
                 const uint16_t *payload, FILE *fout) {
  OracleOutHeader out;
  memset(&out, 0, sizeof(out));
  memcpy(out.magic, ORACLE_OUT_MAGIC, 8);
  MultiresSparseGrid *msbg = MultiresSparseGrid::create(
      "TEST", job.sx, job.sy, job.sz, job.bsx, -1, 0, -1,
      MSBG::OPT_SINGLE_LEVEL | MSBG::OPT_SINGLE_CHANNEL_FLOAT);
  if (!msbg) return 2;
  SparseGrid<uint16_t> *sg0 = MSBG::getChannel<uint16_t>(msbg, MSBG::CH_UINT16_1, 0);
  if (!sg0) return 3;
  const int nBlocks = msbg->nBlocks();
  std::vector<int> levels(nBlocks, msbg->getNumLevels() - 1);
  for (int64_t t = 0; t < job.nBlocksIn; t++) {
    if (bids[t] < 0 || bids[t] >= nBlocks) return 4;
    levels[bids[t]] = 0;
  }
  msbg->regularizeRefinementMap(levels.data());
  msbg->setRefinementMap(levels.data(), NULL, -1, NULL, false);
  sg0->reset();
  sg0->prepareDataAccess();
  sg0->setEmptyValue(0);
  sg0->setFullValue(65535);
  for (int bid = 0; bid < nBlocks; bid++) sg0->setEmptyBlock(bid);
  const size_t nv = (size_t)sg0->nVoxelsInBlock();
  for (int64_t t = 0; t < job.nBlocksIn; t++) {
    uint16_t *data = sg0->getBlockDataPtr(bids[t], 1, 0);
    memcpy(data, payload + (size_t)t * nv, nv * sizeof(uint16_t));
  }
  const int w = job.nIter, h = job.laplTyp;
  RDR::RaymarchRenderer renderer(w, h, sg0);
  // the demo passes float camera values (src/msbg_demo.cpp:123-127, 143-147)
  renderer.setCamera({cam[0], cam[1], cam[2]}, {cam[3], cam[4], cam[5]}, cam[12]);
  renderer.setSunLight({cam[6], cam[7], cam[8]});
  renderer.setSurfaceColor({cam[9], cam[10], cam[11]});
  const double t0 = nowSec();
  BmpBitmap *B = renderer.render();
  out.tPdeSec = nowSec() - t0;
  if (!B) return 6;
  out.nBlocks = nBlocks;
  out.nActive = w * h;
  out.elemBytes = 2;
  out.nThreadsUsed = omp_get_max_threads();
  fwrite(&out, sizeof(out), 1, fout);
  fwrite(B->data, 4, (size_t)w * h, fout);
  MultiresSparseGrid::destroy(msbg);
  return 0;
}

// MultiresSparseGrid::sortBlockListMorton (src/msbg2.cpp:46-58) of a list of block ids.
int runMortonJob(const OracleJobHeader &job, const int32_t *bids, FILE *fout) {
  OracleOutHeader out;
  memset(&out, 0, sizeof(out));
  memcpy(out.magic, ORACLE_OUT_MAGIC, 8);
  MultiresSparseGrid *msbg = MultiresSparseGrid::create(
      "TEST", job.sx, job.sy, job.sz, job.bsx, -1, 0, -1,
      MSBG::OPT_SINGLE_LEVEL | MSBG::OPT_SINGLE_CHANNEL_FLOAT);
  if (!msbg) return 2;
  std::vector<int> list(bids, bids + job.nBlocksIn);
  for (int b : list)
    if (b < 0 || b >= msbg->nBlocks()) return 4;
  const double t0 = nowSec();
  msbg->sortBlockListMorton(list);
  out.tPdeSec = nowSec() - t0;
  out.nBlocks = msbg->nBlocks();
  out.nActive = (int)list.size();
  fwrite(&out, sizeof(out), 1, fout);
  fwrite(list.data(), 4, list.size(), fout);
  MultiresSparseGrid::destroy(msbg);
  return 0;
}


// Loads one channel of a single-level grid: value blocks (bids) get their payload from
// src ([n][bs^3]), every other block is the channel's constant empty block (value 0).
template <typename T>
void loadValueBlocks(SparseGrid<T> *sg, const std::vector<int32_t> &bids, const T *src, int nBlocks,
                     T emptyValue) {
  sg->reset();
  sg->prepareDataAccess();
  sg->setEmptyValue(emptyValue);
  for (int b = 0; b < nBlocks; b++) sg->setEmptyBlock(b);
  const size_t nv = (size_t)sg->nVoxelsInBlock();
  for (size_t t = 0; t < bids.size(); t++) {
    T *d = sg->getBlockDataPtr(bids[t], 1, 0);
    if (src)
      memcpy(d, src + t * nv, nv * sizeof(T));
    else
      for (size_t i = 0; i < nv; i++) d[i] = emptyValue;
  }
}

template <typename T>
void dumpValueBlocks(SparseGrid<T> *sg, const std::vector<int32_t> &bids, FILE *fout) {
  const size_t nv = (size_t)sg->nVoxelsInBlock();
  for (int32_t b : bids) fwrite(sg->getBlockDataPtr(b, 0, 0), sizeof(T), nv, fout);
}

// The solver building blocks of the reference on the value blocks of a single-resolution
// layout (every block at level 0; blocks without payload are constant empty blocks, so
// the operator sees Dirichlet 0 outside the value blocks):
//   multiplyLaplacianMatrixOpt (src/msbg3.cpp:1756-1912): Y = A X with its dot product
//     sum(Y X), and with OPT_CALC_RESIDUAL R = B - A X;
//   dotProdChannel_ (src/msbg.cpp:4524-4646): sum(X B);
//   AXPBYChannelCombined (src/msbg.cpp:4651-4768): X += a P; P = Q + b P;
//   relaxBlockList (src/msbg3.cpp:2170-2239) run job.nIter times as relax() runs it
//     (src/msbg3.cpp:2244-2369): red-black over blocks, _mgSmBlockIter block-local
//     Gauss-Seidel iterations with omega = _mgSmOmega (src/msbg.cpp:814-843).
// The release fills none of the solver's coefficient channels, so this job writes them:
// the face-area channels hold the lower-face coefficients cx, cy, cz of every cell (read
// because each value block is flagged BLK_CUTS_SOLID and each cell CELL_PARTIAL_SOLID),
// CH_DIAGONAL the reciprocal of the diagonal (the operator multiplies by 1/D,
// src/msbg3.cpp:1300-1302).  Inputs after the header: int32 bids[n], then float32
// [n][bs^3] arrays X, B, Q, P, CX, CY, CZ, DINV.  Header: dt = a, rParticle = b,
// nIter = relax passes, constr01 = 1 for the reverse order.
int runSolverJob(const OracleJobHeader &job, const int32_t *bidsIn, const float *arrays, FILE *fout) {
  OracleOutHeader out;
  memset(&out, 0, sizeof(out));
  memcpy(out.magic, ORACLE_OUT_MAGIC, 8);
  MultiresSparseGrid *msbg =
      MultiresSparseGrid::create("TEST", job.sx, job.sy, job.sz, job.bsx, -1, 0, -1, 0, NULL, NULL, 3);
  if (!msbg) return 2;
  const int nBlocks = msbg->nBlocks();
  std::vector<int32_t> bids(bidsIn, bidsIn + job.nBlocksIn);
  std::vector<char> isValue(nBlocks, 0);
  for (int32_t b : bids) {
    if (b < 0 || b >= nBlocks) return 4;
    isValue[b] = 1;
  }
  std::vector<int> levels(nBlocks, 0);
  msbg->setRefinementMap(levels.data(), NULL, 0, NULL, false, false);
  const size_t nv = (size_t)job.bsx * job.bsx * job.bsx, na = bids.size() * nv;
  const float *X = arrays, *B = X + na, *Q = B + na, *P = Q + na, *CX = P + na, *CY = CX + na,
              *CZ = CY + na, *DI = CZ + na;
  using MSBG::CH_PRESSURE;
  using MSBG::CH_DIVERGENCE;
  using MSBG::CH_CG_P;
  using MSBG::CH_CG_Q;
  using MSBG::CH_DIAGONAL;
  SparseGrid<PSFloat> *sgX = msbg->getPSFloatChannel(CH_PRESSURE, 0, 0),
                      *sgB = msbg->getPSFloatChannel(CH_DIVERGENCE, 0, 0),
                      *sgP = msbg->getPSFloatChannel(CH_CG_P, 0, 0),
                      *sgQ = msbg->getPSFloatChannel(CH_CG_Q, 0, 0),
                      *sgD = msbg->getPSFloatChannel(CH_DIAGONAL, 0, 0);
  if (!sgX || !sgB || !sgP || !sgQ || !sgD) return 3;
  loadValueBlocks<float>(sgD, bids, DI, nBlocks, 0.f);
  for (int k = 0; k < 3; k++) {
    SparseGrid<float> *fa = msbg->getFaceAreaChannel(k, 0, 0);
    if (!fa) return 3;
    loadValueBlocks<float>(fa, bids, k == 0 ? CX : k == 1 ? CY : CZ, nBlocks, 0.f);
  }
  {
    SparseGrid<MSBG::CellFlags> *sgF = msbg->getFlagsChannel(MSBG::CH_CELL_FLAGS, 0, 0);
    if (!sgF) return 3;
    sgF->reset();
    sgF->prepareDataAccess();
    sgF->setEmptyValue(MSBG::CELL_EMPTY_VAL);
    for (int b = 0; b < nBlocks; b++) sgF->setEmptyBlock(b);
    for (int32_t b : bids) {
      MSBG::CellFlags *f = sgF->getBlockDataPtr(b, 1, 0);
      for (size_t i = 0; i < nv; i++) f[i] = MSBG::CELL_PARTIAL_SOLID;
    }
  }
  for (int b = 0; b < nBlocks; b++) {
    MSBG::BlockInfo *bi = msbg->getBlockInfo(b, 0);
    if (isValue[b]) {
      bi->flags &= ~(MSBG::BLK_NO_FLUID | MSBG::BLK_FIXED | MSBG::BLK_ONLY_FLUID);
      bi->flags |= MSBG::BLK_CUTS_SOLID;
    } else {
      bi->flags |= MSBG::BLK_NO_FLUID;
    }
  }
  std::vector<int> list(bids.begin(), bids.end());
  auto loadXB = [&]() {
    loadValueBlocks<float>(sgX, bids, X, nBlocks, 0.f);
    loadValueBlocks<float>(sgB, bids, B, nBlocks, 0.f);
  };
  const double t0 = nowSec();
  // Y = A X (into CG_Q) with sum(Y X)
  loadXB();
  loadValueBlocks<float>(sgQ, bids, nullptr, nBlocks, 0.f);
  long double dotYX = 0;
  msbg->multiplyLaplacianMatrixOpt(0, 0, CH_PRESSURE, CH_DIVERGENCE, 0.f, CH_CG_Q, &dotYX, &list);
  std::vector<float> Y(na), R(na);
  for (size_t t = 0; t < bids.size(); t++) memcpy(&Y[t * nv], sgQ->getBlockDataPtr(bids[t], 0, 0), nv * 4);
  // R = B - A X (into CG_Q)
  msbg->multiplyLaplacianMatrixOpt(MSBG::OPT_CALC_RESIDUAL, 0, CH_PRESSURE, CH_DIVERGENCE, 0.f, CH_CG_Q, NULL,
                                   &list);
  for (size_t t = 0; t < bids.size(); t++) memcpy(&R[t * nv], sgQ->getBlockDataPtr(bids[t], 0, 0), nv * 4);
  int err = 0;
  const long double dotXB = msbg->dotProdChannel(CH_PRESSURE, CH_DIVERGENCE, 0, &list, &err);
  // X += a P; P = Q + b P
  loadValueBlocks<float>(sgQ, bids, Q, nBlocks, 0.f);
  loadValueBlocks<float>(sgP, bids, P, nBlocks, 0.f);
  msbg->AXPBYChannelCombined(job.dt, job.rParticle, CH_CG_Q, CH_PRESSURE, CH_CG_P, &list);
  std::vector<float> Xa(na), Pa(na);
  for (size_t t = 0; t < bids.size(); t++) {
    memcpy(&Xa[t * nv], sgX->getBlockDataPtr(bids[t], 0, 0), nv * 4);
    memcpy(&Pa[t * nv], sgP->getBlockDataPtr(bids[t], 0, 0), nv * 4);
  }
  // relax: nIter passes of relaxBlockList in place, as relax() does
  loadXB();
  const unsigned ropt = MSBG::OPT_JACOBI | (job.constr01 ? MSBG::OPT_REVERSE_ORDER : 0);
  for (int it = 0; it < job.nIter; it++) msbg->relaxBlockList(&list, 0, it, CH_PRESSURE, CH_DIVERGENCE, ropt, CH_PRESSURE);
  out.tPdeSec = nowSec() - t0;
  out.nBlocks = nBlocks;
  out.nActive = (int)bids.size();
  out.elemBytes = 4;
  out.nThreadsUsed = omp_get_max_threads();
  out.nActParticles = err;
  fwrite(&out, sizeof(out), 1, fout);
  const double dots[2] = {(double)dotYX, (double)dotXB};
  fwrite(dots, 8, 2, fout);
  fwrite(Y.data(), 4, na, fout);
  fwrite(R.data(), 4, na, fout);
  fwrite(Xa.data(), 4, na, fout);
  fwrite(Pa.data(), 4, na, fout);
  dumpValueBlocks<float>(sgX, bids, fout);
  MultiresSparseGrid::destroy(msbg);
  return 0;
}

// multiplyLaplacianMatrixOpt (src/msbg3.cpp:1756-1912) on a multi-resolution layout: every
// block of the job's level map (already regular) is a fluid block at its own level, so
// blocks of neighbouring levels meet through the mixed-resolution faces of
// procNeighMixedRes2 (src/msbg3.cpp:46-161) and the halo code around it
// (src/msbg3.cpp:664-1042).  No block cuts a solid (no face-area channels are read) and
// every cell is fluid (cell flags 0).  Inputs after the levels: float32 X, B and DINV (what
// CH_DIAGONAL holds; the operator multiplies by 1/DINV), each over the blocks of level 0,
// then level 1, ..., in ascending bid order, (bsx>>l)^3 values per block of level l.
// Output: sum(Y X) (FP64), then Y = A X and R = B - A X in the same order.  With
// job.nIter > 0, X is loaded again and relaxed by job.nIter passes of relaxBlockList
// (src/msbg3.cpp:2170-2239, red-black over the blocks of every level, constr01 = 1 for the
// reverse order), and the relaxed X follows in the same order.
int runMultiresJob(const OracleJobHeader &job, const int32_t *levelsIn, const float *arrays, FILE *fout) {
  OracleOutHeader out;
  memset(&out, 0, sizeof(out));
  memcpy(out.magic, ORACLE_OUT_MAGIC, 8);
  MultiresSparseGrid *msbg = MultiresSparseGrid::create(
      "TEST", job.sx, job.sy, job.sz, job.bsx, -1, 0, -1, 0, NULL, NULL, job.nLevels);
  if (!msbg) return 2;
  const int nBlocks = msbg->nBlocks();
  if ((int64_t)nBlocks != job.nBlocksIn) return 4;
  std::vector<int> levels(levelsIn, levelsIn + nBlocks);
  msbg->regularizeRefinementMap(levels.data());
  for (int b = 0; b < nBlocks; b++)
    if (levels[b] != levelsIn[b]) return 5;
  msbg->setRefinementMap(levels.data(), NULL, 0, NULL, false, false);
  using MSBG::CH_PRESSURE;
  using MSBG::CH_DIVERGENCE;
  using MSBG::CH_CG_Q;
  using MSBG::CH_DIAGONAL;
  std::vector<std::vector<int32_t>> bidsL(job.nLevels);
  for (int b = 0; b < nBlocks; b++) {
    if (levels[b] < 0 || levels[b] >= job.nLevels) return 4;
    bidsL[levels[b]].push_back(b);
  }
  size_t total = 0;
  for (int l = 0; l < job.nLevels; l++) {
    const size_t bs = (size_t)(job.bsx >> l);
    total += bidsL[l].size() * bs * bs * bs;
  }
  const float *X = arrays, *B = X + total, *DI = B + total;
  size_t off = 0;
  for (int l = 0; l < job.nLevels; l++) {
    SparseGrid<PSFloat> *sgX = msbg->getPSFloatChannel(CH_PRESSURE, l, 0),
                        *sgB = msbg->getPSFloatChannel(CH_DIVERGENCE, l, 0),
                        *sgQ = msbg->getPSFloatChannel(CH_CG_Q, l, 0),
                        *sgD = msbg->getPSFloatChannel(CH_DIAGONAL, l, 0);
    SparseGrid<MSBG::CellFlags> *sgF = msbg->getFlagsChannel(MSBG::CH_CELL_FLAGS, l, 0);
    if (!sgX || !sgB || !sgQ || !sgD || !sgF) return 3;
    loadValueBlocks<float>(sgX, bidsL[l], X + off, nBlocks, 0.f);
    loadValueBlocks<float>(sgB, bidsL[l], B + off, nBlocks, 0.f);
    loadValueBlocks<float>(sgD, bidsL[l], DI + off, nBlocks, 0.f);
    loadValueBlocks<float>(sgQ, bidsL[l], nullptr, nBlocks, 0.f);
    loadValueBlocks<MSBG::CellFlags>(sgF, bidsL[l], nullptr, nBlocks, 0);
    for (int k = 0; k < 3; k++) {  // allocated, read by no block (none cuts a solid)
      SparseGrid<float> *fa = msbg->getFaceAreaChannel(k, l, 0);
      if (!fa) return 3;
      loadValueBlocks<float>(fa, bidsL[l], nullptr, nBlocks, 1.f);
    }
    const size_t bs = (size_t)(job.bsx >> l);
    off += bidsL[l].size() * bs * bs * bs;
  }
  for (int b = 0; b < nBlocks; b++) {
    MSBG::BlockInfo *bi = msbg->getBlockInfo(b, 0);
    bi->flags &= ~(MSBG::BLK_NO_FLUID | MSBG::BLK_FIXED | MSBG::BLK_ONLY_FLUID | MSBG::BLK_CUTS_SOLID);
  }
  auto dumpQ = [&](std::vector<float> &dst) {
    dst.resize(total);
    size_t o = 0;
    for (int l = 0; l < job.nLevels; l++) {
      SparseGrid<PSFloat> *sgQ = msbg->getPSFloatChannel(CH_CG_Q, l, 0);
      const size_t nv = (size_t)sgQ->nVoxelsInBlock();
      for (int32_t b : bidsL[l]) {
        memcpy(&dst[o], sgQ->getBlockDataPtr(b, 0, 0), nv * 4);
        o += nv;
      }
    }
  };
  std::vector<int> list;
  for (int l = 0; l < job.nLevels; l++) list.insert(list.end(), bidsL[l].begin(), bidsL[l].end());
  const double t0 = nowSec();
  long double dotYX = 0;
  msbg->multiplyLaplacianMatrixOpt(0, 0, CH_PRESSURE, CH_DIVERGENCE, 0.f, CH_CG_Q, &dotYX, &list);
  std::vector<float> Y, R;
  dumpQ(Y);
  msbg->multiplyLaplacianMatrixOpt(MSBG::OPT_CALC_RESIDUAL, 0, CH_PRESSURE, CH_DIVERGENCE, 0.f, CH_CG_Q, NULL,
                                   &list);
  dumpQ(R);
  std::vector<float> Xr;
  if (job.nIter > 0) {
    size_t o = 0;
    for (int l = 0; l < job.nLevels; l++) {
      SparseGrid<PSFloat> *sgX = msbg->getPSFloatChannel(CH_PRESSURE, l, 0);
      const size_t nv = (size_t)sgX->nVoxelsInBlock();
      for (int32_t b : bidsL[l]) {
        memcpy(sgX->getBlockDataPtr(b, 0, 0), X + o, nv * 4);
        o += nv;
      }
    }
    const unsigned ropt = MSBG::OPT_JACOBI | (job.constr01 ? MSBG::OPT_REVERSE_ORDER : 0);
    for (int it = 0; it < job.nIter; it++)
      msbg->relaxBlockList(&list, 0, it, CH_PRESSURE, CH_DIVERGENCE, ropt, CH_PRESSURE);
    Xr.resize(total);
    o = 0;
    for (int l = 0; l < job.nLevels; l++) {
      SparseGrid<PSFloat> *sgX = msbg->getPSFloatChannel(CH_PRESSURE, l, 0);
      const size_t nv = (size_t)sgX->nVoxelsInBlock();
      for (int32_t b : bidsL[l]) {
        memcpy(&Xr[o], sgX->getBlockDataPtr(b, 0, 0), nv * 4);
        o += nv;
      }
    }
  }
  out.tPdeSec = nowSec() - t0;
  out.nBlocks = nBlocks;
  out.nActive = nBlocks;
  for (int l = 0; l < job.nLevels && l < 8; l++) out.nBlocksPerLevel[l] = (int64_t)bidsL[l].size();
  out.elemBytes = 4;
  out.nThreadsUsed = omp_get_max_threads();
  fwrite(&out, sizeof(out), 1, fout);
  const double dot = (double)dotYX;
  fwrite(&dot, 8, 1, fout);
  fwrite(Y.data(), 4, total, fout);
  fwrite(R.data(), 4, total, fout);
  if (!Xr.empty()) fwrite(Xr.data(), 4, total, fout);
  MultiresSparseGrid::destroy(msbg);
  return 0;
}

// multiplyLaplacianMatrixOpt (src/msbg3.cpp:1756-1812) at the first dense multigrid level
// (levelMg = nLevels: the dense grids MultiresSparseGrid::create adds below the sparse
// levels, src/msbg.cpp:847-1000), i.e. the masked 7-point operator
// ImultiplyLaplacianMatrixProcessSliceDenseLevel (src/msbg3.cpp:166-403).  Inputs after the
// header (job.nBlocksIn = the level's cells sx*sy*sz, x fastest): the cell flags (int32), then
// float32 X, B, DINV (what CH_DIAGONAL holds) and the face areas AX, AY, AZ (lower faces of
// each cell).  Every other cell of the dense arrays (the 2-cell border and the x padding)
// is zero, so X and the face areas read 0 outside the box, except the cell flags, which hold
// the flags grid's empty value CELL_EMPTY_VAL (void) there.  Output: Y = A X, then
// R = B - A X, over the box; with job.nIter > 0 also X after relax() with job.nIter iterations
// at that level (the dense levels' omega-Jacobi, src/msbg3.cpp:1917-2165, between X and a
// temporary channel that starts at zero).
int runDenseJob(const OracleJobHeader &job, const uint16_t *flagsIn, const float *arrays, FILE *fout) {
  OracleOutHeader out;
  memset(&out, 0, sizeof(out));
  memcpy(out.magic, ORACLE_OUT_MAGIC, 8);
  MultiresSparseGrid *msbg = MultiresSparseGrid::create(
      "TEST", job.sx, job.sy, job.sz, job.bsx, -1, 0, -1, 0, NULL, NULL, job.nLevels);
  if (!msbg) return 2;
  const int L = job.nLevels;
  if (msbg->getNumMgLevels() <= L) return 6;
  using MSBG::CH_PRESSURE;
  using MSBG::CH_DIVERGENCE;
  using MSBG::CH_CG_Q;
  using MSBG::CH_DIAGONAL;
  SparseGrid<MSBG::CellFlags> *sgF = msbg->getFlagsChannel(MSBG::CH_CELL_FLAGS, L, L);
  SparseGrid<PSFloat> *sgX = msbg->getPSFloatChannel(CH_PRESSURE, L, L),
                      *sgB = msbg->getPSFloatChannel(CH_DIVERGENCE, L, L),
                      *sgQ = msbg->getPSFloatChannel(CH_CG_Q, L, L),
                      *sgD = msbg->getPSFloatChannel(CH_DIAGONAL, L, L);
  SparseGrid<float> *sgA[3] = {msbg->getFaceAreaChannel(0, L, L), msbg->getFaceAreaChannel(1, L, L),
                               msbg->getFaceAreaChannel(2, L, L)};
  if (!sgF || !sgX || !sgB || !sgQ || !sgD || !sgA[0] || !sgA[1] || !sgA[2]) return 3;
  const int sx = sgF->sx(), sy = sgF->sy(), sz = sgF->sz();
  const int64_t n = (int64_t)sx * sy * sz;
  if (n != job.nBlocksIn) return 4;
  // the dense arrays: sxAct x (sy + 4) x (sz + 4) cells with a 2-cell border (src/sbg.cpp:131-189)
  auto fill = [&](auto *sg, const auto *src, double outside = 0.0) {
    using T = std::remove_pointer_t<decltype(sg->getDataPtrGen_(0, 0, 0, 1))>;
    T *p = sg->getDataPtrGen_(0, 0, 0, 1);
    const size_t all = (size_t)sg->sxAct() * (sy + 4) * (sz + 4);
    for (size_t i = 0; i < all; i++) p[i] = (T)outside;
    if (!src) return;
    for (int z = 0; z < sz; z++)
      for (int y = 0; y < sy; y++)
        for (int x = 0; x < sx; x++) p[sg->getGridIndex(x, y, z)] = src[((int64_t)z * sy + y) * sx + x];
  };
  const float *X = arrays, *B = X + n, *DI = B + n, *A = DI + n;
  fill(sgF, flagsIn, (double)MSBG::CELL_EMPTY_VAL);
  fill(sgX, X);
  fill(sgB, B);
  fill(sgD, DI);
  for (int k = 0; k < 3; k++) fill(sgA[k], A + (int64_t)k * n);
  auto dump = [&](std::vector<float> &dst) {
    const PSFloat *p = sgQ->getDataPtrGen_(0, 0, 0, 1);
    dst.resize((size_t)n);
    for (int z = 0; z < sz; z++)
      for (int y = 0; y < sy; y++)
        for (int x = 0; x < sx; x++) dst[((int64_t)z * sy + y) * sx + x] = p[sgQ->getGridIndex(x, y, z)];
  };
  const double t0 = nowSec();
  std::vector<float> Y, R;
  fill(sgQ, (const float *)nullptr);
  msbg->multiplyLaplacianMatrixOpt(0, L, CH_PRESSURE, CH_DIVERGENCE, 0.f, CH_CG_Q, NULL, NULL);
  dump(Y);
  fill(sgQ, (const float *)nullptr);
  msbg->multiplyLaplacianMatrixOpt(MSBG::OPT_CALC_RESIDUAL, L, CH_PRESSURE, CH_DIVERGENCE, 0.f, CH_CG_Q, NULL, NULL);
  dump(R);
  std::vector<float> Xr;
  if (job.nIter > 0) {
    fill(sgX, X);
    fill(sgQ, (const float *)nullptr);  // the temporary channel of the Jacobi iterations
    msbg->relax(0, job.constr01, L, CH_PRESSURE, CH_DIVERGENCE, CH_CG_Q, job.nIter, 0);
    const PSFloat *p = sgX->getDataPtrGen_(0, 0, 0, 1);
    Xr.resize((size_t)n);
    for (int z = 0; z < sz; z++)
      for (int y = 0; y < sy; y++)
        for (int x = 0; x < sx; x++) Xr[((int64_t)z * sy + y) * sx + x] = p[sgX->getGridIndex(x, y, z)];
  }
  out.tPdeSec = nowSec() - t0;
  out.nBlocks = sx;
  out.nActive = sy;
  out.nActParticles = sz;
  out.elemBytes = 4;
  out.nThreadsUsed = omp_get_max_threads();
  fwrite(&out, sizeof(out), 1, fout);
  fwrite(Y.data(), 4, (size_t)n, fout);
  fwrite(R.data(), 4, (size_t)n, fout);
  if (!Xr.empty()) fwrite(Xr.data(), 4, (size_t)n, fout);
  MultiresSparseGrid::destroy(msbg);
  return 0;
}

// downsampleFloatChannelNew (src/msbg4.cpp:1035-1379) to multigrid level 1 on a
// multi-level grid loaded like the halo job (channel CH_FLOAT_1, every resolution level
// with the job's block states and payloads; job.laplTyp = 0).  constr01 = 1 adds
// OPT_SIMPLE_AVERAGE.  For every block of the level map at level 0 (the blocks the
// function restricts from finer data) the output holds its level-1 block of the
// destination channel CH_FLOAT_2, (bsx/2)^3 floats.
int runDownsampleJob(const OracleJobHeader &job, const int32_t *levelsIn, const int32_t *state,
                     const std::vector<std::vector<uint8_t>> &pay, FILE *fout) {
  OracleOutHeader out;
  memset(&out, 0, sizeof(out));
  memcpy(out.magic, ORACLE_OUT_MAGIC, 8);
  const int chan = MSBG::CH_FLOAT_1, chDst = MSBG::CH_FLOAT_2;
  MultiresSparseGrid *msbg = MultiresSparseGrid::create(
      "TEST", job.sx, job.sy, job.sz, job.bsx, -1, 0, -1, 0, NULL, NULL, job.nLevels);
  if (!msbg) return 2;
  const int nBlocks = msbg->nBlocks();
  if ((int64_t)nBlocks != job.nBlocksIn) return 4;
  std::vector<int> levels(levelsIn, levelsIn + nBlocks);
  msbg->regularizeRefinementMap(levels.data());
  for (int b = 0; b < nBlocks; b++)
    if (levels[b] != levelsIn[b]) return 5;
  msbg->setRefinementMap(levels.data(), NULL, -1, NULL, false, false);
  for (int l = 0; l < job.nLevels; l++) {
    SparseGrid<float> *sg = MSBG::getChannel<float>(msbg, chan, l);
    if (!sg) return 3;
    sg->reset();
    sg->prepareDataAccess();
    sg->setEmptyValue(job.dt);
    sg->setFullValue(job.rParticle);
    const size_t nv = (size_t)sg->nVoxelsInBlock();
    const int32_t *st = state + (size_t)l * nBlocks;
    const float *src = reinterpret_cast<const float *>(pay[l].data());
    for (int b = 0; b < nBlocks; b++) {
      if (st[b] >= 0)
        memcpy(sg->getBlockDataPtr(b, 1, 0), src + (size_t)st[b] * nv, nv * sizeof(float));
      else if (st[b] == -1)
        sg->setEmptyBlock(b);
      else if (st[b] == -2)
        sg->setFullBlock(b);
    }
  }
  const unsigned opt = MSBG::OPT_ALL_CELLS | (job.constr01 ? MSBG::OPT_SIMPLE_AVERAGE : 0);
  const double t0 = nowSec();
  msbg->downsampleFloatChannelNew(1, chan, chDst, opt);
  out.tPdeSec = nowSec() - t0;
  std::vector<int32_t> bids;
  for (int b = 0; b < nBlocks; b++)
    if (levels[b] == 0) bids.push_back(b);
  SparseGrid<float> *dst = MSBG::getChannel<float>(msbg, chDst, 1, 1);
  if (!dst) return 3;
  const size_t nvc = (size_t)dst->nVoxelsInBlock();
  out.nBlocks = nBlocks;
  out.nActive = (int)bids.size();
  out.elemBytes = 4;
  out.nThreadsUsed = omp_get_max_threads();
  fwrite(&out, sizeof(out), 1, fout);
  fwrite(bids.data(), 4, bids.size(), fout);
  for (int32_t b : bids) {
    if (!dst->isValueBlock(b)) return 6;
    fwrite(dst->getBlockDataPtr(b, 0, 0), 4, nvc, fout);
  }
  MultiresSparseGrid::destroy(msbg);
  return 0;
}

// HaloBlockSet::fillHaloBlock3 (src/halo.cpp:536-738), the solver's halo, at multigrid
// level 0: the halo job's multi-level FP32 channel plus the cell flags (CH_CELL_FLAGS) of
// every resolution level and the domain's boundary types; every level-0 block that has a
// block at level 0 is filled (halo 1).  Flags of constant blocks: reserved = empty | full<<16.
int runHalo3Job(const OracleJobHeader &job, const int32_t *levelsIn, const int32_t *state,
                const std::vector<std::vector<uint8_t>> &pay, const int32_t *fstate,
                const std::vector<std::vector<uint16_t>> &fpay, const int32_t *dbc, FILE *fout) {
  OracleOutHeader out;
  memset(&out, 0, sizeof(out));
  memcpy(out.magic, ORACLE_OUT_MAGIC, 8);
  const int chan = MSBG::CH_FLOAT_1;
  MultiresSparseGrid *msbg = MultiresSparseGrid::create(
      "TEST", job.sx, job.sy, job.sz, job.bsx, -1, 0, -1, 0, NULL, NULL, job.nLevels);
  if (!msbg) return 2;
  const int nBlocks = msbg->nBlocks();
  if ((int64_t)nBlocks != job.nBlocksIn) return 4;
  if (msbg->setDomainBoundarySpec_(dbc[0], dbc[1], dbc[2], dbc[3], dbc[4], dbc[5])) return 8;
  std::vector<int> levels(levelsIn, levelsIn + nBlocks);
  msbg->regularizeRefinementMap(levels.data());
  for (int b = 0; b < nBlocks; b++)
    if (levels[b] != levelsIn[b]) return 5;
  msbg->setRefinementMap(levels.data(), NULL, 0, NULL, false, false);
  const uint16_t emptyFlags = (uint16_t)(job.reserved & 0xffff), fullFlags = (uint16_t)((uint32_t)job.reserved >> 16);
  for (int l = 0; l < job.nLevels; l++) {
    SparseGrid<float> *sg = MSBG::getChannel<float>(msbg, chan, l);
    SparseGrid<MSBG::CellFlags> *sf = msbg->getFlagsChannel(MSBG::CH_CELL_FLAGS, l, 0);
    if (!sg || !sf) return 3;
    sg->reset();
    sg->prepareDataAccess();
    sg->setEmptyValue(job.dt);
    sg->setFullValue(job.rParticle);
    sf->reset();
    sf->prepareDataAccess();
    sf->setEmptyValue(emptyFlags);
    sf->setFullValue(fullFlags);
    const size_t nv = (size_t)sg->nVoxelsInBlock();
    const int32_t *st = state + (size_t)l * nBlocks, *ft = fstate + (size_t)l * nBlocks;
    const float *src = reinterpret_cast<const float *>(pay[l].data());
    for (int b = 0; b < nBlocks; b++) {
      if (st[b] >= 0) memcpy(sg->getBlockDataPtr(b, 1, 0), src + (size_t)st[b] * nv, nv * sizeof(float));
      else if (st[b] == -1) sg->setEmptyBlock(b);
      else if (st[b] == -2) sg->setFullBlock(b);
      if (ft[b] >= 0) memcpy(sf->getBlockDataPtr(b, 1, 0), fpay[l].data() + (size_t)ft[b] * nv, nv * 2);
      else if (ft[b] == -1) sf->setEmptyBlock(b);
      else if (ft[b] == -2) sf->setFullBlock(b);
    }
  }
  const int bs = job.bsx, hs = bs + 2;
  std::vector<int32_t> bids;
  for (int b = 0; b < nBlocks; b++)
    if (levels[b] == 0 && state[b] != -3) bids.push_back(b);
  std::vector<float> halo(bids.size() * (size_t)hs * hs * hs);
  MSBG::HaloBlockSet hb(msbg, 1, 1);
  const int nbx = job.sx / bs, nby = job.sy / bs;
  const double t0 = nowSec();
  for (size_t k = 0; k < bids.size(); k++) {
    const int b = bids[k];
    float *p = hb.fillHaloBlock3(chan, b, b % nbx, (b / nbx) % nby, b / (nbx * nby), 0, 0);
    memcpy(halo.data() + k * (size_t)hs * hs * hs, p, sizeof(float) * hs * hs * hs);
  }
  out.tPdeSec = nowSec() - t0;
  out.nBlocks = nBlocks;
  out.nActive = (int)bids.size();
  out.elemBytes = 4;
  out.nThreadsUsed = 1;
  fwrite(&out, sizeof(out), 1, fout);
  fwrite(bids.data(), 4, bids.size(), fout);
  fwrite(halo.data(), 4, halo.size(), fout);
  MultiresSparseGrid::destroy(msbg);
  return 0;
}

// setRefinementMap's outputs beyond the per-block levels and flags (src/msbg.cpp:1428-2165):
// the block lists _blocksExisting and _blocksFineCoarsePerLevel[l] (each sorted: the
// release fills them from per-thread parts in no fixed order), and the fine-coarse distance
// channel CH_DIST_FINECOARSE of every level (value blocks with their uint16 data, then the
// full blocks).  Same grid and calls as the levels job.
int runLayoutJob(const OracleJobHeader &job, const int32_t *levelsIn, FILE *fout) {
  OracleOutHeader out;
  memset(&out, 0, sizeof(out));
  memcpy(out.magic, ORACLE_OUT_MAGIC, 8);
  MultiresSparseGrid *msbg = MultiresSparseGrid::create(
      "TEST", job.sx, job.sy, job.sz, job.bsx, -1, 0, -1, 0, NULL, NULL, job.nLevels);
  if (!msbg) return 2;
  const int nBlocks = msbg->nBlocks();
  if ((int64_t)nBlocks != job.nBlocksIn) return 4;
  std::vector<int> levels(levelsIn, levelsIn + nBlocks);
  msbg->regularizeRefinementMap(levels.data());
  msbg->setRefinementMap(levels.data(), NULL, 0, NULL, false, false);
  out.nBlocks = nBlocks;
  fwrite(&out, sizeof(out), 1, fout);
  auto dumpList = [&](std::vector<int> v) {
    std::sort(v.begin(), v.end());
    const int32_t n = (int32_t)v.size();
    fwrite(&n, 4, 1, fout);
    fwrite(v.data(), 4, v.size(), fout);
  };
  dumpList(msbg->_blocksExisting);
  for (int l = 0; l < job.nLevels; l++) dumpList(msbg->_blocksFineCoarsePerLevel[l]);
  for (int l = 0; l < job.nLevels; l++) {
    SparseGrid<uint16_t> *sg = msbg->getDistFineCoarseChannel(l);
    if (!sg) return 3;
    std::vector<int> val, full;
    for (int b = 0; b < nBlocks; b++) {
      if (sg->isValueBlock(b)) val.push_back(b);
      else if (sg->isFullBlock(b)) full.push_back(b);
    }
    dumpList(val);
    for (int b : val) fwrite(sg->getBlockDataPtr(b, 0, 0), 2, (size_t)sg->nVoxelsInBlock(), fout);
    dumpList(full);
    const uint16_t fv = sg->getFullValue();
    fwrite(&fv, 2, 1, fout);
  }
  MultiresSparseGrid::destroy(msbg);
  return 0;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: %s job.bin out.bin\n", argv[0]);
    return 1;
  }
  FILE *fin = fopen(argv[1], "rb");
  if (!fin) return 1;
  OracleJobHeader job;
  if (fread(&job, sizeof(job), 1, fin) != 1 || memcmp(job.magic, ORACLE_JOB_MAGIC, 8) != 0) {
    fprintf(stderr, "bad job file\n");
    return 1;
  }
  std::vector<float> pts((size_t)job.nPoints * 3);
  std::vector<int32_t> lv((size_t)job.nBlocksIn);
  if (job.nPoints && fread(pts.data(), 4, pts.size(), fin) != pts.size()) return 1;
  if (job.nBlocksIn && fread(lv.data(), 4, lv.size(), fin) != lv.size()) return 1;
  std::vector<uint8_t> payload;
  std::vector<int32_t> state;
  std::vector<std::vector<uint8_t>> levelPay;
  std::vector<float> solverArrays;
  if (job.jobType == ORACLE_JOB_SOLVER) {
    solverArrays.resize((size_t)8 * job.nBlocksIn * job.bsx * job.bsx * job.bsx);
    if (!solverArrays.empty() && fread(solverArrays.data(), 4, solverArrays.size(), fin) != solverArrays.size())
      return 1;
  }
  if (job.jobType == ORACLE_JOB_MULTIRES) {
    size_t total = 0;
    std::vector<size_t> perLevel(job.nLevels > 0 ? job.nLevels : 0, 0);
    for (int64_t b = 0; b < job.nBlocksIn; b++)
      if (lv[b] >= 0 && lv[b] < job.nLevels) perLevel[lv[b]]++;
    for (int l = 0; l < job.nLevels; l++) {
      const size_t bs = (size_t)(job.bsx >> l);
      total += perLevel[l] * bs * bs * bs;
    }
    solverArrays.resize(3 * total);
    if (!solverArrays.empty() && fread(solverArrays.data(), 4, solverArrays.size(), fin) != solverArrays.size())
      return 1;
  }
  std::vector<uint16_t> denseFlags;
  if (job.jobType == ORACLE_JOB_DENSE) {  // the int32 array read above holds the cell flags
    denseFlags.resize((size_t)job.nBlocksIn);
    for (int64_t i = 0; i < job.nBlocksIn; i++) denseFlags[(size_t)i] = (uint16_t)lv[(size_t)i];
    solverArrays.resize((size_t)6 * job.nBlocksIn);
    if (fread(solverArrays.data(), 4, solverArrays.size(), fin) != solverArrays.size()) return 1;
  }
  std::vector<int32_t> fstate, dbc(6, 0);
  std::vector<std::vector<uint16_t>> flagPay;
  if (job.jobType == ORACLE_JOB_HALO || job.jobType == ORACLE_JOB_DOWNSAMPLE || job.jobType == ORACLE_JOB_HALO3) {
    const size_t elem = job.chanType == ORACLE_CHAN_U16 ? 2 : 4;
    state.resize((size_t)job.nLevels * job.nBlocksIn);
    if (fread(state.data(), 4, state.size(), fin) != state.size()) return 1;
    levelPay.resize(job.nLevels);
    for (int l = 0; l < job.nLevels; l++) {
      int32_t mx = -1;
      for (int64_t b = 0; b < job.nBlocksIn; b++) mx = std::max(mx, state[(size_t)l * job.nBlocksIn + b]);
      const size_t bs = (size_t)(job.bsx >> l);
      levelPay[l].resize((size_t)(mx + 1) * bs * bs * bs * elem);
      if (!levelPay[l].empty() && fread(levelPay[l].data(), 1, levelPay[l].size(), fin) != levelPay[l].size())
        return 1;
    }
    if (job.jobType == ORACLE_JOB_HALO3) {  // then the flags' states and payloads, and the domain's boundaries
      fstate.resize((size_t)job.nLevels * job.nBlocksIn);
      if (fread(fstate.data(), 4, fstate.size(), fin) != fstate.size()) return 1;
      flagPay.resize(job.nLevels);
      for (int l = 0; l < job.nLevels; l++) {
        int32_t mx = -1;
        for (int64_t b = 0; b < job.nBlocksIn; b++) mx = std::max(mx, fstate[(size_t)l * job.nBlocksIn + b]);
        const size_t bs = (size_t)(job.bsx >> l);
        flagPay[l].resize((size_t)(mx + 1) * bs * bs * bs);
        if (!flagPay[l].empty() && fread(flagPay[l].data(), 2, flagPay[l].size(), fin) != flagPay[l].size())
          return 1;
      }
      if (fread(dbc.data(), 4, 6, fin) != 6) return 1;
    }
  }
  if (job.jobType == ORACLE_JOB_INTERP || job.jobType == ORACLE_JOB_RENDER) {
    const size_t elem = job.chanType == ORACLE_CHAN_U16 ? 2 : 4;
    payload.resize((size_t)job.nBlocksIn * job.bsx * job.bsx * job.bsx * elem);
    if (!payload.empty() && fread(payload.data(), 1, payload.size(), fin) != payload.size())
      return 1;
  }
  fclose(fin);

  if (job.nThreads > 0) {
    omp_set_num_threads(job.nThreads);
  }
  ThrInit();
  nMaxThreads = omp_get_max_threads();

  FILE *fout = fopen(argv[2], "wb");
  if (!fout) return 1;
  int rc;
  if (job.jobType == ORACLE_JOB_LEVELS)
    rc = runLevelsJob(job, lv.data(), fout);
  else if (job.jobType == ORACLE_JOB_LAYOUT)
    rc = runLayoutJob(job, lv.data(), fout);
  else if (job.jobType == ORACLE_JOB_SOLVER)
    rc = runSolverJob(job, lv.data(), solverArrays.data(), fout);
  else if (job.jobType == ORACLE_JOB_MULTIRES)
    rc = runMultiresJob(job, lv.data(), solverArrays.data(), fout);
  else if (job.jobType == ORACLE_JOB_DENSE)
    rc = runDenseJob(job, denseFlags.data(), solverArrays.data(), fout);
  else if (job.jobType == ORACLE_JOB_HALO3)
    rc = job.chanType == ORACLE_CHAN_F32
             ? runHalo3Job(job, lv.data(), state.data(), levelPay, fstate.data(), flagPay, dbc.data(), fout)
             : 7;
  else if (job.jobType == ORACLE_JOB_DOWNSAMPLE)
    rc = job.chanType == ORACLE_CHAN_F32 ? runDownsampleJob(job, lv.data(), state.data(), levelPay, fout) : 7;
  else if (job.jobType == ORACLE_JOB_MORTON)
    rc = runMortonJob(job, lv.data(), fout);
  else if (job.jobType == ORACLE_JOB_RENDER)
    rc = job.chanType == ORACLE_CHAN_U16 && job.nPoints == 5
             ? runRenderJob(job, pts.data(), lv.data(), reinterpret_cast<const uint16_t *>(payload.data()), fout)
             : 7;
  else if (job.jobType == ORACLE_JOB_HALO && job.chanType == ORACLE_CHAN_U16)
    rc = runHaloJob<uint16_t>(job, lv.data(), state.data(), levelPay, fout);
  else if (job.jobType == ORACLE_JOB_HALO)
    rc = runHaloJob<float>(job, lv.data(), state.data(), levelPay, fout);
  else if (job.jobType == ORACLE_JOB_INTERP && job.chanType == ORACLE_CHAN_U16)
    rc = runInterpJob<uint16_t>(job, pts.data(), lv.data(),
                                reinterpret_cast<const uint16_t *>(payload.data()), fout);
  else if (job.jobType == ORACLE_JOB_INTERP)
    rc = runInterpJob<float>(job, pts.data(), lv.data(),
                             reinterpret_cast<const float *>(payload.data()), fout);
  else if (job.chanType == ORACLE_CHAN_U16)
    rc = runSurfaceJob<uint16_t>(job, pts.data(), job.nBlocksIn ? lv.data() : nullptr, fout);
  else
    rc = runSurfaceJob<float>(job, pts.data(), job.nBlocksIn ? lv.data() : nullptr, fout);
  fclose(fout);
  return rc;
}
