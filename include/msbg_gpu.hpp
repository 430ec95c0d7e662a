/*
 * msbg_gpu.hpp -- header-only C++ facade over the msbg_gpu C ABI (msbg_gpu.h).
 *
 * msbg_gpu::MultiresSparseGrid keeps the method names and argument order of the
 * reference's MSBG::MultiresSparseGrid (src/msbg.h:828-3797) for the hot path, so code
 * written against the reference switches by changing the namespace:
 *   create / destroy                      src/msbg.h:834-852
 *   regularizeRefinementMap               src/msbg.h:897-901
 *   setRefinementMap                      src/msbg.h:903-908
 *   applyChannelPdeFast<T>                src/msbg.h:2150-2172
 *   downsampleFloatChannelNew             src/msbg.h:2198-2201
 *   multiplyLaplacianMatrixOpt            src/msbg.h:3167-3176
 *   relax                                 src/msbg.h:3269-3277
 *   dotProdChannel                        src/msbg.h:3331-3341
 *   AXPBYChannel / AXPBYChannelCombined   src/msbg.h:3356-3368
 *   sortBlockListMorton                   src/msbg.h:3423
 * Block lists are the reference's host `std::vector<int> *` (NULL = all value blocks);
 * the facade copies them to the device for the call.  Channel data lives on the GPU:
 * the reference's per-block pointers become the slab accessors below.  Failures throw
 * msbg_gpu::Error (the reference asserts and exits), except create, which returns NULL
 * as the reference does.  Needs only the C ABI: link -lmsbg_gpu.
 */
#ifndef MSBG_GPU_HPP
#define MSBG_GPU_HPP

#include <stdexcept>
#include <string>
#include <vector>

#include "msbg_gpu.h"

namespace msbg_gpu {

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string &what) : std::runtime_error(what), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

class MultiresSparseGrid {
 public:
  // storage: the type of the density channel 0 (the reference picks it per channel id)
  static MultiresSparseGrid *create(const char *name, int sx0, int sy0, int sz0, int blockSize0 = -1,
                                    int dTransRes = -1, int maxSizeMB = 0, int initialSizeMB = -1,
                                    unsigned options = 0, const void *miscConf = nullptr,
                                    const void *psConf = nullptr, int nLevels = -1, int storage = MSBG_GPU_F32) {
    (void)name; (void)dTransRes; (void)maxSizeMB; (void)initialSizeMB; (void)options; (void)miscConf; (void)psConf;
    if (blockSize0 < 0) blockSize0 = (sx0 < sy0 ? (sx0 < sz0 ? sx0 : sz0) : (sy0 < sz0 ? sy0 : sz0)) >= 400 ? 32 : 16;
    if (nLevels < 0) nLevels = 3;
    msbg_gpu_ctx *c = nullptr;
    if (msbg_gpu_create(&c, sx0, sy0, sz0, blockSize0, nLevels, storage, 0) != MSBG_GPU_OK) return nullptr;
    return new MultiresSparseGrid(c);
  }
  static void destroy(MultiresSparseGrid *&g) {
    delete g;
    g = nullptr;
  }
  ~MultiresSparseGrid() { msbg_gpu_destroy(ctx_); }
  MultiresSparseGrid(const MultiresSparseGrid &) = delete;
  MultiresSparseGrid &operator=(const MultiresSparseGrid &) = delete;

  msbg_gpu_ctx *ctx() const { return ctx_; }
  msbg_gpu_info info() const {
    msbg_gpu_info i;
    check(msbg_gpu_get_info(ctx_, &i));
    return i;
  }
  int nBlocks() const { return (int)info().nBlocks; }

  // regularizeRefinementMap(blockmapIn, blockmapOut, blockFlags, rbzWidthBlk): the map is
  // regularised on the device and written to blockmapOut (blockmapIn when NULL)
  void regularizeRefinementMap(int *blockmapIn, int *blockmapOut = nullptr, unsigned *blockFlags = nullptr,
                               int rbzWidthBlk = 0) {
    (void)blockFlags; (void)rbzWidthBlk;
    check(msbg_gpu_set_levels(ctx_, blockmapIn));
    check(msbg_gpu_regularize_refinement_map(ctx_));
    levelsOut(blockmapOut ? blockmapOut : blockmapIn);
  }
  // setRefinementMap(blockLevels, blockFlags, levelMgMax, msbgObstacles, doInitCellFlags,
  // doResetChannels): the layout (flags, value blocks in ascending id, colour lists); the
  // channels' value blocks are filled with valueBlockFill (the demo's allocation loop
  // fills them with 1, src/msbg_demo.cpp:455-511)
  void setRefinementMap(int *blockLevels, unsigned *blockFlags = nullptr, int levelMgMax = -1,
                        MultiresSparseGrid *msbgObstacles = nullptr, bool doInitCellFlags = true,
                        bool doResetChannels = true, double valueBlockFill = 0.0) {
    (void)blockFlags; (void)levelMgMax; (void)doInitCellFlags; (void)doResetChannels;
    if (msbgObstacles) throw Error(MSBG_GPU_ERR_UNSUPPORTED, "obstacle grids are not on this path");
    check(msbg_gpu_set_levels(ctx_, blockLevels));
    check(msbg_gpu_set_refinement_map(ctx_, valueBlockFill));
  }
  std::vector<int> activeBlocks() const {
    const int64_t n = info().nActive;
    std::vector<int> out((size_t)n);
    int64_t got = 0;
    check(msbg_gpu_get_active_blocks(ctx_, out.data(), n, &got));
    out.resize((size_t)got);
    return out;
  }

  // channels: creation and the value blocks' data, [nActive][bs^3] in ascending block id
  void createChannel(int chan, int storage) { check(msbg_gpu_channel_create(ctx_, chan, storage)); }
  void uploadChannel(int chan, const void *hData) { check(msbg_gpu_upload_payload(ctx_, chan, hData)); }
  void downloadChannel(int chan, void *hData) { check(msbg_gpu_download_payload(ctx_, chan, hData)); }

  // the demo's particle loops (src/msbg_demo.cpp:339-680), points on the host.
  // markParticles returns the level map of the marking (src/msbg_demo.cpp:413-425): 0 for
  // every block in a particle's rScan box, the coarsest level elsewhere
  std::vector<int> markParticles(const float *hPts, int64_t n, float rScan) {
    DeviceVec<float> d(this, hPts, (size_t)n * 3);
    check(msbg_gpu_mark_points(ctx_, d.p, n, rScan));
    check(msbg_gpu_levels_from_marks(ctx_));
    std::vector<int> levels((size_t)info().nBlocks);
    levelsOut(levels.data());
    return levels;
  }
  void splatParticles(const float *hPts, int64_t n, float rParticle, float nbDist) {
    DeviceVec<float> d(this, hPts, (size_t)n * 3);
    check(msbg_gpu_splat(ctx_, d.p, n, rParticle, nbDist));
    check(msbg_gpu_splat_finalize(ctx_, rParticle, nbDist));
    check(msbg_gpu_synchronize(ctx_));
  }

  template <typename Data_T>
  void applyChannelPdeFast(int chPhi, int chTmp, int chTmp2, std::vector<int> *blockList, int laplTyp,
                           int doConstrZeroOne, float densThr, float densThrTol1, float densThrTol2, int numIter,
                           float gridSpacing = 1, float timeStep = 0.025, float velMagThr = 0,
                           MultiresSparseGrid *msbgVel = nullptr, float lambda = 0, float lambdaSDF = 0,
                           float taubin = 0, float redist = 0, float anisDiffAlpha = 0, int veldep_on = 0,
                           float *veldep_fit = nullptr, int visOpt = 0, int variant = MSBG_GPU_SWEEP_EXACT) {
    List l(this, blockList);
    check(msbg_gpu_apply_channel_pde_fast(ctx_, chPhi, chTmp, chTmp2, l.p, l.n, laplTyp, doConstrZeroOne, densThr,
                                          densThrTol1, densThrTol2, numIter, gridSpacing, timeStep, velMagThr,
                                          msbgVel, lambda, lambdaSDF, taubin, redist, anisDiffAlpha, veldep_on,
                                          veldep_fit, visOpt, variant));
    check(msbg_gpu_synchronize(ctx_));
  }

  // downsampleFloatChannelNew(levelMg, chSrc, ...): levelMg 1 of the value blocks into
  // hDst, nActive * (bs/2)^3 floats (the reference writes them to channel chDst)
  void downsampleFloatChannelNew(int levelMg, int chSrc, float *hDst, unsigned options) {
    if (levelMg != 1) throw Error(MSBG_GPU_ERR_UNSUPPORTED, "downsampleFloatChannelNew: levelMg 1 only");
    const msbg_gpu_info i = info();
    const size_t n = (size_t)i.nActive * (i.bsx / 2) * (i.bsx / 2) * (i.bsx / 2);
    DeviceVec<float> d(this, nullptr, n);
    check(msbg_gpu_downsample_channel(ctx_, chSrc, d.p, (options & (1u << 27)) ? 1 : 0));  // OPT_SIMPLE_AVERAGE
    check(msbg_gpu_copy_d2h(ctx_, hDst, d.p, n * sizeof(float)));
    check(msbg_gpu_synchronize(ctx_));
  }

  // Poisson coefficients: lower-face coefficients of every cell and the diagonal (FP32
  // channels); the reference keeps them in its face-area channels and 1/d in CH_DIAGONAL
  void setPoissonCoefficients(int chCx, int chCy, int chCz, int chDiag) {
    check(msbg_gpu_poisson_set_coefficients(ctx_, chCx, chCy, chCz, chDiag));
  }
  void multiplyLaplacianMatrixOpt(unsigned options, int levelMg, int chanX, int chanB, float kap, int chanDstY,
                                  long double *pDotprod, std::vector<int> *blockList) {
    List l(this, blockList);
    double dot = 0.0;
    check(msbg_gpu_multiply_laplacian(ctx_, options, levelMg, chanX, chanB, kap, chanDstY, pDotprod ? &dot : nullptr,
                                      l.p, l.n));
    check(msbg_gpu_synchronize(ctx_));
    if (pDotprod) *pDotprod = dot;
  }
  // relax(...) relaxes the reference's member list _blocksRelax[levelMg]; here that list
  // is set with setRelaxBlockList (empty: all value blocks)
  void setRelaxBlockList(const std::vector<int> &blocks) { relaxBlocks_ = blocks; }
  void relax(int boundaryZoneOnly, int reverseOrder, int levelMg, int chanX, int chanB, int chanTmp, int nIter,
             unsigned options = 0) {
    List l(this, relaxBlocks_.empty() ? nullptr : &relaxBlocks_);
    check(msbg_gpu_relax(ctx_, boundaryZoneOnly, reverseOrder, levelMg, chanX, chanB, chanTmp, nIter, options, l.p,
                         l.n));
    check(msbg_gpu_synchronize(ctx_));
  }
  long double dotProdChannel(int ch1, int ch2, int levelMg = 0, std::vector<int> *blockList = nullptr,
                             int *pErrCode = nullptr) {
    List l(this, blockList);
    double out = 0.0;
    const int rc = msbg_gpu_dot(ctx_, ch1, ch2, levelMg, l.p, l.n, &out);
    if (pErrCode) *pErrCode = rc;
    if (rc != MSBG_GPU_OK && !(rc == MSBG_GPU_ERR_NONFINITE && pErrCode)) check(rc);
    return out;
  }
  void AXPBYChannel(double a, int iChanX, double b, int iChanDstY, int levelMax = 9999, int levelMg = 0,
                    std::vector<int> *blockList = nullptr) {
    List l(this, blockList);
    check(msbg_gpu_axpby(ctx_, a, iChanX, b, iChanDstY, levelMax, levelMg, l.p, l.n));
    check(msbg_gpu_synchronize(ctx_));
  }
  void AXPBYChannelCombined(double a, double b, int iChanQ, int iChanX, int iChanP,
                            std::vector<int> *blockList = nullptr) {
    List l(this, blockList);
    check(msbg_gpu_axpby_combined(ctx_, a, b, iChanQ, iChanX, iChanP, l.p, l.n));
    check(msbg_gpu_synchronize(ctx_));
  }
  void sortBlockListMorton(std::vector<int> &blockList) {
    if (blockList.empty()) return;
    DeviceVec<int32_t> d(this, blockList.data(), blockList.size());
    check(msbg_gpu_sort_block_list_morton(ctx_, d.p, (int64_t)blockList.size()));
    check(msbg_gpu_copy_d2h(ctx_, blockList.data(), d.p, blockList.size() * sizeof(int32_t)));
    check(msbg_gpu_synchronize(ctx_));
  }

  void check(int rc) const {
    if (rc != MSBG_GPU_OK) throw Error(rc, std::string("msbg_gpu: ") + msbg_gpu_last_error(ctx_));
  }

 private:
  explicit MultiresSparseGrid(msbg_gpu_ctx *c) : ctx_(c) {}

  // a device copy of host data for the duration of one call
  template <typename T>
  struct DeviceVec {
    T *p = nullptr;
    DeviceVec(const MultiresSparseGrid *g, const T *h, size_t n) {
      if (msbg_gpu_device_alloc((void **)&p, (n ? n : 1) * sizeof(T)) != MSBG_GPU_OK)
        throw Error(MSBG_GPU_ERR_NOMEM, "msbg_gpu: device allocation failed");
      if (h && n) g->check(msbg_gpu_copy_h2d(g->ctx_, p, h, n * sizeof(T)));
    }
    ~DeviceVec() {
      if (p) msbg_gpu_device_free(p);
    }
  };
  struct List {
    const int32_t *p = nullptr;
    int64_t n = 0;
    DeviceVec<int32_t> *d = nullptr;
    List(const MultiresSparseGrid *g, const std::vector<int> *v) {
      if (!v) return;
      d = new DeviceVec<int32_t>(g, v->data(), v->size());
      p = d->p;
      n = (int64_t)v->size();
    }
    // a call with a list reads it before it returns (it converts the list and
    // synchronizes), so the copy can go with the call
    ~List() { delete d; }
  };
  void levelsOut(int *out) const {
    const int64_t n = info().nBlocks;
    std::vector<int8_t> l8((size_t)n);
    check(msbg_gpu_get_levels(ctx_, l8.data()));
    for (int64_t i = 0; i < n; i++) out[i] = l8[(size_t)i];
  }

  msbg_gpu_ctx *ctx_;
  std::vector<int> relaxBlocks_;
};

}  // namespace msbg_gpu

#endif  // MSBG_GPU_HPP
