// Checkpoint files: the grid geometry, level map and channel payloads of a context,
// written and read back through a pinned staging buffer.  The reference has no on-disk
// format for its grids (VDB writers declared only, src/sbg.h:599-605); the layout
// (slots, active list, flags, colour lists) is not stored but rebuilt from the level
// map on load, as setRefinementMap rebuilds it in the reference.
#include <stdio.h>
#include <string.h>

#include <vector>

#include "internal.cuh"

namespace msbg {

namespace {

constexpr char kMagic[8] = {'M', 'S', 'B', 'G', 'C', 'K', 'P', '1'};
constexpr uint32_t kVersion = 1;
constexpr size_t kStage = (size_t)64 << 20;  // pinned staging per transfer

struct CkptHeader {
  char magic[8];
  uint32_t version, headerBytes;
  int32_t sx, sy, sz, bsx, nLevels, nChans;
  int64_t nBlocks, nActive;
  uint64_t levelsHash;
};
static_assert(sizeof(CkptHeader) == 64, "checkpoint header layout");

struct ChanRecord {
  int32_t chan, storage;
  int64_t bytes;
  uint64_t hash;
};
static_assert(sizeof(ChanRecord) == 24, "checkpoint channel record layout");

// FNV-1a, 64 bit
uint64_t fnv1a(uint64_t h, const void *p, size_t n) {
  const uint8_t *b = (const uint8_t *)p;
  for (size_t i = 0; i < n; i++) {
    h ^= b[i];
    h *= 0x100000001b3ull;
  }
  return h;
}
constexpr uint64_t kFnvBasis = 0xcbf29ce484222325ull;

struct File {
  FILE *f = nullptr;
  ~File() { if (f) fclose(f); }
};
struct Pinned {
  void *p = nullptr;
  ~Pinned() { if (p) cudaFreeHost(p); }
};

}  // namespace

}  // namespace msbg

using namespace msbg;

extern "C" int msbg_gpu_save(msbg_gpu_ctx *ctx, const char *path, const int *chans, int nChans) {
  if (!ctx) return MSBG_GPU_ERR_ARG;
  if (!path || nChans < 0 || (nChans > 0 && !chans)) return fail(ctx, MSBG_GPU_ERR_ARG, "save: bad arguments");
  if (!ctx->layoutValid) return fail(ctx, MSBG_GPU_ERR_STATE, "save: no block layout");
  for (int i = 0; i < nChans; i++) {
    if (chans[i] < 0 || chans[i] >= kMaxChannels || !ctx->ch[chans[i]].exists || !ctx->ch[chans[i]].d)
      return fail(ctx, MSBG_GPU_ERR_ARG, "save: channel %d does not exist", chans[i]);
    for (int j = 0; j < i; j++)
      if (chans[j] == chans[i]) return fail(ctx, MSBG_GPU_ERR_ARG, "save: channel %d listed twice", chans[i]);
  }
  std::vector<int8_t> levels((size_t)ctx->nBlocks);
  int rc = msbg_gpu_get_levels(ctx, levels.data());
  if (rc) return rc;
  CkptHeader h;
  memset(&h, 0, sizeof(h));
  memcpy(h.magic, kMagic, 8);
  h.version = kVersion;
  h.headerBytes = sizeof(h);
  h.sx = ctx->sx; h.sy = ctx->sy; h.sz = ctx->sz; h.bsx = ctx->bsx; h.nLevels = ctx->nLevels;
  h.nChans = nChans;
  h.nBlocks = ctx->nBlocks;
  h.nActive = ctx->nActive;
  h.levelsHash = fnv1a(kFnvBasis, levels.data(), levels.size());
  File f;
  f.f = fopen(path, "wb");
  if (!f.f) return fail(ctx, MSBG_GPU_ERR_IO, "save: cannot open %s", path);
  if (fwrite(&h, sizeof(h), 1, f.f) != 1 || fwrite(levels.data(), 1, levels.size(), f.f) != levels.size())
    return fail(ctx, MSBG_GPU_ERR_IO, "save: write failed");
  Pinned st;
  MSBG_CUDA(ctx, cudaMallocHost(&st.p, kStage));
  for (int i = 0; i < nChans; i++) {
    const Channel &c = ctx->ch[chans[i]];
    ChanRecord r;
    r.chan = chans[i];
    r.storage = c.storage;
    r.bytes = (int64_t)ctx->nActive * ctx->voxPerBlock * (int64_t)storageBytes(c.storage);
    r.hash = kFnvBasis;
    const long recPos = ftell(f.f);
    if (fwrite(&r, sizeof(r), 1, f.f) != 1) return fail(ctx, MSBG_GPU_ERR_IO, "save: write failed");
    for (int64_t off = 0; off < r.bytes; off += (int64_t)kStage) {
      const size_t n = (size_t)((r.bytes - off) < (int64_t)kStage ? (r.bytes - off) : (int64_t)kStage);
      MSBG_CUDA(ctx, cudaMemcpyAsync(st.p, (const char *)c.d + off, n, cudaMemcpyDeviceToHost, ctx->stream));
      MSBG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      r.hash = fnv1a(r.hash, st.p, n);
      if (fwrite(st.p, 1, n, f.f) != n) return fail(ctx, MSBG_GPU_ERR_IO, "save: write failed");
    }
    // the record's checksum, now known
    const long end = ftell(f.f);
    if (fseek(f.f, recPos, SEEK_SET) || fwrite(&r, sizeof(r), 1, f.f) != 1 || fseek(f.f, end, SEEK_SET))
      return fail(ctx, MSBG_GPU_ERR_IO, "save: write failed");
  }
  if (fflush(f.f)) return fail(ctx, MSBG_GPU_ERR_IO, "save: write failed");
  return MSBG_GPU_OK;
}

extern "C" int msbg_gpu_load(msbg_gpu_ctx **out, const char *path) {
  if (!out || !path) return MSBG_GPU_ERR_ARG;
  *out = nullptr;
  File f;
  f.f = fopen(path, "rb");
  if (!f.f) return MSBG_GPU_ERR_IO;
  CkptHeader h;
  if (fread(&h, sizeof(h), 1, f.f) != 1 || memcmp(h.magic, kMagic, 8) || h.version != kVersion ||
      h.headerBytes != sizeof(h) || h.nChans < 0 || h.nChans > kMaxChannels || h.nBlocks <= 0 ||
      h.nActive < 0 || h.nActive > h.nBlocks)
    return MSBG_GPU_ERR_IO;
  msbg_gpu_ctx *ctx = nullptr;
  if (msbg_gpu_create(&ctx, h.sx, h.sy, h.sz, h.bsx, h.nLevels, MSBG_GPU_F32, 0) != MSBG_GPU_OK)
    return MSBG_GPU_ERR_IO;
  int rc = MSBG_GPU_OK;
  do {
    if (ctx->nBlocks != h.nBlocks) { rc = MSBG_GPU_ERR_IO; break; }
    std::vector<int8_t> lv8((size_t)h.nBlocks);
    if (fread(lv8.data(), 1, lv8.size(), f.f) != lv8.size() ||
        fnv1a(kFnvBasis, lv8.data(), lv8.size()) != h.levelsHash) {
      rc = MSBG_GPU_ERR_IO;
      break;
    }
    std::vector<int32_t> lv(lv8.begin(), lv8.end());
    if ((rc = msbg_gpu_set_levels(ctx, lv.data()))) break;
    // channels first, so that the layout sizes their slabs
    std::vector<ChanRecord> recs;
    const long dataPos = ftell(f.f);
    bool seen[kMaxChannels] = {};
    for (int i = 0; i < h.nChans && !rc; i++) {
      ChanRecord r;
      // a channel may appear once: a second record would size the slab by its own
      // storage type while the first record's bytes were also copied into it
      if (fread(&r, sizeof(r), 1, f.f) != 1 || r.chan < 0 || r.chan >= kMaxChannels || seen[r.chan] ||
          r.storage < 0 || r.storage > 3 ||
          r.bytes != h.nActive * ctx->voxPerBlock * (int64_t)storageBytes(r.storage) ||
          fseek(f.f, (long)r.bytes, SEEK_CUR)) {
        rc = MSBG_GPU_ERR_IO;
        break;
      }
      seen[r.chan] = true;
      recs.push_back(r);
      rc = msbg_gpu_channel_create(ctx, r.chan, r.storage);
    }
    if (rc) break;
    if ((rc = msbg_gpu_set_refinement_map(ctx, 0.0))) break;
    if (ctx->nActive != h.nActive) { rc = MSBG_GPU_ERR_IO; break; }
    if (fseek(f.f, dataPos, SEEK_SET)) { rc = MSBG_GPU_ERR_IO; break; }
    Pinned st;
    if (cudaMallocHost(&st.p, kStage) != cudaSuccess) { rc = MSBG_GPU_ERR_NOMEM; break; }
    for (const ChanRecord &r0 : recs) {
      ChanRecord r;
      if (fread(&r, sizeof(r), 1, f.f) != 1 || r.chan != r0.chan) { rc = MSBG_GPU_ERR_IO; break; }
      const Channel &dc = ctx->ch[r.chan];
      // the slab must hold exactly this record's bytes in the channel's current type
      if (!dc.exists || !dc.d || dc.storage != r.storage || dc.capBlocks < (size_t)h.nActive ||
          r.bytes != (int64_t)h.nActive * ctx->voxPerBlock * (int64_t)storageBytes(dc.storage)) {
        rc = MSBG_GPU_ERR_IO;
        break;
      }
      uint64_t hash = kFnvBasis;
      char *dst = (char *)dc.d;
      for (int64_t off = 0; off < r.bytes && !rc; off += (int64_t)kStage) {
        const size_t n = (size_t)((r.bytes - off) < (int64_t)kStage ? (r.bytes - off) : (int64_t)kStage);
        if (fread(st.p, 1, n, f.f) != n) { rc = MSBG_GPU_ERR_IO; break; }
        hash = fnv1a(hash, st.p, n);
        if (cudaMemcpyAsync(dst + off, st.p, n, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess ||
            cudaStreamSynchronize(ctx->stream) != cudaSuccess)
          rc = MSBG_GPU_ERR_CUDA;
      }
      if (!rc && hash != r.hash) rc = MSBG_GPU_ERR_IO;
      if (rc) break;
    }
  } while (0);
  if (rc) {
    msbg_gpu_destroy(ctx);
    return rc;
  }
  *out = ctx;
  return MSBG_GPU_OK;
}
