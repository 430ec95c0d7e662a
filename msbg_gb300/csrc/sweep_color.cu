// In-place colored sweeps (8-color / red-black) of applyChannelPdeFast, the
// streaming kernel.  Same schedule and arithmetic as sweep.cu (which keeps the
// generic gather kernel for the ping-pong schedule and FP64); this kernel is the
// one the in-place schedules use for FP32 / FP16 / uint16 storage.
//
// Per CTA one block.  Warp 0 stages the whole block and every halo piece it
// needs into shared memory with TMA bulk copies (cp.async.bulk) in chunks of 8
// planes, each chunk completing on its own mbarrier, so a CTA has the whole
// block (~77 KB for FP16 32^3) in flight at once and starts computing when the
// first chunk has landed.  Each thread owns a 4-voxel x-strip of every plane and
// marches through the block in z with a register window of three planes (rows
// y-1..y+1, columns x-1..x+4 of planes z-1, z, z+1; the three windows rotate
// roles, so no register moves).  Each warp owns 4 rows (32^3) of every plane and
// converts the rows it needs (its own and one on each side) from the staged raw
// data into its private 2-slot ring of FP32 halo'd rows, so after the staging the
// warps never wait for each other: only __syncwarp orders a warp's ring.  Results go straight to global
// memory; the block is in shared memory before its first store, so the update
// is in place.
//
// Halo traffic.  The block payload is x-fastest (src/sbg.h:1816-1820), so the
// y- and z-neighbour rows/planes are contiguous but an x-neighbour column is one
// element per row.  Each channel therefore keeps, per value block, a cache of
// its two x-faces ([z][y]) and four z-parallel corner columns, written by the
// kernel whenever it updates a block and built once per applyChannelPdeFast
// call.  Same-color blocks are never 26-neighbours, so in a pass no block reads
// a cache entry that the pass writes.  Every piece is a multiple of 16 bytes at
// a 16-byte aligned address, as cp.async.bulk requires.
#include <string.h>

#include <type_traits>

#include "internal.cuh"
#include "sweep_common.cuh"

namespace msbg {

template <typename T> struct Vec4T;
template <> struct Vec4T<float> { using V = float4; };
template <> struct Vec4T<__half> { using V = uint2; };
template <> struct Vec4T<uint16_t> { using V = uint2; };

template <typename T>
__device__ __forceinline__ void unpack4(const typename Vec4T<T>::V &v, float o[4]) {
  if constexpr (sizeof(T) == 4) {
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
  } else {
    const T *e = reinterpret_cast<const T *>(&v);
#pragma unroll
    for (int k = 0; k < 4; k++) o[k] = Store<T>::load(e + k);
  }
}

template <typename T>
__device__ __forceinline__ typename Vec4T<T>::V pack4(const float o[4]) {
  typename Vec4T<T>::V v;
  if constexpr (sizeof(T) == 4) {
    v.x = o[0]; v.y = o[1]; v.z = o[2]; v.w = o[3];
  } else if constexpr (std::is_same<T, __half>::value) {
    // two round-to-nearest-even conversions of a pair each (the same rounding as
    // __float2half_rn per value)
    const __half2 lo = __floats2half2_rn(o[0], o[1]), hi = __floats2half2_rn(o[2], o[3]);
    v.x = *reinterpret_cast<const uint32_t *>(&lo);
    v.y = *reinterpret_cast<const uint32_t *>(&hi);
  } else {
    T *e = reinterpret_cast<T *>(&v);
#pragma unroll
    for (int k = 0; k < 4; k++) Store<T>::storeRNE(e + k, o[k]);
  }
  return v;
}

template <typename T, int BS>
struct ColorSweep {
  static constexpr int NT = BS * BS / 4;     // threads: one 4-voxel x-strip of every plane each
  static constexpr int SPR = BS / 4;         // strips per row
  static constexpr int RPW = 32 / SPR;       // rows per warp
  static constexpr int NW = NT / 32;         // warps
  static constexpr int RS = BS + 8;          // ring row stride (floats); x in [-1,BS] at col x+4
  static constexpr int WR = RPW + 2;         // rows of a warp's ring plane (its rows +-1)
  static constexpr int PL = WR * RS;         // floats per warp ring plane (2 slots per warp)
  static constexpr int PLX = PL + 4;         // slot stride: a 4-float tail takes the fills of idle lanes
  static constexpr int NG = WR * SPR;        // 4-value groups of a warp ring plane
  static constexpr int NGP = (NG + 31) / 32; // groups per lane
  static constexpr int NXH = 2 * WR;         // x-halo values of a warp ring plane
  static constexpr int NHALO = 4 * BS + 4;   // halo elements of a plane (2 cols, 2 rows, 4 corners)
  static constexpr int NH = NHALO <= NT ? 1 : (NHALO + NT - 1) / NT;
  static constexpr int64_t VPB = (int64_t)BS * BS * BS;
  static constexpr int FACE = BS * BS;       // per x-face
  static constexpr int CORN = BS;            // per corner column
  static constexpr int CZ = 8;               // planes per TMA chunk (corner pieces >= 16 B)
  static constexpr int NCH = BS / CZ;        // chunks (one mbarrier each)
  static constexpr int NCC = 1 + 2 + 2 * CZ + 4 + 5;  // copy slots per chunk (<= 32)
};

// Raw (storage-type) staging of one block and its halo in shared memory.
template <typename T, int BS>
struct RawTile {
  T blk[BS * BS * BS];   // own block [z][y][x]
  T zpl[2][BS * BS];     // plane z=-1 (0) and z=BS (1), [y][x]
  T xf[2][BS * BS];      // column x=-1 (0) and x=BS (1), [z][y]
  T yr[2][BS * BS];      // row y=-1 (0) and y=BS (1), [z][x]
  T cn[4][BS];           // corner columns (x=-1|BS, y=-1|BS), k = (dx>0) + 2*(dy>0), [z]
  T zh[2][4][BS];        // planes -1 / BS: x=-1 row, x=BS row (over y), y=-1 row, y=BS row (over x)
  alignas(16) T er[16];  // the empty value (source of every fill from an empty block)
};

__device__ __forceinline__ uint32_t smemAddr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbarInit(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbarExpectTx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smemAddr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbarTryWait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smemAddr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// 1-D TMA bulk copy global -> shared, completion counted in bytes on `bar`.
__device__ __forceinline__ void bulkG2S(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smemAddr(dst)),
      "l"(src), "r"(bytes), "r"(smemAddr(bar))
      : "memory");
}

// Bounded wait on phase 0 of a chunk barrier.  Returns false after the limit.
__device__ __forceinline__ bool waitChunk(uint64_t *bar) {
  for (int it = 0; it < (1 << 22); it++)
    if (mbarTryWait(bar, 0)) return true;
  return false;
}

struct ColorArgs {
  const int32_t *bids;
  const int32_t *slot;
  void *payload;
  void *faces;    // [slot][2][BS(z)][BS(y)]  x=0 face, x=BS-1 face
  void *corners;  // [slot][4][BS(z)]  k = (x==BS-1) + 2*(y==BS-1)
  int nbx, nby, nbz;
  float emptyValue;
  int *status;    // bit 0: a chunk wait timed out
  SweepParams p;
};

// Copy slot c of chunk k (planes k*CZ .. k*CZ+CZ-1) of a block's tile: fills
// (dst, src, bytes) and returns true when the piece exists (its source block is a
// value block).  Chunk 0 also carries plane z=-1, the last chunk plane z=BS.
template <typename T, int BS>
__device__ __forceinline__ bool tileCopy(int k, int c, const int *nbs, const ColorArgs &a,
                                         RawTile<T, BS> &t, void *&dst, const void *&src,
                                         uint32_t &bytes) {
  using C = ColorSweep<T, BS>;
  constexpr int CZ = C::CZ;
  const T *pay = (const T *)a.payload;
  const T *faces = (const T *)a.faces;
  const T *corn = (const T *)a.corners;
  auto NB = [&](int dx, int dy, int dz) { return nbs[(dz + 1) * 9 + (dy + 1) * 3 + (dx + 1)]; };
  auto blkp = [&](int s) { return pay + (int64_t)s * C::VPB; };
  const int z0 = k * CZ;
  if (c == 0) {  // own planes of the chunk
    dst = t.blk + (int64_t)z0 * BS * BS;
    src = blkp(NB(0, 0, 0)) + (int64_t)z0 * BS * BS;
    bytes = CZ * BS * BS * sizeof(T);
    return true;
  }
  c -= 1;
  if (c < 2) {  // x-neighbour face rows from the cache: its x=BS-1 face for dx=-1, x=0 for dx=+1
    const int s = NB(c ? 1 : -1, 0, 0);
    if (s < 0) return false;
    dst = t.xf[c] + z0 * BS;
    src = faces + ((int64_t)s * 2 + (c ? 0 : 1)) * C::FACE + z0 * BS;
    bytes = CZ * BS * sizeof(T);
    return true;
  }
  c -= 2;
  if (c < 2 * CZ) {  // y-neighbour rows, one per plane
    const int side = c / CZ, z = z0 + c % CZ;
    const int s = NB(0, side ? 1 : -1, 0);
    if (s < 0) return false;
    dst = t.yr[side] + z * BS;
    src = blkp(s) + ((int64_t)z * BS + (side ? 0 : BS - 1)) * BS;
    bytes = BS * sizeof(T);
    return true;
  }
  c -= 2 * CZ;
  if (c < 4) {  // corner-column segments of the 4 diagonal neighbours in the block's z-layer
    const int dx = (c & 1) ? 1 : -1, dy = (c & 2) ? 1 : -1;
    const int s = NB(dx, dy, 0);
    if (s < 0) return false;
    const int kSrc = (dx < 0 ? 1 : 0) + 2 * (dy < 0 ? 1 : 0);
    dst = t.cn[c] + z0;
    src = corn + ((int64_t)s * 4 + kSrc) * C::CORN + z0;
    bytes = CZ * sizeof(T);
    return true;
  }
  c -= 4;
  // z-halo plane pieces: first chunk -> plane -1, last chunk -> plane BS
  const bool first = k == 0, last = k == C::NCH - 1;
  if (!first && !last) return false;
  const int zi = first ? 0 : 1;
  if (first && last) return false;  // (single-chunk blocks are not instantiated)
  const int dz = zi ? 1 : -1;
  const int zSrc = zi ? 0 : BS - 1;
  if (c == 0) {
    const int s = NB(0, 0, dz);
    if (s < 0) return false;
    dst = t.zpl[zi];
    src = blkp(s) + (int64_t)zSrc * BS * BS;
    bytes = BS * BS * sizeof(T);
    return true;
  }
  const int j = c - 1;  // 0 x=-1, 1 x=BS (over y), 2 y=-1, 3 y=BS (over x)
  dst = t.zh[zi][j];
  bytes = BS * sizeof(T);
  if (j < 2) {
    const int dx = j ? 1 : -1;
    const int s = NB(dx, 0, dz);
    if (s < 0) return false;
    src = faces + ((int64_t)s * 2 + (dx < 0 ? 1 : 0)) * C::FACE + zSrc * BS;
  } else {
    const int dy = j == 3 ? 1 : -1;
    const int s = NB(0, dy, dz);
    if (s < 0) return false;
    src = blkp(s) + ((int64_t)zSrc * BS + (dy < 0 ? BS - 1 : 0)) * BS;
  }
  return true;
}

template <typename T, int BS>
constexpr size_t rawTileBytes() {
  return (sizeof(RawTile<T, BS>) + 15) & ~size_t(15);
}

template <typename T, int BS>
constexpr size_t colorSmemBytes() {
  return rawTileBytes<T, BS>() + 2 * sizeof(float) * ColorSweep<T, BS>::PLX * ColorSweep<T, BS>::NW;
}

template <typename T>
__device__ __forceinline__ float ldval(const T *p) {
  if constexpr (sizeof(T) == 4) return *p; else return Store<T>::load(p);
}

// FK: the stencil, fixed at compile time.  0 = any kind in the reference's
// operation order (computeStrip); K_MCF / K_JACOBI = the fast forms, plus
// FK_CLAMP when the result is clamped to [0,1].
template <typename T, int BS, int FK>
__global__ void __launch_bounds__(ColorSweep<T, BS>::NT, 2) kSweepColor(ColorArgs a) {
  using C = ColorSweep<T, BS>;
  using V4 = typename Vec4T<T>::V;
  constexpr int RS = C::RS, PL = C::PL, PLX = C::PLX, CZ = C::CZ, NCH = C::NCH;
  extern __shared__ __align__(128) unsigned char dynSmem[];
  RawTile<T, BS> &t = *reinterpret_cast<RawTile<T, BS> *>(dynSmem);
  __shared__ int nbs[27];
  __shared__ __align__(8) uint64_t bar[NCH];

  const int tid = threadIdx.x;
  const int bid = a.bids[blockIdx.x];
  const int64_t nxy = (int64_t)a.nbx * a.nby;
  const int bz = (int)(bid / nxy), by = (int)((bid / a.nbx) % a.nby), bx = (int)(bid % a.nbx);
  if (tid < 27) {
    const int dx = tid % 3 - 1, dy = (tid / 3) % 3 - 1, dz = tid / 9 - 1;
    const int x = bx + dx, y = by + dy, z = bz + dz;
    int s = -2;  // outside the domain
    if (x >= 0 && y >= 0 && z >= 0 && x < a.nbx && y < a.nby && z < a.nbz)
      s = a.slot[(int64_t)z * nxy + (int64_t)y * a.nbx + x];
    nbs[tid] = (s < 0 && s != -2) ? -1 : s;  // -1: constant empty block
  }
  if (tid < NCH) mbarInit(&bar[tid], 1);
  if (tid == 0) asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  if (tid < 16) {
    T e;
    if constexpr (sizeof(T) == 4) e = a.emptyValue; else Store<T>::storeRNE(&e, a.emptyValue);
    t.er[tid] = e;
  }
  __syncthreads();
  if (tid < 32) {
    // warp 0, chunk by chunk: announce the chunk's bytes, then issue its copies lane-parallel
    for (int k = 0; k < NCH; k++) {
      void *d = nullptr;
      const void *s = nullptr;
      uint32_t b = 0;
      const bool has = tid < C::NCC && tileCopy<T, BS>(k, tid, nbs, a, t, d, s, b);
      uint32_t tot = has ? b : 0;
#pragma unroll
      for (int o = 16; o; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
      if (tid == 0) mbarExpectTx(&bar[k], tot);
      __syncwarp();
      if (has) bulkG2S(d, s, b, &bar[k]);
    }
  }

  const int ownSlot = nbs[13];
  const int lane = tid & 31, warp = tid >> 5;
  const int ty = tid / C::SPR, tx = (tid % C::SPR) * 4;  // this thread's strip
  const int y0w = warp * C::RPW;                          // first row of this warp
  const int tyl = ty - y0w;                               // row inside the warp
  float *wring = reinterpret_cast<float *>(dynSmem + rawTileBytes<T, BS>()) + warp * 2 * PLX;
  float emptyF;
  {
    T e;
    if constexpr (sizeof(T) == 4) e = a.emptyValue; else Store<T>::storeRNE(&e, a.emptyValue);
    if constexpr (sizeof(T) == 4) emptyF = e; else emptyF = Store<T>::load(&e);
  }

  // ---- per-lane fill sources for the interior planes 0..BS-1 ------------------
  // Quad groups: ring row rr (y = y0w-1+rr), x = 4j..4j+3; source = base + p*stride.
  // Every lane gets a source for each of its groups: an empty block (and a lane
  // without a k-th group) reads the empty row with stride 0; an idle lane writes to
  // the slot's 4-float tail.  The fill then has no branches.
  const T *gSrc[C::NGP];
  int gStride[C::NGP], gDst[C::NGP];
#pragma unroll
  for (int k = 0; k < C::NGP; k++) {
    const int g = lane + 32 * k;
    const int rr = g / C::SPR, j = g % C::SPR, y = y0w - 1 + rr, x = 4 * j;
    gDst[k] = g < C::NG ? rr * RS + x + 4 : PL;
    gSrc[k] = t.er;
    gStride[k] = 0;
    if (g < C::NG) {
      if (y >= 0 && y < BS) {
        gSrc[k] = t.blk + y * BS + x; gStride[k] = BS * BS;
      } else {
        const int side = y < 0 ? 0 : 1;
        const int s = nbs[9 + (side ? 2 : 0) * 3 + 1];
        if (s >= 0) { gSrc[k] = t.yr[side] + x; gStride[k] = BS; }
        else if (s != -1) { gSrc[k] = t.blk + (side ? BS - 1 : 0) * BS + x; gStride[k] = BS * BS; }  // Neumann
      }
    }
  }
  // x-halo values: side = lane / WR (x=-1 | x=BS), ring row rr = lane % WR
  const T *hSrc = t.er;
  int hStride = 0, hDst = PL;
  if (lane < C::NXH) {
    const int side = lane / C::WR, rr = lane % C::WR, y = y0w - 1 + rr;
    const int dx = side ? 1 : -1, xc = side ? BS - 1 : 0;
    hDst = rr * RS + (side ? BS + 4 : 3);
    if (y >= 0 && y < BS) {
      const int s = nbs[9 + 3 + (dx + 1)];
      if (s >= 0) { hSrc = t.xf[side] + y; hStride = BS; }
      else if (s != -1) { hSrc = t.blk + y * BS + xc; hStride = BS * BS; }
    } else {  // corner column of the diagonal neighbour
      const int dy = y < 0 ? -1 : 1, yc = dy < 0 ? 0 : BS - 1;
      const int s = nbs[9 + (dy + 1) * 3 + (dx + 1)];
      if (s >= 0) { hSrc = t.cn[(dx > 0 ? 1 : 0) + 2 * (dy > 0 ? 1 : 0)]; hStride = 1; }
      else if (s != -1) { hSrc = t.blk + yc * BS + xc; hStride = BS * BS; }
    }
  }

  // planes are consumed in increasing order (fillZ(-1) needs chunk 0, fillZ(BS)
  // comes after plane BS-1), so one counter of the planes known to have landed
  // replaces per-chunk flags
  int readyPlanes = 0;
  bool timedOut = false;
  auto need = [&](int p) {
    if (p >= readyPlanes) {
      if (!waitChunk(&bar[p / CZ])) timedOut = true;
      readyPlanes = (p / CZ + 1) * CZ;
    }
  };

  // ---- interior plane p (0..BS-1) -> this warp's ring slot, in two halves so
  // that the shared-memory reads of plane p overlap the previous plane's update ----
  V4 rawG[C::NGP];
  T rawH;
  auto loadRaw = [&](int p) {
    need(p);
#pragma unroll
    for (int k = 0; k < C::NGP; k++) rawG[k] = *reinterpret_cast<const V4 *>(gSrc[k] + p * gStride[k]);
    rawH = hSrc[p * hStride];
  };
  auto storeRaw = [&](float *pl) {
#pragma unroll
    for (int k = 0; k < C::NGP; k++) {
      float q[4];
      unpack4<T>(rawG[k], q);
      *reinterpret_cast<float4 *>(pl + gDst[k]) = make_float4(q[0], q[1], q[2], q[3]);
    }
    pl[hDst] = ldval<T>(&rawH);
  };
  auto fillInterior = [&](int p, float *pl) {
    loadRaw(p);
    storeRaw(pl);
  };

  // ---- z-halo plane p = -1 or BS -> this warp's ring slot (twice per block) ----
  auto fillZ = [&](int p, float *pl) {
    const int zi = p < 0 ? 0 : 1;
    need(zi ? BS - 1 : 0);
    const int dzb = zi ? 1 : -1;
    const int pc = zi ? BS - 1 : 0;  // Neumann clamp inside the own block
    for (int g = lane; g < C::NG; g += 32) {
      const int rr = g / C::SPR, j = g % C::SPR, y = y0w - 1 + rr, x = 4 * j;
      float q[4] = {emptyF, emptyF, emptyF, emptyF};
      if (y >= 0 && y < BS) {
        const int s = nbs[(dzb + 1) * 9 + 4];
        if (s >= 0) unpack4<T>(*reinterpret_cast<const V4 *>(t.zpl[zi] + y * BS + x), q);
        else if (s == -2) unpack4<T>(*reinterpret_cast<const V4 *>(t.blk + (pc * BS + y) * BS + x), q);
      } else {
        const int dy = y < 0 ? -1 : 1, yc = dy < 0 ? 0 : BS - 1;
        const int s = nbs[(dzb + 1) * 9 + (dy + 1) * 3 + 1];
        if (s >= 0) unpack4<T>(*reinterpret_cast<const V4 *>(t.zh[zi][dy < 0 ? 2 : 3] + x), q);
        else if (s == -2) unpack4<T>(*reinterpret_cast<const V4 *>(t.blk + (pc * BS + yc) * BS + x), q);
      }
      *reinterpret_cast<float4 *>(pl + rr * RS + x + 4) = make_float4(q[0], q[1], q[2], q[3]);
    }
    if (lane < C::NXH) {
      const int side = lane / C::WR, rr = lane % C::WR, y = y0w - 1 + rr;
      const int dx = side ? 1 : -1, xc = side ? BS - 1 : 0;
      float f = 0.0f;  // x-halo corners of a z-halo plane are read by no stencil
      if (y >= 0 && y < BS) {
        const int s = nbs[(dzb + 1) * 9 + 3 + (dx + 1)];
        if (s >= 0) f = ldval<T>(t.zh[zi][side] + y);
        else if (s == -1) f = emptyF;
        else f = ldval<T>(t.blk + (pc * BS + y) * BS + xc);
      }
      pl[rr * RS + (side ? BS + 4 : 3)] = f;
    }
  };

  // ---- warp ring slot -> this thread's plane (rows y-1..y+1, x-1..x+4) ----
  constexpr int FKK = FK & ~FK_CLAMP;
  using PW = std::conditional_t<FKK == K_MCF, PlaneMcf, std::conditional_t<FKK == K_JACOBI, PlaneJac, PlaneRaw>>;
  const int winOff = tyl * RS + tx + 3;
  auto window = [&](const float *pl, PW &w) { loadPlane<RS>(pl + winOff, w); };

  T *outp = (T *)a.payload + (int64_t)ownSlot * C::VPB + ty * BS + tx;
  // x-face / corner cache entries this thread maintains (x = 0 or BS-1 strips)
  const bool faceThread = tx == 0 || tx == BS - 4;
  const int kx = tx == 0 ? 0 : 1;
  T *facep = (T *)a.faces + ((int64_t)ownSlot * 2 + kx) * C::FACE + ty;
  const bool cornThread = faceThread && (ty == 0 || ty == BS - 1);
  T *cornp = (T *)a.corners + ((int64_t)ownSlot * 4 + kx + 2 * (ty == 0 ? 0 : 1)) * C::CORN;
  PW Wa, Wb, Wc;

  auto emit = [&](int z, const PW &Wm, const PW &W0, const PW &Wp) {
    float out[4];
    constexpr bool CL = (FK & FK_CLAMP) != 0;
    if constexpr (FKK == K_MCF) mcfFastStrip<CL>(Wm, W0, Wp, a.p.dt, out);
    else if constexpr (FKK == K_JACOBI) jacobiFastStrip<CL>(Wm, W0, Wp, a.p.dt, out);
    else computeStrip(Wm.w, W0.w, Wp.w, a.p, out);
    const V4 pk = pack4<T>(out);
    *reinterpret_cast<V4 *>(outp + z * BS * BS) = pk;
    T v;
    if constexpr (sizeof(T) == 4) {
      v = kx ? pk.w : pk.x;
    } else {
      const uint16_t bits = kx ? (uint16_t)(pk.y >> 16) : (uint16_t)(pk.x & 0xffffu);
      v = *reinterpret_cast<const T *>(&bits);
    }
    if (faceThread) facep[z * BS] = v;
    if (cornThread) cornp[z] = v;
  };
  // One plane.  On entry A, B, C hold planes z-1, z, z+1 and, for an interior
  // plane z+2, its raw values are in registers.  Plane z+2 is staged into the
  // warp's ring slot (z & 1), which held plane z, last read before the previous
  // step's __syncwarp; the raw values of plane z+3 are read; on exit A holds
  // plane z+2.  KIND: 0 = planes z+2 and z+3 are interior planes, 3 = only plane
  // z+2 is, 1 = plane z+2 is the z-halo plane BS, 2 = there is no plane z+2.
  auto step = [&](auto kind, int z, PW &A, PW &B, PW &Cw) {
    constexpr int KIND = decltype(kind)::value;
    float *slot = wring + (z & 1) * PLX;
    if constexpr (KIND == 0 || KIND == 3) {
      storeRaw(slot);
      if constexpr (KIND == 0) loadRaw(z + 3);
    } else if constexpr (KIND == 1) {
      fillZ(BS, slot);
    }
    __syncwarp();
    emit(z, A, B, Cw);
    if constexpr (KIND != 2) window(slot, A);
  };
  using Interior = std::integral_constant<int, 0>;

  // planes -1, 0, 1 into the windows (warp-local ring slots 0/1)
  fillZ(-1, wring);
  fillInterior(0, wring + PLX);
  __syncwarp();
  window(wring, Wa);
  window(wring + PLX, Wb);
  __syncwarp();
  fillInterior(1, wring);
  loadRaw(2);
  __syncwarp();
  window(wring, Wc);
  __syncwarp();
  // The window roles rotate every plane: (a,b,c) -> (b,c,a).  The main loop runs
  // the planes z whose planes z+2 and z+3 are interior, three at a time; the
  // last planes follow with their kinds known at compile time.
  constexpr int MAIN = 3 * ((BS - 3) / 3);
#pragma unroll 1
  for (int z = 0; z < MAIN; z += 3) {
    step(Interior{}, z, Wa, Wb, Wc);
    step(Interior{}, z + 1, Wb, Wc, Wa);
    step(Interior{}, z + 2, Wc, Wa, Wb);
  }
  static_assert(BS - MAIN >= 3 && BS - MAIN <= 5, "tail of 3..5 planes");
  auto tail = [&](auto zc) {
    constexpr int z = decltype(zc)::value;
    if constexpr (z < BS) {
      constexpr int K = z + 3 < BS ? 0 : z + 2 < BS ? 3 : (z + 2 == BS ? 1 : 2);
      using KT = std::integral_constant<int, K>;
      constexpr int r = (z - MAIN) % 3;
      if constexpr (r == 0) step(KT{}, z, Wa, Wb, Wc);
      else if constexpr (r == 1) step(KT{}, z, Wb, Wc, Wa);
      else step(KT{}, z, Wc, Wa, Wb);
    }
  };
  tail(std::integral_constant<int, MAIN>{});
  tail(std::integral_constant<int, MAIN + 1>{});
  tail(std::integral_constant<int, MAIN + 2>{});
  tail(std::integral_constant<int, MAIN + 3>{});
  tail(std::integral_constant<int, MAIN + 4>{});
  if (timedOut) {
    atomicOr(a.status, 1);
    for (int k = 0; k < NCH; k++) waitChunk(&bar[k]);  // no copy may land after exit
  }
}

// Builds the x-face and corner caches of every value block from the payload.
template <typename T, int BS>
__global__ void kExtractFaces(const T *__restrict__ pay, int64_t nAct, T *__restrict__ faces,
                              T *__restrict__ corners) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;  // (slot, z, y)
  if (i >= nAct * BS * BS) return;
  const int64_t s = i / (BS * BS);
  const int z = (int)((i / BS) % BS), y = (int)(i % BS);
  const T *row = pay + s * (int64_t)BS * BS * BS + ((int64_t)z * BS + y) * BS;
  faces[(s * 2 + 0) * BS * BS + z * BS + y] = row[0];
  faces[(s * 2 + 1) * BS * BS + z * BS + y] = row[BS - 1];
  if (y == 0 || y == BS - 1) {
    const int ky = y == 0 ? 0 : 1;
    corners[(s * 4 + 0 + 2 * ky) * BS + z] = row[0];
    corners[(s * 4 + 1 + 2 * ky) * BS + z] = row[BS - 1];
  }
}

template <typename T, int BS>
static int runColorT(msbg_gpu_ctx *ctx, Channel &c, bool exact, bool color8, int nIter,
                     const SweepParams &p, const int32_t *bids, const int *cs) {
  const int64_t nAct = ctx->nActive;
  if (nAct == 0) return MSBG_GPU_OK;
  const size_t faceBytes = (size_t)nAct * (2 * BS * BS + 4 * BS) * sizeof(T);
  if (c.cacheBytes < faceBytes) {
    if (c.cache) MSBG_CUDA(ctx, cudaFree(c.cache));
    c.cache = nullptr;
    c.cacheBytes = 0;
    MSBG_CUDA(ctx, cudaMalloc(&c.cache, faceBytes));
    c.cacheBytes = faceBytes;
  }
  T *faces = (T *)c.cache;
  T *corners = faces + (size_t)nAct * 2 * BS * BS;
  const int64_t n = nAct * BS * BS;
  MSBG_LAUNCH(ctx, (kExtractFaces<T, BS>), gridFor(n, 256), 256, 0, (const T *)c.d, nAct, faces, corners);
  ColorArgs a;
  a.slot = ctx->dSlot;
  a.payload = c.d;
  a.faces = faces;
  a.corners = corners;
  a.nbx = ctx->nbx; a.nby = ctx->nby; a.nbz = ctx->nbz;
  a.emptyValue = 0.0f;
  a.status = ctx->dStatus;
  a.p = p;
  constexpr size_t smem = colorSmemBytes<T, BS>();
  void (*const kerns[5])(ColorArgs) = {kSweepColor<T, BS, 0>, kSweepColor<T, BS, K_MCF>,
                                       kSweepColor<T, BS, K_MCF | FK_CLAMP>, kSweepColor<T, BS, K_JACOBI>,
                                       kSweepColor<T, BS, K_JACOBI | FK_CLAMP>};
  int ki = 0;  // the exact variant and the other kinds: the generic kernel
  if (!exact && p.kind == K_MCF) ki = p.constr01 ? 2 : 1;
  else if (!exact && p.kind == K_JACOBI) ki = p.constr01 ? 4 : 3;
  const auto kern = kerns[ki];
  static bool attrSet[5] = {false, false, false, false, false};
  if (!attrSet[ki]) {
    MSBG_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attrSet[ki] = true;
  }
  static const int rbOrder[2][4] = {{1, 2, 4, 7}, {0, 3, 5, 6}};
  constexpr int NT = ColorSweep<T, BS>::NT;
  int nLaunch = 0;
  for (int pass = 0; pass < 8; pass++) nLaunch += cs[pass + 1] > cs[pass];
  nLaunch *= nIter;
  if (nLaunch == 0) return MSBG_GPU_OK;
  auto launchAll = [&](cudaStream_t st) -> int {
    for (int it = 0; it < nIter; it++) {
      for (int pass = 0; pass < 8; pass++) {
        const int col = color8 ? pass : rbOrder[pass / 4][pass % 4];
        const int cnt = cs[col + 1] - cs[col];
        if (cnt <= 0) continue;
        a.bids = bids + cs[col];
        kern<<<(unsigned)cnt, NT, smem, st>>>(a);
        if (cudaGetLastError() != cudaSuccess) return MSBG_GPU_ERR_CUDA;
      }
    }
    return MSBG_GPU_OK;
  };
  // The colour passes go out as one CUDA graph, captured the first time a call
  // presents these launches (kernel, arguments, grids) and replayed after that: a
  // small layout's passes (a few hundred blocks each) are otherwise bound by the
  // launches themselves.  A context whose stream is being captured by its caller
  // launches them directly.
  cudaStreamCaptureStatus outer = cudaStreamCaptureStatusNone;
  MSBG_CUDA(ctx, cudaStreamIsCapturing(ctx->stream, &outer));
  if (outer != cudaStreamCaptureStatusNone) {
    if (launchAll(ctx->stream)) return fail(ctx, MSBG_GPU_ERR_CUDA, "sweep: launch failed");
    ctx->launches += nLaunch;
    return MSBG_GPU_OK;
  }
  std::vector<unsigned char> key;
  auto put = [&key](const auto &v) {
    const unsigned char *b = reinterpret_cast<const unsigned char *>(&v);
    key.insert(key.end(), b, b + sizeof(v));
  };
  put(reinterpret_cast<const void *>(kern)); put(bids); put(a.slot); put(a.payload); put(a.faces); put(a.corners);
  put(a.nbx); put(a.nby); put(a.nbz); put(a.emptyValue); put(a.status);
  put(p.kind); put(p.constr01); put(p.dt); put(p.anisAlpha); put(nIter); put(color8);
  for (int i = 0; i < 9; i++) put(cs[i]);
  cudaGraphExec_t exec = nullptr;
  for (size_t i = 0; i < c.sweepGraphs.size(); i++)
    if (c.sweepGraphs[i].key == key) {
      CachedGraph hit = std::move(c.sweepGraphs[i]);
      c.sweepGraphs.erase(c.sweepGraphs.begin() + i);
      c.sweepGraphs.push_back(std::move(hit));
      exec = c.sweepGraphs.back().exec;
      break;
    }
  if (!exec) {
    if (!ctx->captureStream) MSBG_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->captureStream, cudaStreamNonBlocking));
    MSBG_CUDA(ctx, cudaStreamBeginCapture(ctx->captureStream, cudaStreamCaptureModeThreadLocal));
    const int lrc = launchAll(ctx->captureStream);
    cudaGraph_t graph = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(ctx->captureStream, &graph);
    if (lrc || ee != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return fail(ctx, MSBG_GPU_ERR_CUDA, "sweep: capturing the colour passes failed");
    }
    const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) return cudaFail(ctx, ie, "cudaGraphInstantiate");
    if (c.sweepGraphs.size() >= 4) {  // keep the four most recent
      cudaGraphExecDestroy(c.sweepGraphs.front().exec);
      c.sweepGraphs.erase(c.sweepGraphs.begin());
    }
    c.sweepGraphs.push_back(CachedGraph{std::move(key), exec});
  }
  MSBG_CUDA(ctx, cudaGraphLaunch(exec, ctx->stream));
  ctx->launches += nLaunch;
  return MSBG_GPU_OK;
}

int colorSweepRun(msbg_gpu_ctx *ctx, Channel &c, bool exact, bool color8, int nIter, const SweepParams &p,
                  const int32_t *bids, const int *cs) {
  if (ctx->bsx == 32) {
    switch (c.storage) {
      case MSBG_GPU_F32: return runColorT<float, 32>(ctx, c, exact, color8, nIter, p, bids, cs);
      case MSBG_GPU_F16: return runColorT<__half, 32>(ctx, c, exact, color8, nIter, p, bids, cs);
      case MSBG_GPU_U16: return runColorT<uint16_t, 32>(ctx, c, exact, color8, nIter, p, bids, cs);
    }
  } else if (ctx->bsx == 16) {
    switch (c.storage) {
      case MSBG_GPU_F32: return runColorT<float, 16>(ctx, c, exact, color8, nIter, p, bids, cs);
      case MSBG_GPU_F16: return runColorT<__half, 16>(ctx, c, exact, color8, nIter, p, bids, cs);
      case MSBG_GPU_U16: return runColorT<uint16_t, 16>(ctx, c, exact, color8, nIter, p, bids, cs);
    }
  }
  return 1;  // not handled: caller uses the gather kernel
}

}  // namespace msbg
