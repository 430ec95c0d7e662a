"""ctypes front end of the project's C restatement (oracle/msbg_oracle.c).

Test infrastructure only: the checker that GPU results are compared with, and
the timed CPU baseline.  ``surface_pipeline`` runs the same stages, in the same
order, as the reference demo (src/msbg_demo.cpp:228-727) and returns the same
fields as ``oracle_io.run_reference_surface``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import time
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmsbg_oracle.so")

F32, U16, F16, F64 = 0, 1, 2, 3
BLK_DOM_BORDER, BLK_COARSE_FINE, BLK_FINE_COARSE = 1 << 1, 1 << 2, 1 << 3
BLK_EXISTS, BLK_UNIFORM_EMPTY = 1 << 12, 1 << 13
NP_STORAGE = {F32: np.float32, U16: np.uint16, F16: np.uint16, F64: np.float64}

_lib = None


class Grid(C.Structure):
    _fields_ = [("sx", C.c_int32), ("sy", C.c_int32), ("sz", C.c_int32), ("bsx", C.c_int32),
                ("nbx", C.c_int32), ("nby", C.c_int32), ("nbz", C.c_int32),
                ("storage", C.c_int32), ("emptyValue", C.c_double)]


def build() -> None:
    subprocess.run(["make", "-C", HERE, "port"], check=True, stdout=subprocess.DEVNULL)


def lib():
    global _lib
    if _lib is None:
        if not os.path.isfile(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        L.orc_grid_init.argtypes = [C.POINTER(Grid), C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_mark_blocks.argtypes = [C.POINTER(Grid), P, C.c_int64, C.c_float, P, P]
        L.orc_mark_blocks.restype = C.c_int64
        L.orc_bucket_points.argtypes = [C.POINTER(Grid), P, C.c_int64, P, P, P]
        L.orc_band_levels.argtypes = [C.POINTER(Grid), P, C.c_int64, P, P, C.c_int, C.c_int, P]
        L.orc_regularize.argtypes = [P, P, C.c_int, C.c_int, C.c_int, C.c_int, P]
        L.orc_block_flags.argtypes = [P, P, P, C.c_int, C.c_int, C.c_int]
        L.orc_build_slots.argtypes = [P, C.c_int, P, P]
        L.orc_build_slots.restype = C.c_int32
        L.orc_fill.argtypes = [C.POINTER(Grid), P, C.c_int64, C.c_double]
        L.orc_splat.argtypes = [C.POINTER(Grid), P, P, P, P, P, C.c_int32, P, C.c_float, C.c_float]
        L.orc_splat.restype = C.c_int64
        L.orc_finalize.argtypes = [C.POINTER(Grid), P, C.c_int64, C.c_float, C.c_float]
        L.orc_pde.argtypes = [C.POINTER(Grid), P, P, C.c_int32, P, P, C.c_int, C.c_int, C.c_int,
                              C.c_float, C.c_float]
        L.orc_pde.restype = C.c_int
        L.orc_face_coeff.argtypes = [C.c_uint32, C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_face_coeff.restype = C.c_float
        L.orc_poisson_apply.argtypes = [P, P, P, P, C.c_int]
        L.orc_poisson_rbgs.argtypes = [P, P, P, C.c_int, C.c_int]
        L.orc_poisson_smooth.argtypes = [P, C.c_int, P, P, C.c_int, C.c_int, C.c_int]
        L.orc_poisson_vcycle.argtypes = [P, C.c_int, P, P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int64]
        L.orc_poisson_vcycle.restype = C.c_int
        L.orc_poisson_mgpcg.argtypes = [P, C.c_int, P, P, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int,
                                        C.c_int, C.c_int64, C.POINTER(C.c_int), C.POINTER(C.c_double)]
        L.orc_poisson_coeffs_dense.argtypes = [C.c_uint32, C.c_int, C.c_int, C.c_int, P, P, P, P, P]
        L.orc_downsample.argtypes = [C.POINTER(Grid), P, P, C.c_int32, P, C.c_int, P]
        L.orc_interpolate.argtypes = [C.POINTER(Grid), P, P, P, C.c_int64, C.c_int, P]
        L.orc_fill_halo.argtypes = [C.POINTER(Grid), C.c_int, P, C.c_void_p, C.c_int, P, C.c_int64,
                                    C.c_int, C.c_uint, P]
        L.orc_fill_halo.restype = C.c_int64
        L.orc_render.argtypes = [C.POINTER(Grid), P, P, C.c_int, C.c_int, C.c_void_p, C.c_int, P]
        L.orc_restrict_level.argtypes = [C.POINTER(Grid), C.c_int, P, C.c_void_p, C.c_int, P, C.c_int64,
                                         C.c_int, P]
        L.orc_restrict_level.restype = C.c_int64
        L.orc_sort_blocks_morton.argtypes = [C.c_int, C.c_int, C.c_int, P, C.c_int64]
        L.orc_morton64.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32]
        L.orc_morton64.restype = C.c_uint64
        L.orc_f32_to_f16.argtypes = [C.c_float]
        L.orc_f32_to_f16.restype = C.c_uint16
        L.orc_relax_ref.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, P, P, P, P, P, P, P, C.c_int64,
                                    C.c_int, C.c_int, C.c_int, C.c_float]
        L.orc_fill_halo3.argtypes = [C.POINTER(Grid), C.c_int, P, P, P, P, C.c_int64, P, P]
        L.orc_fill_halo3.restype = C.c_int64
        L.orc_dist_fine_coarse.argtypes = [P, P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, P, P]
        L.orc_dist_fine_coarse.restype = C.c_int64
        L.orc_f16_to_f32.argtypes = [C.c_uint16]
        L.orc_f16_to_f32.restype = C.c_float
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def grid(sx, sy, sz, bsx, storage) -> Grid:
    g = Grid()
    lib().orc_grid_init(C.byref(g), sx, sy, sz, bsx, storage)
    return g


@dataclass
class PortResult:
    n_blocks: int
    n_active: int
    n_act_particles: int
    n_aborted: int
    blocks_per_level: np.ndarray
    levels: np.ndarray
    flags: np.ndarray
    active_bids: np.ndarray
    slot: np.ndarray
    after_finalize: np.ndarray
    after_pde: np.ndarray
    times: dict


def mark_blocks(g: Grid, pts: np.ndarray, r_scan: float):
    n_blocks = g.nbx * g.nby * g.nbz
    cnt = np.zeros(n_blocks, np.int32)
    valid = np.zeros(len(pts), np.uint8)
    n_valid = lib().orc_mark_blocks(C.byref(g), _p(pts), len(pts), r_scan, _p(cnt), _p(valid))
    return cnt, valid, n_valid


def particles_per_block(g: Grid, pts: np.ndarray):
    """The demo's per-block particle lists particlesPerBlock restated
    (src/msbg_demo.cpp:349-390): each point that passes the marking loop's domain tests
    (orc_mark_blocks) goes to the list of the block containing it.  CSR form: offsets
    [nBlocks+1] and point indices, each list in ascending index."""
    _, valid, _ = mark_blocks(g, pts, 0.0)
    idx = np.nonzero(valid)[0]
    ip = pts[idx].astype(np.float32).astype(np.int64)  # (int)p, as the demo's getBlockCoords
    s = int(g.bsx).bit_length() - 1
    bid = ((ip[:, 2] >> s) * g.nby + (ip[:, 1] >> s)) * g.nbx + (ip[:, 0] >> s)
    order = np.argsort(bid, kind="stable")
    cnt = np.bincount(bid, minlength=g.nbx * g.nby * g.nbz)
    off = np.zeros(len(cnt) + 1, np.int64)
    np.cumsum(cnt, out=off[1:])
    return off, idx[order].astype(np.int32)


def regularize(levels: np.ndarray, nbx, nby, nbz, n_levels):
    lv = np.ascontiguousarray(levels, np.int32).copy()
    per = np.zeros(8, np.int64)
    lib().orc_regularize(_p(lv), _p(lv), nbx, nby, nbz, n_levels, _p(per))
    return lv, per


def block_flags(levels: np.ndarray, nbx, nby, nbz, exists: np.ndarray | None = None):
    lv = np.ascontiguousarray(levels, np.int32)
    fl = np.zeros(lv.size, np.uint16)
    ex = None if exists is None else np.ascontiguousarray(exists, np.uint16)
    lib().orc_block_flags(_p(lv), None if ex is None else _p(ex), _p(fl), nbx, nby, nbz)
    return fl


def pde(g: Grid, slot, active_bids, payload: np.ndarray, lapl_typ: int, constr01: int,
        n_iter: int, dt: float, anis_alpha: float = 0.0, tmp: np.ndarray | None = None):
    if lapl_typ > 0 and tmp is None:
        tmp = np.empty_like(payload)
    rc = lib().orc_pde(C.byref(g), _p(slot), _p(active_bids), len(active_bids), _p(payload),
                       None if tmp is None else _p(tmp), lapl_typ, constr01, n_iter, dt,
                       anis_alpha)
    if rc != 0:
        raise ValueError(f"orc_pde rc={rc}")
    return payload


def downsample(g: Grid, slot, active_bids, payload: np.ndarray, simple_average: bool = False) -> np.ndarray:
    """downsampleFloatChannelNew restated (src/msbg4.cpp:1035-1379): [nActive][(bs/2)^3]."""
    cb = g.bsx // 2
    slot = np.ascontiguousarray(slot, np.int32)
    bids = np.ascontiguousarray(active_bids, np.int32)
    payload = np.ascontiguousarray(payload)
    out = np.zeros((len(bids), cb ** 3), np.float32)
    lib().orc_downsample(C.byref(g), _p(slot), _p(bids), len(bids), _p(payload), int(simple_average), _p(out))
    return out


IP_CORNER, IP_BC_DIRICHLET, IP_BC_DIRICHLET_OLD = 1 << 0, 1 << 13, 1 << 14
IP_NO_BORDER_CHECK, IP_RENDER_DENS = 1 << 15, 1 << 18


def interpolate(g: Grid, slot, payload: np.ndarray, pts: np.ndarray, opt: int = 0) -> np.ndarray:
    """Trilinear interpolation at points, restated from interpolateFloatFast /
    interpolateUint16ToFloatFast (src/sbg.h:4623-4792, src/sbg.h:4920-5032): float32 [n]."""
    slot = np.ascontiguousarray(slot, np.int32)
    payload = np.ascontiguousarray(payload)
    pts = np.ascontiguousarray(pts, np.float32).reshape(-1, 3)
    out = np.zeros(pts.shape[0], np.float32)
    lib().orc_interpolate(C.byref(g), _p(slot), _p(payload), _p(pts), pts.shape[0], int(opt), _p(out))
    return out


BC_NEUMANN, BC_COARSE_LEVEL = 1 << 10, 1 << 26
LBLK_EMPTY, LBLK_FULL, LBLK_NONE = -1, -2, -3


class LevelGrid(C.Structure):
    _fields_ = [("state", C.c_void_p), ("payload", C.c_void_p), ("emptyValue", C.c_float),
                ("fullValue", C.c_float)]


def fill_halo(g: Grid, levels, states: list, payloads: list, level: int, bids, halo: int, opt: int,
              empty_value: float = 0.0, full_value: float = 1.0) -> tuple[np.ndarray, int]:
    """fillHaloBlock_ restated (src/halo.cpp:266-479, src/halo.h:270-330) on a multi-level
    channel: float32 [len(bids)][(bs+2h)^3] and the number of skipped blocks."""
    n_levels = len(states)
    levels = np.ascontiguousarray(levels, np.int32)
    keep = []
    lgs = (LevelGrid * n_levels)()
    for l in range(n_levels):
        st = np.ascontiguousarray(states[l], np.int32)
        pay = np.ascontiguousarray(payloads[l]) if payloads[l] is not None else np.zeros(1, np.float32)
        keep += [st, pay]
        lgs[l] = LevelGrid(st.ctypes.data, pay.ctypes.data, empty_value, full_value)
    bids = np.ascontiguousarray(bids, np.int32)
    hs = (g.bsx >> level) + 2 * halo
    out = np.zeros((len(bids), hs ** 3), np.float32)
    skipped = lib().orc_fill_halo(C.byref(g), n_levels, _p(levels), C.cast(lgs, C.c_void_p), level,
                                  _p(bids), len(bids),
                                  halo, opt, _p(out))
    return out, int(skipped)


def dist_fine_coarse(levels, flags, nb, bsx: int, level: int, d_trans_res: int = 6):
    """CH_DIST_FINECOARSE of level `level` restated: (state int32 [nBlocks], uint16 [n][(bsx>>l)^3])."""
    lv = np.ascontiguousarray(levels, np.int32)
    fl = np.ascontiguousarray(flags, np.uint16)
    bs = bsx >> level
    state = np.empty(lv.size, np.int32)
    data = np.zeros((lv.size, bs ** 3), np.uint16)
    n = lib().orc_dist_fine_coarse(_p(lv), _p(fl), nb[0], nb[1], nb[2], bsx, level, d_trans_res, _p(state), _p(data))
    return state, data[:n].copy()


class FlagGrid(C.Structure):
    _fields_ = [("state", C.c_void_p), ("payload", C.c_void_p), ("emptyFlags", C.c_uint16),
                ("fullFlags", C.c_uint16)]


def fill_halo3(g: Grid, levels, states: list, payloads: list, flag_states: list, flag_payloads: list, bids,
               domain_bc, empty_value: float = 0.0, full_value: float = 1.0, empty_flags: int = 0,
               full_flags: int = 0) -> tuple[np.ndarray, int]:
    """fillHaloBlock3 restated (src/halo.cpp:536-738) at multigrid level 0: float32
    [len(bids)][(bsx+2)^3] and the number of skipped blocks."""
    n_levels = len(states)
    levels = np.ascontiguousarray(levels, np.int32)
    keep = []
    lgs = (LevelGrid * n_levels)()
    lfs = (FlagGrid * n_levels)()
    for l in range(n_levels):
        st = np.ascontiguousarray(states[l], np.int32)
        pay = np.ascontiguousarray(payloads[l]) if payloads[l] is not None else np.zeros(1, np.float32)
        fs = np.ascontiguousarray(flag_states[l], np.int32)
        fp = np.ascontiguousarray(flag_payloads[l], np.uint16) if flag_payloads[l] is not None else np.zeros(1, np.uint16)
        keep += [st, pay, fs, fp]
        lgs[l] = LevelGrid(st.ctypes.data, pay.ctypes.data, empty_value, full_value)
        lfs[l] = FlagGrid(fs.ctypes.data, fp.ctypes.data, empty_flags, full_flags)
    bids = np.ascontiguousarray(bids, np.int32)
    hs = g.bsx + 2
    out = np.zeros((len(bids), hs ** 3), np.float32)
    dbc = np.ascontiguousarray(domain_bc, np.int32)
    skipped = lib().orc_fill_halo3(C.byref(g), n_levels, _p(levels), C.cast(lgs, C.c_void_p), C.cast(lfs, C.c_void_p),
                                   _p(bids), len(bids), _p(dbc), _p(out))
    return out, int(skipped)


def restrict_level(g: Grid, levels, states: list, payloads: list, level: int, bids,
                   simple_average: bool = False, empty_value: float = 0.0, full_value: float = 1.0):
    """downsampleFloatChannelNew restated for blocks of a multi-level channel (cross-resolution
    halo): float32 [len(bids)][(bs/2)^3] and the number of skipped blocks."""
    n_levels = len(states)
    levels = np.ascontiguousarray(levels, np.int32)
    keep = []
    lgs = (LevelGrid * n_levels)()
    for l in range(n_levels):
        st = np.ascontiguousarray(states[l], np.int32)
        pay = np.ascontiguousarray(payloads[l]) if payloads[l] is not None else np.zeros(1, np.float32)
        keep += [st, pay]
        lgs[l] = LevelGrid(st.ctypes.data, pay.ctypes.data, empty_value, full_value)
    bids = np.ascontiguousarray(bids, np.int32)
    cb = (g.bsx >> level) // 2
    out = np.zeros((len(bids), cb ** 3), np.float32)
    skipped = lib().orc_restrict_level(C.byref(g), n_levels, _p(levels), C.cast(lgs, C.c_void_p), level,
                                       _p(bids), len(bids), int(simple_average), _p(out))
    return out, int(skipped)


def sort_blocks_morton(nbx: int, nby: int, nbz: int, bids) -> np.ndarray:
    """sortBlockListMorton restated (src/msbg2.cpp:46-58): the list in Morton order."""
    out = np.ascontiguousarray(bids, np.int32).copy()
    lib().orc_sort_blocks_morton(nbx, nby, nbz, _p(out), out.size)
    return out


class Camera(C.Structure):
    _fields_ = [("pos", C.c_double * 3), ("lookAt", C.c_double * 3), ("sun", C.c_double * 3),
                ("color", C.c_double * 3), ("zoom", C.c_double)]


# the demo's camera (src/msbg_demo.cpp:123-127) and surface colour (src/msbg_demo.cpp:150),
# float literals as the demo passes them
DEMO_CAMERA = {"pos": (0.5, 0.8, 0.7), "look_at": (0.5, 0.5, 0.5), "sun": (0.5, 5.0, 5.0),
               "color": (0.8, 0.6, 0.4), "zoom": 1.0}


def camera(cam: dict | None = None) -> Camera:
    cam = DEMO_CAMERA if cam is None else cam
    f = lambda v: [float(np.float32(x)) for x in v]  # noqa: E731
    return Camera((C.c_double * 3)(*f(cam["pos"])), (C.c_double * 3)(*f(cam["look_at"])),
                  (C.c_double * 3)(*f(cam["sun"])), (C.c_double * 3)(*f(cam["color"])),
                  float(np.float32(cam["zoom"])))


def render(g: Grid, slot, payload: np.ndarray, width: int, height: int, cam: dict | None = None,
           opt: int = 0) -> np.ndarray:
    """RaymarchRenderer::render restated (src/render.cpp:20-101): int32 [height][width]
    pixels as BMP_MKRGB (0x02000000 | b<<16 | g<<8 | r)."""
    slot = np.ascontiguousarray(slot, np.int32)
    payload = np.ascontiguousarray(payload)
    out = np.zeros((height, width), np.int32)
    c = camera(cam)
    lib().orc_render(C.byref(g), _p(slot), _p(payload), width, height, C.cast(C.byref(c), C.c_void_p), opt,
                     _p(out))
    return out


def surface_pipeline(pts: np.ndarray, res, bsx: int, storage: int = F32, n_iter: int = 20,
                     lapl_typ: int = -(4 + (1 << 29)), constr01: int = 1, dt: float = 0.1,
                     r_particle: float = 2.0, nb_dist: float = 2.0, n_levels: int = 3,
                     bands=None, levels_in: np.ndarray | None = None,
                     anis_alpha: float = 0.0) -> PortResult:
    """Mark -> levels -> regularize -> slots -> fill(1) -> splat -> finalize -> sweeps.

    ``bands`` (optional, e.g. (8, 16)) selects the distance-band level map of the
    multi-level workload instead of the demo's single band of width rScan.
    """
    sx, sy, sz = (res, res, res) if np.isscalar(res) else res
    pts = np.ascontiguousarray(pts, np.float32).reshape(-1, 3)
    g = grid(sx, sy, sz, bsx, storage)
    n_blocks = g.nbx * g.nby * g.nbz
    times = {}
    t0 = time.perf_counter()
    cnt, valid, n_valid = mark_blocks(g, pts, r_particle + nb_dist)
    times["mark"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    if levels_in is not None:
        levels = np.ascontiguousarray(levels_in, np.int32).copy()
    elif bands is None:
        levels = np.where(cnt > 0, 0, n_levels - 1).astype(np.int32)
    else:
        levels = np.zeros(n_blocks, np.int32)
        rb = np.asarray(bands, np.float32)
        lib().orc_band_levels(C.byref(g), _p(pts), len(pts), _p(valid), _p(rb), len(rb),
                              n_levels, _p(levels))
    levels, per = regularize(levels, g.nbx, g.nby, g.nbz, n_levels)
    # setRefinementMap sees no BLK_EXISTS; the demo's allocation loop then sets it
    # on every level-0 block (src/msbg_demo.cpp:477-491).
    flags = block_flags(levels, g.nbx, g.nby, g.nbz)
    flags[levels == 0] |= BLK_EXISTS
    times["levels"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    slot = np.empty(n_blocks, np.int32)
    bids = np.empty(n_blocks, np.int32)
    n_active = lib().orc_build_slots(_p(levels), n_blocks, _p(slot), _p(bids))
    bids = bids[:n_active].copy()
    nv = bsx ** 3
    payload = np.empty(n_active * nv, NP_STORAGE[storage])
    lib().orc_fill(C.byref(g), _p(payload), n_active, 1.0)
    bstart = np.empty(n_blocks + 1, np.int64)
    bidx = np.empty(max(int(n_valid), 1), np.int64)
    lib().orc_bucket_points(C.byref(g), _p(pts), len(pts), _p(valid), _p(bstart), _p(bidx))
    times["alloc"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    n_abort = lib().orc_splat(C.byref(g), _p(pts), _p(bstart), _p(bidx), _p(slot), _p(bids),
                              n_active, _p(payload), r_particle, nb_dist)
    times["splat"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    lib().orc_finalize(C.byref(g), _p(payload), n_active, r_particle, nb_dist)
    times["final"] = time.perf_counter() - t0
    after_final = payload.copy()
    t0 = time.perf_counter()
    if n_iter > 0:
        pde(g, slot, bids, payload, lapl_typ, constr01, n_iter, dt, anis_alpha)
    times["pde"] = time.perf_counter() - t0
    return PortResult(n_blocks, n_active, int(n_valid), int(n_abort), per, levels.astype(np.int8),
                      flags, bids, slot, after_final.reshape(n_active, nv),
                      payload.reshape(n_active, nv), times)


def to_float(storage: int, a: np.ndarray) -> np.ndarray:
    """Payload values as float64 (uint16 densities scaled by 1/65535)."""
    if storage == U16:
        return a.astype(np.float64) / 65535.0
    if storage == F16:
        return a.view(np.float16).astype(np.float64)
    return a.astype(np.float64)


# ---- sparse Poisson (FP64 restatement) ------------------------------------------------
class Level0(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("act", C.c_void_p),
                ("cx", C.c_void_p), ("cy", C.c_void_p), ("cz", C.c_void_p), ("d", C.c_void_p)]


def payload_to_dense(payload: np.ndarray, bids: np.ndarray, nb, bs: int, dtype=np.float64):
    """[nActive][bs^3] payload -> dense (nz*bs, ny*bs, nx*bs) array (zeros elsewhere)."""
    nbx, nby, nbz = nb
    out = np.zeros((nbz * bs, nby * bs, nbx * bs), dtype)
    pay = np.asarray(payload).reshape(len(bids), bs, bs, bs)
    bx, by, bz = bids % nbx, (bids // nbx) % nby, bids // (nbx * nby)
    for k in range(len(bids)):
        out[bz[k] * bs:(bz[k] + 1) * bs, by[k] * bs:(by[k] + 1) * bs, bx[k] * bs:(bx[k] + 1) * bs] = pay[k]
    return out


def dense_to_payload(dense: np.ndarray, bids: np.ndarray, nb, bs: int, dtype=np.float32):
    nbx, nby, nbz = nb
    out = np.empty((len(bids), bs, bs, bs), dtype)
    bx, by, bz = bids % nbx, (bids // nbx) % nby, bids // (nbx * nby)
    for k in range(len(bids)):
        out[k] = dense[bz[k] * bs:(bz[k] + 1) * bs, by[k] * bs:(by[k] + 1) * bs, bx[k] * bs:(bx[k] + 1) * bs]
    return out.reshape(len(bids), bs ** 3)


def active_mask(bids: np.ndarray, nb, bs: int) -> np.ndarray:
    return payload_to_dense(np.ones((len(bids), bs ** 3), np.uint8), bids, nb, bs, np.uint8)


# Multigrid parameters shared with the GPU solver's defaults: smoothing passes
# before / after the coarse correction, in-tile red-black sweeps per pass, the
# coarsest level's red-black sweeps (0 = exact Cholesky solve), and the cell
# count at which coarsening stops.
MG_PRE, MG_POST, MG_TILE_ITERS, MG_COARSEST_ITER, MG_COARSEST_CELLS = 2, 2, 3, 0, 512
# The reference's smoother constants (src/msbg.cpp:814-843): omega = 6/7 (as a float),
# 5 block-local iterations.
REF_SM_OMEGA, REF_SM_BLOCK_ITER = float(np.float32(6.0) / np.float32(7.0)), 5


class PoissonProblem:
    """Dense FP64 restatement of one Poisson problem on a value-block layout."""

    def __init__(self, bids: np.ndarray, nb, bs: int, seed: int, pre: int = MG_PRE, post: int = MG_POST,
                 tile_iters: int = MG_TILE_ITERS, coarsest_iter: int = MG_COARSEST_ITER,
                 coarsest_cells: int = MG_COARSEST_CELLS):
        self.bids, self.nb, self.bs, self.seed = np.asarray(bids, np.int64), nb, bs, seed
        self.pre, self.post, self.k = pre, post, tile_iters
        self.coarsest_iter, self.coarsest_cells = coarsest_iter, coarsest_cells
        self.act = np.ascontiguousarray(active_mask(self.bids, nb, bs))
        nz, ny, nx = self.act.shape
        self.cx, self.cy, self.cz, self.d = (np.zeros(self.act.shape) for _ in range(4))
        lib().orc_poisson_coeffs_dense(seed, nx, ny, nz, _p(self.act), _p(self.cx), _p(self.cy),
                                       _p(self.cz), _p(self.d))
        self.L = Level0(nx, ny, nz, self.act.ctypes.data, self.cx.ctypes.data, self.cy.ctypes.data,
                        self.cz.ctypes.data, self.d.ctypes.data)
        self.log2bs = int(round(np.log2(bs)))

    def dense(self, payload):
        return np.ascontiguousarray(payload_to_dense(payload, self.bids, self.nb, self.bs))

    def payload(self, dense):
        return dense_to_payload(dense, self.bids, self.nb, self.bs)

    def apply(self, x, b=None):
        y = np.zeros_like(self.d)
        bb = np.zeros_like(self.d) if b is None else np.ascontiguousarray(b, np.float64)
        lib().orc_poisson_apply(C.byref(self.L), _p(np.ascontiguousarray(x, np.float64)), _p(bb), _p(y),
                                0 if b is None else 1)
        return y

    def rbgs(self, x, b, n, red_first=True):
        x = np.ascontiguousarray(x, np.float64).copy()
        lib().orc_poisson_rbgs(C.byref(self.L), _p(x), _p(np.ascontiguousarray(b, np.float64)), n,
                               int(red_first))
        return x

    def smooth(self, x, b, passes, reverse=False):
        """Smoothing passes of level 0 (tile or pointwise red-black, k in-tile sweeps)."""
        x = np.ascontiguousarray(x, np.float64).copy()
        lib().orc_poisson_smooth(C.byref(self.L), self.log2bs, _p(x), _p(np.ascontiguousarray(b, np.float64)),
                                 passes, self.k, int(reverse))
        return x

    def vcycle(self, b):
        x = np.zeros_like(self.d)
        nlev = lib().orc_poisson_vcycle(C.byref(self.L), self.log2bs, _p(np.ascontiguousarray(b, np.float64)),
                                        _p(x), self.pre, self.post, self.k, self.coarsest_iter,
                                        self.coarsest_cells)
        return x, nlev

    def solve(self, b, tol=1e-6, max_iter=200, x0=None):
        x = np.zeros_like(self.d) if x0 is None else np.ascontiguousarray(x0, np.float64).copy()
        it, rel = C.c_int(), C.c_double()
        lib().orc_poisson_mgpcg(C.byref(self.L), self.log2bs, _p(np.ascontiguousarray(b, np.float64)),
                                _p(x), tol, max_iter, self.pre, self.post, self.k, self.coarsest_iter,
                                self.coarsest_cells, C.byref(it), C.byref(rel))
        return x, it.value, rel.value

    def relax_reference(self, x, b, passes=1, reverse=False, block_iter=REF_SM_BLOCK_ITER,
                        omega=REF_SM_OMEGA, block_list=None):
        """The reference's block smoother (orc_relax_ref) in FP32 on this problem's
        coefficients: dense x, b in, relaxed dense x (float32) out."""
        nz, ny, nx = self.act.shape
        f = lambda a: np.ascontiguousarray(a, np.float32)
        xx = f(np.where(self.act > 0, x, 0.0)).copy()
        dinv = f(np.where(self.act > 0, 1.0 / np.where(self.act > 0, self.d.astype(np.float32), 1.0), 0.0))
        bl = np.ascontiguousarray(self.bids if block_list is None else block_list, np.int32)
        lib().orc_relax_ref(nx, ny, nz, self.bs, _p(xx), _p(f(b)), _p(f(self.cx)), _p(f(self.cy)),
                            _p(f(self.cz)), _p(dinv), _p(bl), len(bl), passes, int(reverse), block_iter, omega)
        return xx

    def rel_residual(self, x, b):
        r = self.apply(x, b)
        return float(np.linalg.norm(r) / np.linalg.norm(b))


# procNeighMixedRes2's face weights (src/msbg.h:82-87, src/msbg3.cpp:46-161), as the FP32
# values the reference forms: a coarse cell next to finer blocks takes 1/3 of each of the
# four fine cells across the face (DPMR_GRAD_COEFF_CF), a fine cell next to a coarser block
# 2/3 of the one coarse cell (h * 2 * DPMR_GRAD_COEFF_CF with h = 1).
MR_COEFF_CF = np.float32(1.0 / (4 * 0.75))
MR_COEFF_FC = np.float32(1.0 * 2 * (1.0 / (4 * 0.75)))


class _MultiresLayout:
    """Blocks of a multi-resolution layout over flat float32 arrays ordered by level, then
    ascending bid ((bsx>>l)^3 values [z][y][x] per block of level l), and the halo of a block
    as the reference's operator and smoother read it (IprocessBlockLaplacian,
    src/msbg3.cpp:563-1042): h X inside, h X of a same-level face neighbour, procNeighMixedRes2's
    weighted values across a face to another level (src/msbg3.cpp:46-161), zero outside."""

    def __init__(self, sx, sy, sz, bsx, n_levels, levels, x):
        self.bsx, self.lv = bsx, np.asarray(levels).ravel()
        self.nbx, self.nby, self.nbz = sx // bsx, sy // bsx, sz // bsx
        self.blocks, self.order, off = {}, [], 0
        for l in range(n_levels):
            bs = bsx >> l
            for bid in np.flatnonzero(self.lv == l):
                n = bs ** 3
                self.blocks[int(bid)] = (l, off, x[off:off + n].reshape(bs, bs, bs))
                self.order.append(int(bid))
                off += n
        if off != x.size:
            raise ValueError("array sizes do not match the level map")

    def face(self, bid, l, axis, side):
        """Halo plane of block bid (level l) on face (axis 0 x / 1 y / 2 z, side 0 low /
        1 high), as [z][y] (x faces), [z][x] (y faces) or [y][x] (z faces), scaled by h."""
        f32, f64 = np.float32, np.float64
        bs, h = self.bsx >> l, f32(2 ** l)
        nbx, nby, nbz = self.nbx, self.nby, self.nbz
        bxyz = [bid % nbx, (bid // nbx) % nby, bid // (nbx * nby)]
        bxyz[axis] += 1 if side else -1
        if not (0 <= bxyz[0] < nbx and 0 <= bxyz[1] < nby and 0 <= bxyz[2] < nbz):
            return np.zeros((bs, bs), f32)
        l2, _, X2 = self.blocks[bxyz[0] + bxyz[1] * nbx + bxyz[2] * nbx * nby]
        k = (self.bsx >> l2) - 1 if side == 0 else 0  # the neighbour's plane that touches the face
        plane = (X2[:, :, k], X2[:, k, :], X2[k, :, :])[axis]
        if l2 == l:
            return plane * h
        if l2 == l + 1:  # coarser neighbour: each coarse cell serves 2x2 fine cells
            v = (MR_COEFF_FC * plane) * h
            return np.repeat(np.repeat(v, 2, axis=0), 2, axis=1)
        if l2 == l - 1:  # finer neighbour: four fine cells per coarse cell, FP64 sum
            p = (MR_COEFF_CF * plane).astype(f64)
            # plane axes (outer, inner): x faces (z, y), y faces (z, x), z faces (y, x);
            # the reference adds (inner, outer) offsets (0,0), (1,0), (0,1), (1,1)
            s = p[0::2, 0::2] + p[0::2, 1::2]
            s = s + p[1::2, 0::2]
            s = s + p[1::2, 1::2]
            return (s * f64(h)).astype(f32)
        raise ValueError("level map is not regular")

    def halo(self, bid):
        """(level, offset, h X of the block with its six face layers, (bs+2)^3 float32)."""
        l, o, X = self.blocks[bid]
        bs = self.bsx >> l
        P = np.zeros((bs + 2,) * 3, np.float32)
        P[1:-1, 1:-1, 1:-1] = X * np.float32(2 ** l)
        P[1:-1, 1:-1, 0], P[1:-1, 1:-1, -1] = self.face(bid, l, 0, 0), self.face(bid, l, 0, 1)
        P[1:-1, 0, 1:-1], P[1:-1, -1, 1:-1] = self.face(bid, l, 1, 0), self.face(bid, l, 1, 1)
        P[0, 1:-1, 1:-1], P[-1, 1:-1, 1:-1] = self.face(bid, l, 2, 0), self.face(bid, l, 2, 1)
        return l, o, P


def _six(P):
    """The six neighbours F1..F6 (x-1, x+1, y-1, y+1, z-1, z+1) of every interior cell of P."""
    return (P[1:-1, 1:-1, :-2], P[1:-1, 1:-1, 2:], P[1:-1, :-2, 1:-1], P[1:-1, 2:, 1:-1],
            P[:-2, 1:-1, 1:-1], P[2:, 1:-1, 1:-1])


def multiply_laplacian_levels(sx, sy, sz, bsx, n_levels, levels, x, b, dinv):
    """multiplyLaplacianMatrixOpt (src/msbg3.cpp:1756-1912, IprocessBlockLaplacian
    src/msbg3.cpp:418-1335) on a multi-resolution layout, every block a fluid block at its
    level (levels: regular, one entry per block), unit face areas, fluid cells.  x, b, dinv:
    float32 over the blocks of level 0, then level 1, ..., ascending bid, (bsx>>l)^3 values
    [z][y][x] per block of level l; dinv is what CH_DIAGONAL holds.

    Per cell of a block at level l (h = 2^l): F0 = h X; the six neighbours F1..F6 (x-1, x+1,
    y-1, y+1, z-1, z+1) are h X of the neighbour cell, in the block or in a face neighbour at
    the same level (zero outside the domain); across a face to a coarser block h times the
    FP32 product 2/3 X_coarse (src/msbg3.cpp:109-141); across a face to a finer block h times
    the FP64 sum, in the reference's order, of the four FP32 products 1/3 X_fine
    (src/msbg3.cpp:77-107).  S = F1 + ... + F6 and Y = (1/dinv) F0 - S where dinv != 0,
    else 0 (src/msbg3.cpp:1266-1285), all FP32; R = B - Y; the dot product sum(Y * F0/h)
    in FP64.  The reference as compiled here (-O3 -ffast-math -march=native) adds S as
    (F1+F2) + (F3+F4) + (F5+F6) and forms Y with one fused multiply-add in its 4- and 8-wide
    SIMD paths (blocks of edge >= 4), and keeps the source order (S left to right, Y a
    multiply then a subtraction) in its 2-wide path (blocks of edge 2); this restatement does
    the same (the product of two FP32 values is exact in FP64) and matches it bit for bit.
    Returns (dot, y, r) in x's order."""
    f32, f64 = np.float32, np.float64
    x, b, dinv = (np.asarray(a, f32).ravel() for a in (x, b, dinv))
    L = _MultiresLayout(sx, sy, sz, bsx, n_levels, levels, x)
    y, r = np.empty_like(x), np.empty_like(x)
    dot = 0.0
    for bid in L.order:
        l, o, P = L.halo(bid)
        bs, h = bsx >> l, f32(2 ** l)
        n = bs ** 3
        F0 = P[1:-1, 1:-1, 1:-1]
        F = _six(P)
        if bs >= 4:
            S = ((F[0] + F[1]) + (F[2] + F[3])) + (F[4] + F[5])
        else:
            S = ((((F[0] + F[1]) + F[2]) + F[3]) + F[4]) + F[5]
        D = dinv[o:o + n].reshape(bs, bs, bs)
        with np.errstate(divide="ignore"):
            rD = f32(1.0) / D
        if bs >= 4:
            Y = np.where(D != 0, (rD.astype(f64) * F0.astype(f64) - S.astype(f64)).astype(f32), f32(0.0))
        else:
            Y = np.where(D != 0, rD * F0 - S, f32(0.0)).astype(f32)
        y[o:o + n] = Y.ravel()
        r[o:o + n] = (b[o:o + n] - Y.ravel()).astype(f32)
        dot += float((Y.astype(f64) * (F0 * f32(1.0 / h)).astype(f64)).sum())
    return dot, y, r


def relax_levels(sx, sy, sz, bsx, n_levels, levels, x, b, dinv, passes=1, reverse=False,
                 block_iter=REF_SM_BLOCK_ITER, omega=REF_SM_OMEGA):
    """relaxBlockList (src/msbg3.cpp:2170-2239), `passes` times, on a multi-resolution layout
    laid out as for multiply_laplacian_levels: red-black over the blocks of every level (parity
    (bx+by+bz)&1 = 1 first, 0 first with reverse), each block relaxed in place from its halo
    (the operator's, read once at its start) by block_iter block-local iterations
    (IprocessBlockLaplacian's RELAX mode, src/msbg3.cpp:1108-1398): groups of the reference's
    SIMD width (8 cells along x, or the block edge below 8) in z, y, x order, backward on
    alternate iterations (the other way with reverse), each group computed from the buffer
    before it is stored; the last iteration, computed from the buffer without storing
    into it, gives X = Y / h.  Per cell Y = omega (B + S) D + (1 - omega) F0 with S = F1 + ...
    + F6 and D what CH_DIAGONAL holds.  The reference's build evaluates it in its 4- and 8-wide
    paths (block edge >= 4) as S = (F1+F2) + (F3+F4) + (F5+F6), t = S + B,
    Y = fma(1 - omega, F0, (omega D) t), and in its 2-wide path in source order; this
    restatement does the same and matches it bit for bit.  Returns the relaxed x."""
    f32, f64 = np.float32, np.float64
    x = np.asarray(x, f32).ravel().copy()
    b, dinv = (np.asarray(a, f32).ravel() for a in (b, dinv))
    L = _MultiresLayout(sx, sy, sz, bsx, n_levels, levels, x)
    om = f32(omega)
    om1 = f32(1.0) - om
    parities = (0, 1) if reverse else (1, 0)
    for _ in range(passes):
        for par in parities:
            for bid in L.order:
                if (bid % L.nbx + (bid // L.nbx) % L.nby + bid // (L.nbx * L.nby)) & 1 != par:
                    continue
                l, o, Pb = L.halo(bid)
                bs, h = bsx >> l, f32(2 ** l)
                n = bs ** 3
                B = b[o:o + n].reshape(bs, bs, bs)
                D = dinv[o:o + n].reshape(bs, bs, bs)
                gw = 8 if bs >= 8 else bs
                ng = bs // gw

                def update(k, j, i):
                    F0 = Pb[k + 1, j + 1, i + 1]
                    F = (Pb[k + 1, j + 1, i], Pb[k + 1, j + 1, i + 2], Pb[k + 1, j, i + 1], Pb[k + 1, j + 2, i + 1],
                         Pb[k, j + 1, i + 1], Pb[k + 2, j + 1, i + 1])
                    Bc, Dc = B[k, j, i], D[k, j, i]
                    if bs >= 4:
                        t = (((F[0] + F[1]) + (F[2] + F[3])) + (F[4] + F[5])) + Bc
                        return (om1.astype(f64) * F0.astype(f64) + ((om * Dc) * t).astype(f64)).astype(f32)
                    t = (((((F[0] + F[1]) + F[2]) + F[3]) + F[4]) + F[5]) + Bc
                    return ((om * t) * Dc + om1 * F0).astype(f32)

                gi, jj, kk = np.meshgrid(np.arange(ng), np.arange(bs), np.arange(bs), indexing="ij")
                wave = gi + jj + kk  # groups on one wavefront share no face: updated together
                for it in range(block_iter):
                    if it < block_iter - 1:
                        backward = bool(reverse) == bool(it & 1)
                        for t in range(ng + 2 * bs - 2):
                            m = wave == t
                            g0, j0, k0 = gi[m], jj[m], kk[m]
                            if backward:
                                g0, j0, k0 = ng - 1 - g0, bs - 1 - j0, bs - 1 - k0
                            ci = (g0[:, None] * gw + np.arange(gw)[None, :]).ravel()
                            cj, ck = np.repeat(j0, gw), np.repeat(k0, gw)
                            Pb[ck + 1, cj + 1, ci + 1] = update(ck, cj, ci)
                    else:
                        ck, cj, ci = (a.ravel() for a in np.meshgrid(np.arange(bs), np.arange(bs), np.arange(bs),
                                                                     indexing="ij"))
                        L.blocks[bid][2][...] = (update(ck, cj, ci) * f32(1.0 / h)).reshape(bs, bs, bs)
    return x


CELL_SOLID, CELL_PARTIAL_SOLID, CELL_VOID = 1 << 0, 1 << 6, 1 << 12


def multiply_laplacian_dense(flags, x, b, dinv, area_x, area_y, area_z, h):
    """multiplyLaplacianMatrixOpt at a dense multigrid level: the masked 7-point operator of
    ImultiplyLaplacianMatrixProcessSliceDenseLevel (src/msbg3.cpp:166-403) on [sz][sy][sx]
    arrays (x fastest), X and the face areas 0 outside the box.  The reference walks each row
    in groups of 4 cells from x = 0: a group without a fluid cell (not CELL_SOLID or
    CELL_VOID) is skipped (its outputs are not written: 0 here); a group in which some cell is
    CELL_SOLID or CELL_PARTIAL_SOLID weighs every cell's neighbours F1..F6 by the face areas
    (lower faces of the cell, upper faces = lower faces of the next cell).  Per cell
    Y = h (1/dinv) X - h S with S = F1 + ... + F6, zero for non-fluid cells; the residual
    B - Y for every cell of a processed group.  The reference as compiled here folds the
    reciprocal into a division and adds S as (F1+F2) + ((F3+F4) + (F5+F6)):
    Y = h (X / dinv - S), which this restatement follows bit for bit.  Returns (y, r)."""
    f32 = np.float32
    fl = np.asarray(flags).astype(np.int64)
    sz, sy, sx = fl.shape
    x, b, dinv, ax, ay, az = (np.asarray(a, f32).reshape(fl.shape) for a in (x, b, dinv, area_x, area_y, area_z))
    X = np.pad(x, 1)
    AX, AY, AZ = np.pad(ax, 1), np.pad(ay, 1), np.pad(az, 1)
    F = [X[1:-1, 1:-1, :-2], X[1:-1, 1:-1, 2:], X[1:-1, :-2, 1:-1], X[1:-1, 2:, 1:-1], X[:-2, 1:-1, 1:-1],
         X[2:, 1:-1, 1:-1]]
    W = [ax, AX[1:-1, 1:-1, 2:], ay, AY[1:-1, 2:, 1:-1], az, AZ[2:, 1:-1, 1:-1]]
    fluid = (fl & (CELL_SOLID | CELL_VOID)) == 0
    part = (fl & (CELL_SOLID | CELL_PARTIAL_SOLID)) != 0
    g = -(-sx // 4) * 4

    def group_any(m):
        mm = np.zeros((sz, sy, g), bool)
        mm[:, :, :sx] = m
        return np.repeat(mm.reshape(sz, sy, g // 4, 4).any(-1), 4, axis=-1)[:, :, :sx]

    weighted, active = group_any(part), group_any(fluid)
    Fw = [np.where(weighted, Fi * Wi, Fi).astype(f32) for Fi, Wi in zip(F, W)]
    S = (Fw[0] + Fw[1]) + ((Fw[2] + Fw[3]) + (Fw[4] + Fw[5]))
    with np.errstate(divide="ignore", invalid="ignore"):
        Y = ((x / dinv).astype(f32) - S) * f32(h)
    Y = np.where(fluid, Y, f32(0.0)).astype(f32)
    y = np.where(active, Y, f32(0.0)).astype(f32)
    r = np.where(active, b - Y, f32(0.0)).astype(f32)
    return y, r


def relax_dense(flags, x, b, dinv, area_x, area_y, area_z, h, iters, omega=REF_SM_OMEGA, tmp=None):
    """relax() at a dense multigrid level (src/msbg3.cpp:2244-2310 -> 1917-2165): `iters`
    omega-Jacobi iterations of the operator of multiply_laplacian_dense, alternating between x
    and a temporary array (tmp, zero by default), the result copied to x after an odd count.
    Per iteration the 4-cell groups of multiply_laplacian_dense decide skipping (a skipped
    group's cells keep what the destination held) and weighting; fluid cells get
    Y = omega h^-1 D (B + h S) + (1 - omega) F0, other cells of a processed group 0.  The
    reference's build evaluates it as fma(1 - omega, F0, (B + h S) (D omega/h)) with S as in
    the operator; so does this restatement, which matches it bit for bit.  Returns x after
    the iterations."""
    f32, f64 = np.float32, np.float64
    fl = np.asarray(flags).astype(np.int64)
    sz, sy, sx = fl.shape
    x, b, dinv, ax, ay, az = (np.asarray(a, f32).reshape(fl.shape) for a in (x, b, dinv, area_x, area_y, area_z))
    fluid = (fl & (CELL_SOLID | CELL_VOID)) == 0
    part = (fl & (CELL_SOLID | CELL_PARTIAL_SOLID)) != 0
    g = -(-sx // 4) * 4

    def group_any(m):
        mm = np.zeros((sz, sy, g), bool)
        mm[:, :, :sx] = m
        return np.repeat(mm.reshape(sz, sy, g // 4, 4).any(-1), 4, axis=-1)[:, :, :sx]

    weighted, active = group_any(part), group_any(fluid)
    AX, AY, AZ = np.pad(ax, 1), np.pad(ay, 1), np.pad(az, 1)
    W = [ax, AX[1:-1, 1:-1, 2:], ay, AY[1:-1, 2:, 1:-1], az, AZ[2:, 1:-1, 1:-1]]
    hh, om = f32(h), f32(omega)
    om1 = f32(1.0) - om
    dho = dinv * (om / hh)
    src = x.copy()
    dst = np.zeros_like(x) if tmp is None else np.asarray(tmp, f32).reshape(fl.shape).copy()
    for _ in range(iters):
        X = np.pad(src, 1)
        F = [X[1:-1, 1:-1, :-2], X[1:-1, 1:-1, 2:], X[1:-1, :-2, 1:-1], X[1:-1, 2:, 1:-1], X[:-2, 1:-1, 1:-1],
             X[2:, 1:-1, 1:-1]]
        Fw = [np.where(weighted, Fi * Wi, Fi).astype(f32) for Fi, Wi in zip(F, W)]
        S = ((Fw[0] + Fw[1]) + ((Fw[2] + Fw[3]) + (Fw[4] + Fw[5]))) * hh
        t = b + S
        Y = (om1.astype(f64) * src.astype(f64) + (t * dho).astype(f64)).astype(f32)
        Y = np.where(fluid, Y, f32(0.0))
        dst = np.where(active, Y, dst).astype(f32)
        src, dst = dst, src
    return src
