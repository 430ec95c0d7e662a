"""Python host side of the msbg_gpu C ABI (include/msbg_gpu.h), through ctypes.

``MultiresSparseGrid`` mirrors the method names and argument meaning of the
reference's MSBG::MultiresSparseGrid for the hot path (src/msbg.h:828-3797):
``create``, ``regularizeRefinementMap``, ``setRefinementMap``,
``applyChannelPdeFast`` ... so that tests and tools read like code written
against the reference.  Every call goes to the CUDA library; there is no CPU
fallback: loading fails loudly when ``libmsbg_gpu.so`` is missing.
"""
from __future__ import annotations

import ctypes as C
import os
import struct
from dataclasses import dataclass

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libmsbg_gpu.so")

OK = 0
ERR_ARG, ERR_CUDA, ERR_NOMEM, ERR_STATE, ERR_CAPACITY, ERR_NONFINITE, ERR_DIVERGED, ERR_UNSUPPORTED, ERR_TIMEOUT = \
    -1, -2, -3, -4, -5, -6, -7, -8, -9
ERR_IO = -10

F32, U16, F16, F64 = 0, 1, 2, 3
NP_STORAGE = {F32: np.float32, U16: np.uint16, F16: np.float16, F64: np.float64}

OPT_8_COLOR_SCHEME = 1 << 29
PDE_MEAN_CURVATURE = 4
LAPL_MCF_8COLOR = -(PDE_MEAN_CURVATURE + OPT_8_COLOR_SCHEME)
SWEEP_EXACT, SWEEP_FAST = 0, 1
# interpolation options (src/sbg.h:140-170) and the uint16 render-density scale
IP_CORNER, IP_CHKBLK, IP_BC_DIRICHLET, IP_BC_DIRICHLET_OLD = 1 << 0, 1 << 5, 1 << 13, 1 << 14
IP_NO_BORDER_CHECK, IP_RENDER_DENS = 1 << 15, 1 << 18
# halo fill options (OPT_BC_NEUMANN, OPT_BC_COARSE_LEVEL; src/msbg.h:101-131) and the
# block states of a level grid
BC_NEUMANN, BC_COARSE_LEVEL = 1 << 10, 1 << 26
LBLK_EMPTY, LBLK_FULL, LBLK_NONE = -1, -2, -3

# solver options: OPT_CALC_RESIDUAL (src/msbg.h:115); the tile smoother of msbg_gpu_relax
OPT_CALC_RESIDUAL, RELAX_TILES = 1 << 12, 1 << 31
CH_NULL = 0  # no channel (the reference's CH_NULL)

BLK_DOM_BORDER, BLK_COARSE_FINE, BLK_FINE_COARSE = 1 << 1, 1 << 2, 1 << 3
BLK_EXISTS, BLK_UNIFORM_EMPTY = 1 << 12, 1 << 13

# Every function the header declares, with its ctypes signature.
P, I, I64, F, D, SZ = C.c_void_p, C.c_int, C.c_int64, C.c_float, C.c_double, C.c_size_t
SIGNATURES = {
    "msbg_gpu_create": (I, [C.POINTER(P), I, I, I, I, I, I, I64]),
    "msbg_gpu_destroy": (I, [P]),
    "msbg_gpu_last_error": (C.c_char_p, [P]),
    "msbg_gpu_set_stream": (I, [P, P]),
    "msbg_gpu_get_info": (I, [P, P]),
    "msbg_gpu_synchronize": (I, [P]),
    "msbg_gpu_channel_create": (I, [P, I, I]),
    "msbg_gpu_mark_points": (I, [P, P, I64, F]),
    "msbg_gpu_levels_from_marks": (I, [P]),
    "msbg_gpu_levels_from_bands": (I, [P, P, I64, P, I]),
    "msbg_gpu_set_levels": (I, [P, P]),
    "msbg_gpu_regularize_refinement_map": (I, [P]),
    "msbg_gpu_set_refinement_map": (I, [P, D]),
    "msbg_gpu_get_levels": (I, [P, P]),
    "msbg_gpu_get_flags": (I, [P, P]),
    "msbg_gpu_get_active_blocks": (I, [P, P, I64, C.POINTER(I64)]),
    "msbg_gpu_get_slots": (I, [P, P]),
    "msbg_gpu_get_block_list": (I, [P, I, I, P, C.POINTER(I64)]),
    "msbg_gpu_dist_fine_coarse": (I, [P, I, P, P, I64, C.POINTER(I64)]),
    "msbg_gpu_upload_payload": (I, [P, I, P]),
    "msbg_gpu_download_payload": (I, [P, I, P]),
    "msbg_gpu_payload_ptr": (I, [P, I, C.POINTER(P)]),
    "msbg_gpu_fill": (I, [P, I, D]),
    "msbg_gpu_splat": (I, [P, P, I64, F, F]),
    "msbg_gpu_splat_finalize": (I, [P, F, F]),
    "msbg_gpu_particles_per_block": (I, [P, P, I64, P, P, C.POINTER(I64)]),
    "msbg_gpu_apply_channel_pde_fast": (I, [P, I, I, I, P, I64, I, I, F, F, F, I, F, F, F, P, F, F, F, F, F, I, P,
                                            I, I]),
    "msbg_gpu_surface_job": (I, [P, P, I64, F, F, P, I, I, I, F, I, P, SZ, C.POINTER(I64)]),
    "msbg_gpu_surface_job_stages": (I, [P, P, I, C.POINTER(I)]),
    "msbg_gpu_surface_job_submit": (I, [P, P, I64, F, F, P, I, I, I, F, I, P, SZ, C.POINTER(I64)]),
    "msbg_gpu_surface_job_wait": (I, [P]),
    "msbg_gpu_event_record": (I, [P, I]),
    "msbg_gpu_event_elapsed": (I, [P, I, I, C.POINTER(F)]),
    "msbg_gpu_launch_count": (I64, [P]),
    "msbg_gpu_host_alloc": (I, [C.POINTER(P), SZ]),
    "msbg_gpu_host_free": (I, [P]),
    "msbg_gpu_device_alloc": (I, [C.POINTER(P), SZ]),
    "msbg_gpu_device_free": (I, [P]),
    "msbg_gpu_copy_h2d": (I, [P, P, P, SZ]),
    "msbg_gpu_copy_d2h": (I, [P, P, P, SZ]),
    "msbg_gpu_copy_d2d": (I, [P, P, P, SZ]),
    "msbg_gpu_warmnet_param_count": (I, [C.POINTER(I), C.POINTER(I)]),
    "msbg_gpu_warmnet_set_weights": (I, [P, P, P, I]),
    "msbg_gpu_warmnet_get_weights": (I, [P, P, P]),
    "msbg_gpu_warmnet_predict": (I, [P, I, I]),
    "msbg_gpu_warmnet_set_loss": (I, [P, I]),
    "msbg_gpu_batch_set_volumes": (I, [P, P, I]),
    "msbg_gpu_batch_mgpcg_solve": (I, [P, I, I, D, I, I, P, P, P, C.POINTER(F)]),
    "msbg_gpu_warmnet_loss_grad": (I, [P, I, I, C.POINTER(D), P, P]),
    "msbg_gpu_warmnet_train_step": (I, [P, P, P, F, C.POINTER(D)]),
    "msbg_gpu_assign_slots_noalloc": (I, [P, I64, P, P, P, P]),
    "msbg_gpu_poisson_set_coefficients": (I, [P, I, I, I, I]),
    "msbg_gpu_poisson_procedural_coefficients": (I, [P, C.c_uint32, I, I, I, I]),
    "msbg_gpu_multiply_laplacian": (I, [P, C.c_uint, I, I, I, F, I, C.POINTER(D), P, I64]),
    "msbg_gpu_relax": (I, [P, I, I, I, I, I, I, I, C.c_uint, P, I64]),
    "msbg_gpu_set_relax_params": (I, [P, F, I]),
    "msbg_gpu_downsample_channel": (I, [P, I, P, I]),
    "msbg_gpu_interpolate": (I, [P, I, P, I64, P, I]),
    "msbg_gpu_level_grid_set": (I, [P, I, I, I, P, P, I64, C.c_float, C.c_float]),
    "msbg_gpu_level_grid_bind": (I, [P, I, I, I, P, P, C.c_float, C.c_float]),
    "msbg_gpu_render": (I, [P, I, I, I, P, P]),
    "msbg_gpu_sort_block_list_morton": (I, [P, P, I64]),
    "msbg_gpu_save": (I, [P, C.c_char_p, P, I]),
    "msbg_gpu_load": (I, [C.POINTER(P), C.c_char_p]),
    "msbg_gpu_fill_halo_blocks": (I, [P, I, I, P, I64, I, I, P, C.POINTER(I64)]),
    "msbg_gpu_restrict_level_blocks": (I, [P, I, I, P, I64, I, P, C.POINTER(I64)]),
    "msbg_gpu_multiply_laplacian_levels": (I, [P, C.c_uint, I, I, I, I, P, I64, P, C.POINTER(D), C.POINTER(I64)]),
    "msbg_gpu_relax_levels": (I, [P, I, I, I, I, P, I64, C.POINTER(I64)]),
    "msbg_gpu_multiply_laplacian_dense": (I, [P, C.c_uint, I, I, I, I, P, P, P, P, P, P, P, P]),
    "msbg_gpu_relax_dense": (I, [P, I, I, I, I, I, P, P, P, P, P, P, P, P]),
    "msbg_gpu_level_flags_set": (I, [P, I, I, P, P, I64, C.c_uint16, C.c_uint16]),
    "msbg_gpu_fill_halo_blocks3": (I, [P, I, I, I, P, I64, P, P, C.POINTER(I64)]),
    "msbg_gpu_diag_wait_timeout": (I, [P, I]),
    "msbg_gpu_vcycle": (I, [P, I, I]),
    "msbg_gpu_dot": (I, [P, I, I, I, P, I64, C.POINTER(D)]),
    "msbg_gpu_axpby": (I, [P, D, I, D, I, I, I, P, I64]),
    "msbg_gpu_axpby_combined": (I, [P, D, D, I, I, I, P, I64]),
    "msbg_gpu_mgpcg_solve": (I, [P, I, I, D, I, C.POINTER(I), C.POINTER(D)]),
    "msbg_gpu_mg_info": (I, [P, C.POINTER(I), P, I]),
    "msbg_gpu_poisson_tuning": (I, [P, I, P, I, C.POINTER(I)]),
    "msbg_gpu_poisson_release_work": (I, [P]),
    "msbg_gpu_poisson_set_params": (I, [P, I, I, I, I]),
    "msbg_gpu_mgpcg_solve_mixed": (I, [P, I, I, D, I, D, I, C.POINTER(I), C.POINTER(I), C.POINTER(D)]),
}

_lib = None


class Info(C.Structure):
    _fields_ = [("sx", C.c_int32), ("sy", C.c_int32), ("sz", C.c_int32), ("bsx", C.c_int32),
                ("nbx", C.c_int32), ("nby", C.c_int32), ("nbz", C.c_int32), ("nLevels", C.c_int32),
                ("nBlocks", C.c_int64), ("nActive", C.c_int64), ("capacityBlocks", C.c_int64),
                ("blocksPerLevel", C.c_int64 * 8), ("colorCount", C.c_int32 * 8),
                ("nActParticles", C.c_int64), ("nAborted", C.c_int64)]


class MsbgGpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"msbg_gpu error {code}: {msg}")
        self.code = code


def load_library(path: str = LIB_PATH) -> C.CDLL:
    """Load libmsbg_gpu.so and bind every ABI function (raises if it is missing)."""
    global _lib
    if _lib is not None and path == LIB_PATH:
        return _lib
    if not os.path.isfile(path):
        raise OSError(f"{path} not found: run `python -m msbg_gb300.build` (the GPU path has no fallback)")
    L = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    if path == LIB_PATH:
        _lib = L
    return L


def _ptr(a) -> C.c_void_p | None:
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data_as(C.c_void_p)
    return C.c_void_p(int(a))


@dataclass
class DeviceBuffer:
    """Raw device allocation owned by Python (freed on close/GC)."""
    ptr: int
    nbytes: int

    @classmethod
    def alloc(cls, nbytes: int) -> "DeviceBuffer":
        p = C.c_void_p()
        if load_library().msbg_gpu_device_alloc(C.byref(p), max(int(nbytes), 1)) != OK:
            raise MsbgGpuError(ERR_NOMEM, "device alloc")
        return cls(p.value, int(nbytes))

    def free(self):
        if self.ptr:
            load_library().msbg_gpu_device_free(C.c_void_p(self.ptr))
            self.ptr = 0

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


# the demo's camera (src/msbg_demo.cpp:123-127) and surface colour (src/msbg_demo.cpp:150)
DEMO_CAMERA = {"pos": (0.5, 0.8, 0.7), "look_at": (0.5, 0.5, 0.5), "sun": (0.5, 5.0, 5.0),
               "color": (0.8, 0.6, 0.4), "zoom": 1.0}


class Camera(C.Structure):
    """msbg_gpu_camera; the demo passes float values, so they are rounded to float first."""
    _fields_ = [("pos", C.c_double * 3), ("lookAt", C.c_double * 3), ("sun", C.c_double * 3),
                ("color", C.c_double * 3), ("zoom", C.c_double)]

    @classmethod
    def of(cls, cam: dict) -> "Camera":
        f = lambda v: (C.c_double * 3)(*[float(np.float32(x)) for x in v])  # noqa: E731
        return cls(f(cam["pos"]), f(cam["look_at"]), f(cam["sun"]), f(cam["color"]), float(np.float32(cam["zoom"])))


CKPT_HEADER = struct.Struct("<8sII6i2qQ")  # magic, version, header bytes, sx sy sz bsx nLevels nChans,
CKPT_CHANNEL = struct.Struct("<iiqQ")      # nBlocks nActive, levels checksum; chan storage bytes checksum


def read_checkpoint_index(path: str) -> dict:
    """The header and channel records of a checkpoint file (msbg_gpu_save), without payloads."""
    with open(path, "rb") as f:
        magic, version, hbytes, sx, sy, sz, bsx, n_levels, n_chans, n_blocks, n_active, lhash = \
            CKPT_HEADER.unpack(f.read(CKPT_HEADER.size))
        if magic != b"MSBGCKP1" or version != 1 or hbytes != CKPT_HEADER.size:
            raise ValueError(f"{path}: not a version-1 checkpoint")
        f.seek(n_blocks, 1)
        chans = []
        for _ in range(n_chans):
            chan, storage, nbytes, chash = CKPT_CHANNEL.unpack(f.read(CKPT_CHANNEL.size))
            chans.append({"chan": chan, "storage": storage, "bytes": nbytes, "checksum": chash,
                          "offset": f.tell()})
            f.seek(nbytes, 1)
    return {"sx": sx, "sy": sy, "sz": sz, "bsx": bsx, "n_levels": n_levels, "n_blocks": n_blocks,
            "n_active": n_active, "levels_checksum": lhash, "channels": chans}


class MultiresSparseGrid:
    """GPU MultiresSparseGrid over one context of the C ABI."""

    def __init__(self, sx: int, sy: int, sz: int, bsx: int, n_levels: int = 3, storage: int = F32,
                 capacity_blocks: int = 0):
        self.L = load_library()
        h = C.c_void_p()
        rc = self.L.msbg_gpu_create(C.byref(h), sx, sy, sz, bsx, n_levels, storage, capacity_blocks)
        if rc != OK:
            raise MsbgGpuError(rc, "msbg_gpu_create failed")
        self.h = h
        self.sx, self.sy, self.sz, self.bsx, self.n_levels = sx, sy, sz, bsx, n_levels
        self.nbx, self.nby, self.nbz = sx // bsx, sy // bsx, sz // bsx
        self.n_blocks = self.nbx * self.nby * self.nbz
        self.storage = {0: storage}

    # reference: MultiresSparseGrid::create (src/msbg.h:834-852)
    @classmethod
    def create(cls, name: str, sx: int, sy: int, sz: int, blockSize0: int, nLevels: int = 3,
               storage: int = F32, capacity_blocks: int = 0) -> "MultiresSparseGrid":
        return cls(sx, sy, sz, blockSize0, nLevels, storage, capacity_blocks)

    # checkpoint files (no reference counterpart: the reference has no grid file format)
    def save(self, path: str, chans=(0,)):
        """Geometry, level map and the payload of channels chans to a checkpoint file."""
        ch = np.ascontiguousarray(list(chans), np.int32)
        self._check(self.L.msbg_gpu_save(self.h, os.fsencode(path), _ptr(ch), len(ch)))

    @classmethod
    def load(cls, path: str) -> "MultiresSparseGrid":
        """A grid restored from a checkpoint file (layout rebuilt from its level map)."""
        L = load_library()
        h = C.c_void_p()
        rc = L.msbg_gpu_load(C.byref(h), os.fsencode(path))
        if rc != OK:
            raise MsbgGpuError(rc, f"msbg_gpu_load failed for {path}")
        g = cls.__new__(cls)
        g.L, g.h = L, h
        info = Info()
        g._check(L.msbg_gpu_get_info(h, C.byref(info)))
        g.sx, g.sy, g.sz, g.bsx, g.n_levels = info.sx, info.sy, info.sz, info.bsx, info.nLevels
        g.nbx, g.nby, g.nbz = info.nbx, info.nby, info.nbz
        g.n_blocks = g.nbx * g.nby * g.nbz
        g.storage = {0: F32}
        for rec in read_checkpoint_index(path)["channels"]:
            g.storage[rec["chan"]] = rec["storage"]
        return g

    def _check(self, rc: int):
        if rc != OK:
            raise MsbgGpuError(rc, self.L.msbg_gpu_last_error(self.h).decode(errors="replace"))

    def close(self):
        if getattr(self, "h", None):
            self.L.msbg_gpu_destroy(self.h)
            self.h = None

    destroy = close

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- info ---------------------------------------------------------------------
    def info(self) -> Info:
        inf = Info()
        self._check(self.L.msbg_gpu_get_info(self.h, C.byref(inf)))
        return inf

    def nBlocks(self) -> int:
        return self.n_blocks

    def set_stream(self, stream_handle: int):
        self._check(self.L.msbg_gpu_set_stream(self.h, C.c_void_p(stream_handle)))

    def synchronize(self):
        self._check(self.L.msbg_gpu_synchronize(self.h))

    def launch_count(self) -> int:
        return int(self.L.msbg_gpu_launch_count(self.h))

    # ---- device memory --------------------------------------------------------------
    def to_device(self, a: np.ndarray) -> DeviceBuffer:
        a = np.ascontiguousarray(a)
        p = C.c_void_p()
        if self.L.msbg_gpu_device_alloc(C.byref(p), max(a.nbytes, 1)) != OK:
            raise MsbgGpuError(ERR_NOMEM, "device alloc")
        buf = DeviceBuffer(p.value, a.nbytes)
        if a.nbytes:
            self._check(self.L.msbg_gpu_copy_h2d(self.h, C.c_void_p(buf.ptr), _ptr(a), a.nbytes))
        self.synchronize()
        return buf

    # ---- layout -----------------------------------------------------------------------
    def channel_create(self, chan: int, storage: int):
        self._check(self.L.msbg_gpu_channel_create(self.h, chan, storage))
        self.storage[chan] = storage

    def mark_points(self, d_pts: DeviceBuffer, n: int, r_scan: float):
        self._check(self.L.msbg_gpu_mark_points(self.h, C.c_void_p(d_pts.ptr), n, r_scan))

    def levels_from_marks(self):
        self._check(self.L.msbg_gpu_levels_from_marks(self.h))

    def levels_from_bands(self, d_pts: DeviceBuffer, n: int, bands):
        b = np.ascontiguousarray(bands, np.float32)
        self._check(self.L.msbg_gpu_levels_from_bands(self.h, C.c_void_p(d_pts.ptr), n, _ptr(b), len(b)))

    def set_levels(self, levels: np.ndarray):
        lv = np.ascontiguousarray(levels, np.int32)
        self._check(self.L.msbg_gpu_set_levels(self.h, _ptr(lv)))

    # reference: regularizeRefinementMap (src/msbg.h:897-901)
    def regularizeRefinementMap(self):
        self._check(self.L.msbg_gpu_regularize_refinement_map(self.h))

    # reference: setRefinementMap (src/msbg.h:903-908) + the demo's allocation loop
    def setRefinementMap(self, fill_value: float = 1.0):
        self._check(self.L.msbg_gpu_set_refinement_map(self.h, fill_value))

    def levels(self) -> np.ndarray:
        out = np.empty(self.n_blocks, np.int8)
        self._check(self.L.msbg_gpu_get_levels(self.h, _ptr(out)))
        return out

    def flags(self) -> np.ndarray:
        out = np.empty(self.n_blocks, np.uint16)
        self._check(self.L.msbg_gpu_get_flags(self.h, _ptr(out)))
        return out

    def active_blocks(self) -> np.ndarray:
        n = C.c_int64()
        self._check(self.L.msbg_gpu_get_active_blocks(self.h, None, 0, C.byref(n)))
        out = np.empty(n.value, np.int32)
        self._check(self.L.msbg_gpu_get_active_blocks(self.h, _ptr(out), n.value, C.byref(n)))
        return out

    def slots(self) -> np.ndarray:
        out = np.empty(self.n_blocks, np.int32)
        self._check(self.L.msbg_gpu_get_slots(self.h, _ptr(out)))
        return out

    # ---- data ---------------------------------------------------------------------------
    def payload(self, chan: int = 0) -> np.ndarray:
        n = self.info().nActive
        out = np.empty((n, self.bsx ** 3), NP_STORAGE[self.storage[chan]])
        self._check(self.L.msbg_gpu_download_payload(self.h, chan, _ptr(out)))
        return out

    def upload_payload(self, data: np.ndarray, chan: int = 0):
        a = np.ascontiguousarray(data, NP_STORAGE[self.storage[chan]])
        self._check(self.L.msbg_gpu_upload_payload(self.h, chan, _ptr(a)))
        self.synchronize()

    def payload_ptr(self, chan: int = 0) -> int:
        p = C.c_void_p()
        self._check(self.L.msbg_gpu_payload_ptr(self.h, chan, C.byref(p)))
        return p.value or 0

    def fill(self, value: float, chan: int = 0):
        self._check(self.L.msbg_gpu_fill(self.h, chan, value))

    def splat(self, d_pts: DeviceBuffer, n: int, r_particle: float = 2.0, nb_dist: float = 2.0):
        self._check(self.L.msbg_gpu_splat(self.h, C.c_void_p(d_pts.ptr), n, r_particle, nb_dist))

    def splat_finalize(self, r_particle: float = 2.0, nb_dist: float = 2.0):
        self._check(self.L.msbg_gpu_splat_finalize(self.h, r_particle, nb_dist))

    def particles_per_block(self, d_pts: DeviceBuffer, n: int):
        """The demo's particlesPerBlock as CSR: (offsets int64 [nBlocks+1], point indices
        int32 [count]); the order inside a list is unspecified."""
        off_d = DeviceBuffer.alloc((self.n_blocks + 1) * 8)
        idx_d = DeviceBuffer.alloc(max(n, 1) * 4)
        cnt = C.c_int64()
        try:
            self._check(self.L.msbg_gpu_particles_per_block(self.h, C.c_void_p(d_pts.ptr), n, C.c_void_p(off_d.ptr),
                                                            C.c_void_p(idx_d.ptr), C.byref(cnt)))
            off = np.empty(self.n_blocks + 1, np.int64)
            idx = np.empty(cnt.value, np.int32)
            self._check(self.L.msbg_gpu_copy_d2h(self.h, _ptr(off), C.c_void_p(off_d.ptr), off.nbytes))
            if cnt.value:
                self._check(self.L.msbg_gpu_copy_d2h(self.h, _ptr(idx), C.c_void_p(idx_d.ptr), idx.nbytes))
            self.synchronize()
        finally:
            off_d.free()
            idx_d.free()
        return off, idx

    # reference: applyChannelPdeFast<T> (src/msbg.h:2150-2172); the reference's
    # (chPhi, laplTyp, doConstrZeroOne, numIter, timeStep, anisDiffAlpha) subset
    def _block_list(self, blockList):
        """(device pointer, count, buffer to keep alive) of a block list: None (all value
        blocks), a DeviceBuffer of int32 ids, or host ids (copied to the device)."""
        if blockList is None:
            return None, 0, None
        if isinstance(blockList, DeviceBuffer):
            return C.c_void_p(blockList.ptr), blockList.nbytes // 4, blockList
        a = np.ascontiguousarray(blockList, np.int32).ravel()
        buf = self.to_device(a if a.size else np.zeros(1, np.int32))
        return C.c_void_p(buf.ptr), a.size, buf

    # reference: applyChannelPdeFast<T> (src/msbg.h:2150-2172), the same arguments in the same
    # order (msbgVel / veldep_fit must stay None), plus the kernel variant
    def applyChannelPdeFast(self, chPhi: int, chTmp: int = CH_NULL, chTmp2: int = CH_NULL, blockList=None,
                            laplTyp: int = LAPL_MCF_8COLOR, doConstrZeroOne: int = 1, densThr: float = 0.0,
                            densThrTol1: float = 0.0, densThrTol2: float = 0.0, numIter: int = 1,
                            gridSpacing: float = 1.0, timeStep: float = 0.025, velMagThr: float = 0.0,
                            msbgVel=None, lambda_: float = 0.0, lambdaSDF: float = 0.0, taubinStrength: float = 0.0,
                            redist: float = 0.0, anisDiffAlpha: float = 0.0, veldep_on: int = 0, veldep_fit=None,
                            visOpt: int = 0, variant: int = SWEEP_EXACT):
        lp, ln, keep = self._block_list(blockList)
        self._check(self.L.msbg_gpu_apply_channel_pde_fast(
            self.h, chPhi, chTmp, chTmp2, lp, ln, laplTyp, int(doConstrZeroOne), densThr, densThrTol1, densThrTol2,
            numIter, gridSpacing, timeStep, velMagThr, msbgVel, lambda_, lambdaSDF, taubinStrength, redist,
            anisDiffAlpha, veldep_on, veldep_fit, visOpt, variant))
        if keep is not None and keep is not blockList:
            self.synchronize()

    def surface_job(self, pts: np.ndarray, r_particle=2.0, nb_dist=2.0, bands=None,
                    laplTyp=LAPL_MCF_8COLOR, numIter=20, timeStep=0.1, variant=SWEEP_EXACT,
                    out: np.ndarray | None = None):
        """Whole pipeline from host points to the host payload (the e2e entry point)."""
        pts = np.ascontiguousarray(pts, np.float32).reshape(-1, 3)
        b = None if bands is None else np.ascontiguousarray(bands, np.float32)
        n_act = C.c_int64()
        cap = 0 if out is None else out.nbytes
        self._check(self.L.msbg_gpu_surface_job(
            self.h, _ptr(pts), len(pts), r_particle, nb_dist, _ptr(b), 0 if b is None else len(b),
            laplTyp, numIter, timeStep, variant, _ptr(out), cap, C.byref(n_act)))
        return n_act.value

    def surface_job_submit(self, pts: np.ndarray, out: np.ndarray, r_particle=2.0, nb_dist=2.0, bands=None,
                           laplTyp=LAPL_MCF_8COLOR, numIter=20, timeStep=0.1, variant=SWEEP_EXACT) -> int:
        """The streaming form: queues the job (out is complete after surface_job_wait); returns
        its value-block count.  pts may be reused when the call returns."""
        pts = np.ascontiguousarray(pts, np.float32).reshape(-1, 3)
        b = None if bands is None else np.ascontiguousarray(bands, np.float32)
        n_act = C.c_int64()
        self._check(self.L.msbg_gpu_surface_job_submit(
            self.h, _ptr(pts), len(pts), r_particle, nb_dist, _ptr(b), 0 if b is None else len(b),
            laplTyp, numIter, timeStep, variant, _ptr(out), out.nbytes, C.byref(n_act)))
        return n_act.value

    def surface_job_wait(self):
        self._check(self.L.msbg_gpu_surface_job_wait(self.h))

    # ---- Poisson solve (src/msbg3.cpp, src/msbg.cpp:4524-4872) --------------------------
    def poisson_set_coefficients(self, cx: int, cy: int, cz: int, diag: int):
        self._check(self.L.msbg_gpu_poisson_set_coefficients(self.h, cx, cy, cz, diag))

    def poisson_procedural_coefficients(self, seed: int, cx=-1, cy=-1, cz=-1, diag=-1):
        self._check(self.L.msbg_gpu_poisson_procedural_coefficients(self.h, seed, cx, cy, cz, diag))

    # reference: multiplyLaplacianMatrixOpt(options, levelMg, chanX, chanB, kap, chanDstY,
    # pDotprod, blockList) (src/msbg.h:3167-3176); returns sum(Y X) when withDotprod
    SURFACE_JOB_STAGES = ("upload", "layout", "splat", "finalize", "sweeps", "download")

    def surface_job_stages(self) -> dict:
        """Stream milliseconds of the stages of the last surface_job."""
        ms = (C.c_float * 8)()
        n = C.c_int()
        self._check(self.L.msbg_gpu_surface_job_stages(self.h, ms, 8, C.byref(n)))
        return {k: float(ms[i]) for i, k in enumerate(self.SURFACE_JOB_STAGES[: n.value])}

    def multiplyLaplacianMatrixOpt(self, options: int, levelMg: int, chanX: int, chanB: int, kap: float,
                                   chanDstY: int, withDotprod: bool = False, blockList=None):
        lp, ln, keep = self._block_list(blockList)
        dot = C.c_double()
        self._check(self.L.msbg_gpu_multiply_laplacian(self.h, options, levelMg, chanX, chanB, kap, chanDstY,
                                                       C.byref(dot) if withDotprod else None, lp, ln))
        if keep is not None and keep is not blockList:
            self.synchronize()
        return dot.value if withDotprod else None

    def multiplyLaplacianMatrix(self, chanX: int, chanB: int, chanDstY: int, calcResidual: bool = False):
        """Y = A X (or B - A X) over all value blocks."""
        self.multiplyLaplacianMatrixOpt(OPT_CALC_RESIDUAL if calcResidual else 0, 0, chanX, chanB, 0.0, chanDstY)

    # reference: relax(boundaryZoneOnly, reverseOrder, levelMg, chanX, chanB, chanTmp, nIter,
    # options) (src/msbg.h:3269-3277); blockList stands in for the member list _blocksRelax
    def relax(self, boundaryZoneOnly: int, reverseOrder: int, levelMg: int, chanX: int, chanB: int,
              chanTmp: int, nIter: int, options: int = 0, blockList=None):
        lp, ln, keep = self._block_list(blockList)
        self._check(self.L.msbg_gpu_relax(self.h, int(boundaryZoneOnly), int(reverseOrder), levelMg, chanX, chanB,
                                          chanTmp, nIter, options, lp, ln))
        if keep is not None and keep is not blockList:
            self.synchronize()

    def relax_tiles(self, chanX: int, chanB: int, nIter: int, reverseOrder: bool = False):
        """nIter passes of the multigrid's tile smoother (relax with RELAX_TILES)."""
        self.relax(0, int(reverseOrder), 0, chanX, chanB, CH_NULL, nIter, RELAX_TILES)

    def set_relax_params(self, omega: float = 6.0 / 7.0, block_iter: int = 5):
        self._check(self.L.msbg_gpu_set_relax_params(self.h, omega, block_iter))

    def vcycle(self, chanX: int, chanB: int):
        self._check(self.L.msbg_gpu_vcycle(self.h, chanX, chanB))

    def diag_wait_timeout(self, polls: int = 1000):
        """Runs the bounded-wait failure path once (raises MsbgGpuError, code ERR_TIMEOUT)."""
        self._check(self.L.msbg_gpu_diag_wait_timeout(self.h, polls))

    def downsampleFloatChannelNew(self, chSrc: int, simpleAverage: bool = False) -> np.ndarray:
        """Restriction of channel chSrc to the next coarser level, per value block:
        [nActive][(bs/2)^3] float32 (src/msbg4.cpp:1035-1379)."""
        cb = self.bsx // 2
        n = self.info().nActive * cb ** 3
        out = np.empty(n, np.float32)
        buf = DeviceBuffer.alloc(max(n, 1) * 4)
        try:
            self._check(self.L.msbg_gpu_downsample_channel(self.h, chSrc, C.c_void_p(buf.ptr), int(simpleAverage)))
            if n:
                self._check(self.L.msbg_gpu_copy_d2h(self.h, _ptr(out), C.c_void_p(buf.ptr), n * 4))
            self.synchronize()
        finally:
            buf.free()
        return out.reshape(-1, cb ** 3)

    def interpolate_device(self, chan: int, d_pts: DeviceBuffer, n: int, d_out: DeviceBuffer,
                           opt: int = 0):
        """Trilinear interpolation of channel chan at n device points (xyz float32) into
        n device floats; asynchronous on the context's stream."""
        self._check(self.L.msbg_gpu_interpolate(self.h, chan, C.c_void_p(d_pts.ptr), n,
                                                C.c_void_p(d_out.ptr), opt))

    def interpolate(self, chan: int, pts: np.ndarray, opt: int = 0) -> np.ndarray:
        """Per-point interpolateFloatFast / interpolateUint16ToFloatFast (src/sbg.h:4623-4792,
        src/sbg.h:4920-5032); with IP_RENDER_DENS, interpolateRenderDensity
        (src/msbg.h:478-484).  Host points in, host float32 values out."""
        pts = np.ascontiguousarray(pts, np.float32).reshape(-1, 3)
        n = pts.shape[0]
        out = np.empty(n, np.float32)
        dp = DeviceBuffer.alloc(max(n, 1) * 12)
        do = DeviceBuffer.alloc(max(n, 1) * 4)
        try:
            if n:
                self._check(self.L.msbg_gpu_copy_h2d(self.h, C.c_void_p(dp.ptr), _ptr(pts), n * 12))
            self.interpolate_device(chan, dp, n, do, opt)
            if n:
                self._check(self.L.msbg_gpu_copy_d2h(self.h, _ptr(out), C.c_void_p(do.ptr), n * 4))
            self.synchronize()
        finally:
            dp.free()
            do.free()
        return out

    # ---- multi-level channels: HaloBlockSet::fillHaloBlock_ (src/halo.cpp:266-479) ----------
    def level_grid_set(self, lchan: int, level: int, storage: int, state: np.ndarray,
                       payload: np.ndarray | None, empty_value: float = 0.0, full_value: float = 1.0):
        """Resolution level `level` of level channel lchan: per-block states (>= 0 payload
        index, LBLK_EMPTY / LBLK_FULL / LBLK_NONE) and the payload [n][(bsx>>level)^3]."""
        st = np.ascontiguousarray(state, np.int32)
        n_data = 0 if payload is None else int(np.asarray(payload).reshape(-1).size // ((self.bsx >> level) ** 3))
        pay = None if payload is None else np.ascontiguousarray(payload)
        self._check(self.L.msbg_gpu_level_grid_set(self.h, lchan, level, storage, _ptr(st),
                                                   None if pay is None else _ptr(pay), n_data,
                                                   empty_value, full_value))

    def level_grid_bind(self, lchan: int, level: int, storage: int, d_state: int, d_payload: int,
                        empty_value: float = 0.0, full_value: float = 1.0):
        """Binds device arrays (pointers) as level `level` of level channel lchan, no copy."""
        self._check(self.L.msbg_gpu_level_grid_bind(self.h, lchan, level, storage, C.c_void_p(d_state),
                                                    C.c_void_p(d_payload), empty_value, full_value))

    def fill_halo_blocks_device(self, lchan: int, level: int, d_bids: DeviceBuffer, n: int, halo: int,
                                opt: int, d_out: DeviceBuffer, count_skipped: bool = False) -> int:
        """fillHaloBlock_ of n listed blocks (device int32 bids) into d_out
        ([n][(bs+2h)^3] floats); returns the skipped count when asked (synchronizes)."""
        sk = C.c_int64(-1)
        self._check(self.L.msbg_gpu_fill_halo_blocks(self.h, lchan, level, C.c_void_p(d_bids.ptr), n, halo,
                                                     opt, C.c_void_p(d_out.ptr),
                                                     C.byref(sk) if count_skipped else None))
        return int(sk.value)

    def fill_halo_blocks(self, lchan: int, level: int, bids: np.ndarray, halo: int, opt: int):
        """Host wrapper: (halo boxes float32 [n][(bs+2h)^3], skipped count)."""
        bids = np.ascontiguousarray(bids, np.int32)
        n = len(bids)
        hs = (self.bsx >> max(level, 0)) + 2 * max(halo, 0)  # the call itself rejects bad values
        out = np.empty((n, hs ** 3), np.float32)
        db = self.to_device(bids)
        do = DeviceBuffer.alloc(max(out.nbytes, 4))
        try:
            sk = self.fill_halo_blocks_device(lchan, level, db, n, halo, opt, do, count_skipped=True)
            if n:
                self._check(self.L.msbg_gpu_copy_d2h(self.h, _ptr(out), C.c_void_p(do.ptr), out.nbytes))
            self.synchronize()
        finally:
            db.free()
            do.free()
        return out, sk

    # reference: sortBlockListMorton (src/msbg2.cpp:46-58)
    def sortBlockListMorton(self, bids: np.ndarray) -> np.ndarray:
        """The block list in Morton order of the block coordinates (host in, host out)."""
        bids = np.ascontiguousarray(bids, np.int32)
        d = self.to_device(bids)
        try:
            self._check(self.L.msbg_gpu_sort_block_list_morton(self.h, C.c_void_p(d.ptr), len(bids)))
            out = np.empty_like(bids)
            if len(bids):
                self._check(self.L.msbg_gpu_copy_d2h(self.h, _ptr(out), C.c_void_p(d.ptr), out.nbytes))
            self.synchronize()
        finally:
            d.free()
        return out

    # ---- RDR::RaymarchRenderer (src/render.h:52-160, src/render.cpp:20-101) -------------
    def render_device(self, chan: int, width: int, height: int, cam: dict, d_rgb: DeviceBuffer):
        c = Camera.of(cam)
        self._check(self.L.msbg_gpu_render(self.h, chan, width, height, C.byref(c), C.c_void_p(d_rgb.ptr)))

    def render(self, chan: int, width: int, height: int, cam: dict | None = None) -> np.ndarray:
        """The iso-0.5 surface of channel chan seen from cam (default: the demo's camera):
        uint8 [height][width][3] RGB."""
        out = np.empty((height, width, 3), np.uint8)
        d = DeviceBuffer.alloc(out.nbytes)
        try:
            self.render_device(chan, width, height, DEMO_CAMERA if cam is None else cam, d)
            self._check(self.L.msbg_gpu_copy_d2h(self.h, _ptr(out), C.c_void_p(d.ptr), out.nbytes))
            self.synchronize()
        finally:
            d.free()
        return out

    LIST_EXISTING, LIST_FINE_COARSE = 0, 1

    def block_list(self, which: int, level: int = 0) -> np.ndarray:
        """setRefinementMap's _blocksExisting (LIST_EXISTING) or _blocksFineCoarsePerLevel[level]
        (LIST_FINE_COARSE), ascending."""
        d = DeviceBuffer.alloc(self.n_blocks * 4)
        n = C.c_int64()
        try:
            self._check(self.L.msbg_gpu_get_block_list(self.h, which, level, C.c_void_p(d.ptr), C.byref(n)))
            out = np.empty(n.value, np.int32)
            if n.value:
                self._check(self.L.msbg_gpu_copy_d2h(self.h, _ptr(out), C.c_void_p(d.ptr), out.nbytes))
            self.synchronize()
        finally:
            d.free()
        return out

    def dist_fine_coarse(self, level: int):
        """CH_DIST_FINECOARSE of one level: (state int32 [nBlocks], uint16 [n][(bsx>>level)^3])."""
        nv = (self.bsx >> level) ** 3
        ds = DeviceBuffer.alloc(self.n_blocks * 4)
        dd = DeviceBuffer.alloc(self.n_blocks * nv * 2)
        n = C.c_int64()
        try:
            self._check(self.L.msbg_gpu_dist_fine_coarse(self.h, level, C.c_void_p(ds.ptr), C.c_void_p(dd.ptr),
                                                         self.n_blocks, C.byref(n)))
            st = np.empty(self.n_blocks, np.int32)
            data = np.empty((n.value, nv), np.uint16)
            self._check(self.L.msbg_gpu_copy_d2h(self.h, _ptr(st), C.c_void_p(ds.ptr), st.nbytes))
            if n.value:
                self._check(self.L.msbg_gpu_copy_d2h(self.h, _ptr(data), C.c_void_p(dd.ptr), data.nbytes))
            self.synchronize()
        finally:
            ds.free()
            dd.free()
        return st, data

    def level_flags_set(self, fchan: int, level: int, state: np.ndarray, flags: np.ndarray | None,
                        empty_flags: int = 0, full_flags: int = 0):
        """Cell flags of resolution level `level` of flags channel fchan: per-block states and
        the uint16 flags [n][(bsx>>level)^3] (the reference's CH_CELL_FLAGS grid)."""
        st = np.ascontiguousarray(state, np.int32)
        f = None if flags is None else np.ascontiguousarray(flags, np.uint16)
        n_data = 0 if f is None else int(f.size // ((self.bsx >> level) ** 3))
        self._check(self.L.msbg_gpu_level_flags_set(self.h, fchan, level, _ptr(st), None if f is None else _ptr(f),
                                                    n_data, empty_flags, full_flags))

    # reference: HaloBlockSet::fillHaloBlock3 (src/halo.h:396-401), one call for a list
    def fillHaloBlock3(self, lchan: int, fchan: int, bids: np.ndarray, domain_bc, levelMg: int = 0):
        """The solver's halo of the listed blocks: (float32 [n][(bsx+2)^3], skipped count)."""
        bids = np.ascontiguousarray(bids, np.int32)
        hs = self.bsx + 2
        out = np.empty((len(bids), hs ** 3), np.float32)
        db = self.to_device(bids if len(bids) else np.zeros(1, np.int32))
        do = DeviceBuffer.alloc(max(out.nbytes, 4))
        dbc = np.ascontiguousarray(domain_bc, np.int32)
        sk = C.c_int64(-1)
        try:
            self._check(self.L.msbg_gpu_fill_halo_blocks3(self.h, lchan, fchan, levelMg, C.c_void_p(db.ptr), len(bids),
                                                          _ptr(dbc), C.c_void_p(do.ptr), C.byref(sk)))
            if len(bids):
                self._check(self.L.msbg_gpu_copy_d2h(self.h, _ptr(out), C.c_void_p(do.ptr), out.nbytes))
            self.synchronize()
        finally:
            db.free()
            do.free()
        return out, int(sk.value)

    def restrict_level_blocks(self, lchan: int, level: int, bids: np.ndarray, simple_average: bool = False):
        """downsampleFloatChannelNew for blocks of a level channel (cross-resolution halo):
        (float32 [n][(bs/2)^3], skipped count)."""
        bids = np.ascontiguousarray(bids, np.int32)
        cb = (self.bsx >> max(level, 0)) // 2
        out = np.empty((len(bids), max(cb, 1) ** 3), np.float32)
        db = self.to_device(bids)
        do = DeviceBuffer.alloc(max(out.nbytes, 4))
        sk = C.c_int64(-1)
        try:
            self._check(self.L.msbg_gpu_restrict_level_blocks(self.h, lchan, level, C.c_void_p(db.ptr), len(bids),
                                                              int(simple_average), C.c_void_p(do.ptr), C.byref(sk)))
            if len(bids):
                self._check(self.L.msbg_gpu_copy_d2h(self.h, _ptr(out), C.c_void_p(do.ptr), out.nbytes))
            self.synchronize()
        finally:
            db.free()
            do.free()
        return out, int(sk.value)

    # reference: multiplyLaplacianMatrixOpt (src/msbg3.cpp:1756-1912) on a multi-resolution
    # layout, one layout level per call
    def multiply_laplacian_levels(self, level: int, lchan_x: int, lchan_d: int, bids: np.ndarray,
                                  lchan_b: int = -1, residual: bool = False):
        """Y = A X (or B - A X) for the listed blocks of layout level `level`, operands in FP32
        level channels: (float32 [n][(bs)^3], sum(Y X) or None, skipped count)."""
        bids = np.ascontiguousarray(bids, np.int32)
        bs = self.bsx >> max(level, 0)
        out = np.empty((len(bids), max(bs, 1) ** 3), np.float32)
        db = self.to_device(bids)
        do = DeviceBuffer.alloc(max(out.nbytes, 4))
        dot, sk = C.c_double(), C.c_int64(-1)
        opt = OPT_CALC_RESIDUAL if residual else 0
        try:
            self._check(self.L.msbg_gpu_multiply_laplacian_levels(
                self.h, opt, level, lchan_x, lchan_b, lchan_d, C.c_void_p(db.ptr), len(bids), C.c_void_p(do.ptr),
                None if residual else C.byref(dot), C.byref(sk)))
            if len(bids):
                self._check(self.L.msbg_gpu_copy_d2h(self.h, _ptr(out), C.c_void_p(do.ptr), out.nbytes))
            self.synchronize()
        finally:
            db.free()
            do.free()
        return out, (None if residual else dot.value), int(sk.value)

    # reference: multiplyLaplacianMatrixOpt at a dense multigrid level (src/msbg3.cpp:166-403)
    def multiply_laplacian_dense(self, level_mg: int, flags, x, dinv, area_x, area_y, area_z, b=None,
                                 residual: bool = False, y_init=None) -> np.ndarray:
        """Host arrays [sz][sy][sx] in, Y (or B - A X) out; cells of skipped groups keep y_init
        (0 by default)."""
        fl = np.ascontiguousarray(flags, np.uint16)
        sz, sy, sx = fl.shape
        arrs = [np.ascontiguousarray(a, np.float32).reshape(fl.shape) for a in (x, dinv, area_x, area_y, area_z)]
        bb = np.ascontiguousarray(b if b is not None else np.zeros(fl.shape), np.float32).reshape(fl.shape)
        y = np.ascontiguousarray(np.zeros(fl.shape, np.float32) if y_init is None else y_init, np.float32).copy()
        bufs = [self.to_device(a) for a in [fl, *arrs, bb, y]]
        try:
            df, dx, dd, da, db_, dc, dbb, dy = (C.c_void_p(u.ptr) for u in bufs)
            self._check(self.L.msbg_gpu_multiply_laplacian_dense(
                self.h, OPT_CALC_RESIDUAL if residual else 0, level_mg, sx, sy, sz, df, dx, dbb, dd, da, db_, dc, dy))
            self._check(self.L.msbg_gpu_copy_d2h(self.h, _ptr(y), dy, y.nbytes))
            self.synchronize()
        finally:
            for u in bufs:
                u.free()
        return y

    # reference: relax() at a dense multigrid level (src/msbg3.cpp:1917-2165)
    def relax_dense(self, level_mg: int, n_iter: int, flags, x, b, dinv, area_x, area_y, area_z,
                    tmp=None) -> np.ndarray:
        """Host arrays [sz][sy][sx] in (tmp: the temporary channel, zero by default), X after the
        iterations out."""
        fl = np.ascontiguousarray(flags, np.uint16)
        sz, sy, sx = fl.shape
        arrs = [np.ascontiguousarray(a, np.float32).reshape(fl.shape) for a in (x, b, dinv, area_x, area_y, area_z)]
        t = np.ascontiguousarray(np.zeros(fl.shape) if tmp is None else tmp, np.float32).reshape(fl.shape)
        bufs = [self.to_device(a) for a in [fl, *arrs, t]]
        out = np.empty(fl.shape, np.float32)
        try:
            df, dx, db_, dd, da, dby, dc, dt = (C.c_void_p(u.ptr) for u in bufs)
            self._check(self.L.msbg_gpu_relax_dense(self.h, level_mg, sx, sy, sz, n_iter, df, dx, db_, dd, da, dby,
                                                    dc, dt))
            self._check(self.L.msbg_gpu_copy_d2h(self.h, _ptr(out), dx, out.nbytes))
            self.synchronize()
        finally:
            for u in bufs:
                u.free()
        return out

    # reference: relaxBlockList (src/msbg3.cpp:2170-2239) on a multi-resolution layout
    def relax_levels(self, lchan_x: int, lchan_b: int, lchan_d: int, bids: np.ndarray, reverse: bool = False) -> int:
        """One pass of the block smoother over the listed blocks (any level), X relaxed in place
        in its level channel; returns the number of skipped blocks."""
        bids = np.ascontiguousarray(bids, np.int32)
        db = self.to_device(bids)
        sk = C.c_int64(-1)
        try:
            self._check(self.L.msbg_gpu_relax_levels(self.h, int(reverse), lchan_x, lchan_b, lchan_d,
                                                     C.c_void_p(db.ptr), len(bids), C.byref(sk)))
            self.synchronize()
        finally:
            db.free()
        return int(sk.value)

    # reference: dotProdChannel(ch1, ch2, levelMg, blockList, pErrCode) (src/msbg.h:3331-3341);
    # a non-finite sum raises MsbgGpuError with ERR_NONFINITE (the reference's pErrCode)
    def dotProdChannel(self, a: int, b: int, levelMg: int = 0, blockList=None) -> float:
        lp, ln, keep = self._block_list(blockList)
        out = C.c_double()
        self._check(self.L.msbg_gpu_dot(self.h, a, b, levelMg, lp, ln, C.byref(out)))
        return out.value

    # reference: AXPBYChannel(a, iChanX, b, iChanDstY, levelMax, levelMg, blockList)
    # (src/msbg.h:3356-3362)
    def AXPBYChannel(self, a: float, chanX: int, b: float, chanY: int, levelMax: int = 9999, levelMg: int = 0,
                     blockList=None):
        lp, ln, keep = self._block_list(blockList)
        self._check(self.L.msbg_gpu_axpby(self.h, a, chanX, b, chanY, levelMax, levelMg, lp, ln))
        if keep is not None and keep is not blockList:
            self.synchronize()

    # reference: AXPBYChannelCombined(a, b, iChanQ, iChanX, iChanP, blockList) (src/msbg.h:3364-3368)
    def AXPBYChannelCombined(self, a: float, b: float, chanQ: int, chanX: int, chanP: int, blockList=None):
        lp, ln, keep = self._block_list(blockList)
        self._check(self.L.msbg_gpu_axpby_combined(self.h, a, b, chanQ, chanX, chanP, lp, ln))
        if keep is not None and keep is not blockList:
            self.synchronize()

    def poisson_release_work(self):
        """Frees the solver's level-0 work vectors and FP16 copies (reallocated on demand)."""
        self._check(self.L.msbg_gpu_poisson_release_work(self.h))

    def mgpcg_solve(self, chanX: int, chanB: int, tol: float = 1e-6, max_iter: int = 200):
        it, rel = C.c_int(), C.c_double()
        self._check(self.L.msbg_gpu_mgpcg_solve(self.h, chanX, chanB, tol, max_iter, C.byref(it), C.byref(rel)))
        return it.value, rel.value

    def mgpcg_solve_mixed(self, chanX: int, chanB: int, tol: float = 1e-6, max_outer: int = 10,
                          inner_tol: float = 1e-3, max_inner: int = 60):
        o, i, rel = C.c_int(), C.c_int(), C.c_double()
        self._check(self.L.msbg_gpu_mgpcg_solve_mixed(self.h, chanX, chanB, tol, max_outer, inner_tol,
                                                      max_inner, C.byref(o), C.byref(i), C.byref(rel)))
        return o.value, i.value, rel.value

    def poisson_set_params(self, pre: int = 2, post: int = 2, tile_iters: int = 3, coarsest_iter: int = 0):
        self._check(self.L.msbg_gpu_poisson_set_params(self.h, pre, post, tile_iters, coarsest_iter))

    # ---- batched solves ---------------------------------------------------------------------
    def batch_set_volumes(self, vol_of_block: np.ndarray, n_vol: int):
        v = np.ascontiguousarray(vol_of_block, np.int32)
        self._check(self.L.msbg_gpu_batch_set_volumes(self.h, _ptr(v), int(n_vol)))
        self._n_vol = int(n_vol)

    def batch_mgpcg_solve(self, chanX: int, chanB: int, tol: float = 1e-6, max_iter: int = 100,
                          use_graph: bool = True):
        nv = self._n_vol
        its = np.zeros(nv, np.int32)
        ms = np.zeros(nv, np.float32)
        rel = np.zeros(nv, np.float64)
        tot = C.c_float()
        self._check(self.L.msbg_gpu_batch_mgpcg_solve(self.h, chanX, chanB, tol, max_iter, int(use_graph),
                                                      _ptr(its), _ptr(ms), _ptr(rel), C.byref(tot)))
        return its, ms, rel, tot.value

    # ---- learned warm start ----------------------------------------------------------------
    WARMNET_CH = (2, 16, 16, 16, 2)

    @classmethod
    def _wn_split(cls, flat_w, flat_b):
        W, B, ow, ob = [], [], 0, 0
        for l in range(4):
            cin, cout = cls.WARMNET_CH[l], cls.WARMNET_CH[l + 1]
            n = 27 * cin * cout
            W.append(flat_w[ow:ow + n].reshape(27, cin, cout).copy())
            B.append(flat_b[ob:ob + cout].copy())
            ow += n
            ob += cout
        return W, B

    def warmnet_set(self, weights, biases, reset_optimizer: bool = True):
        w = np.ascontiguousarray(np.concatenate([np.asarray(x, np.float32).ravel() for x in weights]))
        b = np.ascontiguousarray(np.concatenate([np.asarray(x, np.float32).ravel() for x in biases]))
        self._check(self.L.msbg_gpu_warmnet_set_weights(self.h, _ptr(w), _ptr(b), int(reset_optimizer)))

    def warmnet_get(self):
        nw, nb = C.c_int(), C.c_int()
        self.L.msbg_gpu_warmnet_param_count(C.byref(nw), C.byref(nb))
        w = np.zeros(nw.value, np.float32)
        b = np.zeros(nb.value, np.float32)
        self._check(self.L.msbg_gpu_warmnet_get_weights(self.h, _ptr(w), _ptr(b)))
        return self._wn_split(w, b)

    def warmnet_set_loss(self, mode: str):
        self._check(self.L.msbg_gpu_warmnet_set_loss(self.h, {"coarse": 0, "residual": 1}[mode]))

    def warmnet_predict(self, chanB: int, chanX0: int):
        self._check(self.L.msbg_gpu_warmnet_predict(self.h, chanB, chanX0))

    def warmnet_loss_grad(self, chanB: int, chanXstar: int):
        nw, nb = C.c_int(), C.c_int()
        self.L.msbg_gpu_warmnet_param_count(C.byref(nw), C.byref(nb))
        gw = np.zeros(nw.value, np.float32)
        gb = np.zeros(nb.value, np.float32)
        loss = C.c_double()
        self._check(self.L.msbg_gpu_warmnet_loss_grad(self.h, chanB, chanXstar, C.byref(loss), _ptr(gw), _ptr(gb)))
        W, B = self._wn_split(gw, gb)
        return loss.value, W, B

    def warmnet_train_step(self, dB: int, dXstar: int, lr: float) -> float:
        loss = C.c_double()
        self._check(self.L.msbg_gpu_warmnet_train_step(self.h, C.c_void_p(int(dB)), C.c_void_p(int(dXstar)), lr,
                                                       C.byref(loss)))
        return loss.value

    def copy_d2d(self, dst: int, src: int, nbytes: int):
        self._check(self.L.msbg_gpu_copy_d2d(self.h, C.c_void_p(int(dst)), C.c_void_p(int(src)), int(nbytes)))

    def mg_info(self):
        n = C.c_int()
        cells = np.zeros(32, np.int64)
        self._check(self.L.msbg_gpu_mg_info(self.h, C.byref(n), _ptr(cells), 32))
        return cells[: n.value].copy()

    def poisson_tuning(self, enable: int = -1) -> list:
        """The operator launch shapes the autotuner picked: (level, bytes per value, mode,
        cells per thread, grid) each; enable 1 / 0 switches tuning on / off (-1: as is)."""
        n = C.c_int()
        out = np.zeros((64, 5), np.int32)
        self._check(self.L.msbg_gpu_poisson_tuning(self.h, enable, _ptr(out), 64, C.byref(n)))
        return [tuple(int(v) for v in r) for r in out[: min(n.value, 64)]]

    # ---- timing -------------------------------------------------------------------------
    def event_record(self, slot: int):
        self._check(self.L.msbg_gpu_event_record(self.h, slot))

    def event_elapsed_ms(self, a: int, b: int) -> float:
        ms = C.c_float()
        self._check(self.L.msbg_gpu_event_elapsed(self.h, a, b, C.byref(ms)))
        return ms.value


def surface_pipeline(pts: np.ndarray, res, bsx: int, storage: int = F32, n_iter: int = 20,
                     lapl_typ: int = LAPL_MCF_8COLOR, dt: float = 0.1, r_particle: float = 2.0,
                     nb_dist: float = 2.0, n_levels: int = 3, bands=None, variant: int = SWEEP_EXACT,
                     keep_after_finalize: bool = True):
    """Step-by-step GPU pipeline (same stages as the reference demo); returns a dict."""
    sx, sy, sz = (res, res, res) if np.isscalar(res) else res
    pts = np.ascontiguousarray(pts, np.float32).reshape(-1, 3)
    g = MultiresSparseGrid(sx, sy, sz, bsx, n_levels, storage)
    try:
        d = g.to_device(pts)
        if bands is None:
            g.mark_points(d, len(pts), r_particle + nb_dist)
            g.levels_from_marks()
        else:
            g.levels_from_bands(d, len(pts), bands)
        g.regularizeRefinementMap()
        g.setRefinementMap(1.0)
        g.splat(d, len(pts), r_particle, nb_dist)
        g.splat_finalize(r_particle, nb_dist)
        after_final = g.payload(0) if keep_after_finalize else None
        if n_iter > 0:
            g.applyChannelPdeFast(0, laplTyp=lapl_typ, doConstrZeroOne=1, numIter=n_iter, timeStep=dt,
                                  variant=variant)
        out = dict(levels=g.levels(), flags=g.flags(), active_bids=g.active_blocks(),
                   after_finalize=after_final, after_pde=g.payload(0), info=g.info(),
                   launches=g.launch_count())
        d.free()
        return out
    finally:
        g.close()
