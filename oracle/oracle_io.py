"""Job/result files for the CPU oracles (test infrastructure only).

Two oracles share one binary layout (``oracle_common.h``):

* ``_ref/msbg_ref_driver`` - the MSBG reference library compiled from its own
  sources (x86-64 only; built by ``make -C oracle ref``);
* ``_build/libmsbg_oracle.so`` - the project's C restatement (any arch; built by
  ``make -C oracle port``), reached through ctypes in ``oracle/port.py``.

Only tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use
this module.
"""
from __future__ import annotations

import os
import struct
import subprocess
import tempfile
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DRIVER = os.path.join(HERE, "_ref", "msbg_ref_driver")

JOB_MAGIC = b"MSBGJOB2"
OUT_MAGIC = b"MSBGOUT2"
CHAN_F32, CHAN_U16 = 0, 1
JOB_SURFACE, JOB_LEVELS, JOB_INTERP, JOB_HALO, JOB_RENDER, JOB_MORTON = 1, 2, 3, 4, 5, 6

# interpolation options: the reference's bits (src/sbg.h:140-170) and the render-density
# scale of the uint16 channel (a bit the reference's enum leaves unused)
IP_CORNER = 1 << 0
IP_BC_DIRICHLET = 1 << 13
IP_BC_DIRICHLET_OLD = 1 << 14
IP_NO_BORDER_CHECK = 1 << 15
IP_RENDER_DENS = 1 << 18

# OracleJobHeader: magic[8], 11 x int32, 4 x float, int32, 2 x int64
_JOB_FMT = "<8s11i4fi2q"
# OracleOutHeader: magic[8], int32 nBlocks, int32 nActive, int64 nActParticles,
# int64[8], 6 x double, int32 elemBytes, int32 nThreadsUsed
_OUT_FMT = "<8s2iq8q6d2i"

PDE_MEAN_CURVATURE = 4
OPT_8_COLOR_SCHEME = 1 << 29
LAPL_MCF_8COLOR = -(PDE_MEAN_CURVATURE + OPT_8_COLOR_SCHEME)


@dataclass
class SurfaceJob:
    sx: int
    sy: int
    sz: int
    bsx: int
    points: np.ndarray
    chan: int = CHAN_F32
    n_iter: int = 20
    lapl_typ: int = LAPL_MCF_8COLOR
    constr01: int = 1
    dt: float = 0.1
    r_particle: float = 2.0
    nb_dist: float = 2.0
    n_levels: int = 3
    n_threads: int = 0
    levels: np.ndarray | None = None  # optional caller-supplied level map
    anis_alpha: float = 0.0


@dataclass
class OracleResult:
    n_blocks: int
    n_active: int
    n_act_particles: int
    blocks_per_level: np.ndarray
    times: dict
    levels: np.ndarray          # int8 [nBlocks]
    flags: np.ndarray           # uint16 [nBlocks]
    active_bids: np.ndarray     # int32 [nActive]
    after_finalize: np.ndarray  # [nActive, bsx^3]
    after_pde: np.ndarray       # [nActive, bsx^3]
    threads: int


def write_surface_job(path: str, job: SurfaceJob) -> None:
    pts = np.ascontiguousarray(job.points, dtype=np.float32).reshape(-1, 3)
    lv = None if job.levels is None else np.ascontiguousarray(job.levels, np.int32).ravel()
    hdr = struct.pack(_JOB_FMT, JOB_MAGIC, JOB_SURFACE, job.sx, job.sy, job.sz, job.bsx,
                      job.n_levels, job.chan, job.n_iter, job.lapl_typ, job.constr01,
                      job.n_threads, job.dt, job.r_particle, job.nb_dist, job.anis_alpha, 0,
                      pts.shape[0], 0 if lv is None else lv.size)
    with open(path, "wb") as f:
        f.write(hdr)
        f.write(pts.tobytes())
        if lv is not None:
            f.write(lv.tobytes())


def write_levels_job(path: str, sx: int, sy: int, sz: int, bsx: int, n_levels: int,
                     levels: np.ndarray, n_threads: int = 0) -> None:
    lv = np.ascontiguousarray(levels, dtype=np.int32).ravel()
    hdr = struct.pack(_JOB_FMT, JOB_MAGIC, JOB_LEVELS, sx, sy, sz, bsx, n_levels, 0, 0, 0, 0,
                      n_threads, 0.0, 0.0, 0.0, 0.0, 0, 0, lv.size)
    with open(path, "wb") as f:
        f.write(hdr)
        f.write(lv.tobytes())


def write_interp_job(path: str, sx: int, sy: int, sz: int, bsx: int, chan: int,
                     active_bids: np.ndarray, payload: np.ndarray, points: np.ndarray,
                     opt: int = 0, n_threads: int = 0) -> None:
    pts = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
    bids = np.ascontiguousarray(active_bids, dtype=np.int32).ravel()
    pay = np.ascontiguousarray(payload, dtype=np.float32 if chan == CHAN_F32 else np.uint16)
    if pay.size != bids.size * bsx ** 3:
        raise ValueError("payload size does not match the active blocks")
    hdr = struct.pack(_JOB_FMT, JOB_MAGIC, JOB_INTERP, sx, sy, sz, bsx, 3, chan, 0, 0, opt,
                      n_threads, 0.0, 0.0, 0.0, 0.0, 0, pts.shape[0], bids.size)
    with open(path, "wb") as f:
        f.write(hdr)
        f.write(pts.tobytes())
        f.write(bids.tobytes())
        f.write(pay.tobytes())


def run_reference_interp(sx, sy, sz, bsx, chan, active_bids, payload, points, opt: int = 0,
                         n_threads: int = 0, timeout: float = 600) -> tuple[np.ndarray, float, int]:
    """Interpolate a payload at points with the reference's own functions.

    Returns (values float32 [n], seconds spent in the interpolation loop, threads)."""
    with tempfile.TemporaryDirectory() as td:
        jp, op = os.path.join(td, "job.bin"), os.path.join(td, "out.bin")
        write_interp_job(jp, sx, sy, sz, bsx, chan, active_bids, payload, points, opt, n_threads)
        subprocess.run([REF_DRIVER, jp, op], check=True, cwd=td, timeout=timeout,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        with open(op, "rb") as f:
            buf = f.read()
    hsz = struct.calcsize(_OUT_FMT)
    h = struct.unpack(_OUT_FMT, buf[:hsz])
    if h[0] != OUT_MAGIC:
        raise ValueError("bad oracle output")
    n = np.asarray(points).reshape(-1, 3).shape[0]
    vals = np.frombuffer(buf, np.float32, n, hsz).copy()
    return vals, float(h[17]), int(h[19])


# halo fill options (src/msbg.h:101-131) and level-grid block states
BC_NEUMANN = 1 << 10
BC_COARSE_LEVEL = 1 << 26
LBLK_EMPTY, LBLK_FULL, LBLK_NONE = -1, -2, -3


def write_halo_job(path: str, sx: int, sy: int, sz: int, bsx: int, n_levels: int, chan: int,
                   levels: np.ndarray, states: list, payloads: list, level: int, halo: int,
                   opt: int, empty_value: float = 0.0, full_value: float = 1.0) -> None:
    lv = np.ascontiguousarray(levels, dtype=np.int32).ravel()
    dt = np.float32 if chan == CHAN_F32 else np.uint16
    hdr = struct.pack(_JOB_FMT, JOB_MAGIC, JOB_HALO, sx, sy, sz, bsx, n_levels, chan, halo, level, opt,
                      1, empty_value, full_value, 0.0, 0.0, 0, 0, lv.size)
    with open(path, "wb") as f:
        f.write(hdr)
        f.write(lv.tobytes())
        for l in range(n_levels):
            f.write(np.ascontiguousarray(states[l], dtype=np.int32).tobytes())
        for l in range(n_levels):
            n = int(np.max(states[l])) + 1 if len(states[l]) else 0
            bs = bsx >> l
            pay = np.ascontiguousarray(payloads[l], dtype=dt).reshape(-1)
            if pay.size < n * bs ** 3:
                raise ValueError(f"level {l}: payload smaller than its states need")
            f.write(pay[: n * bs ** 3].tobytes())


def run_reference_halo(sx, sy, sz, bsx, n_levels, chan, levels, states, payloads, level, halo, opt,
                       empty_value=0.0, full_value=1.0, timeout: float = 600):
    """HaloBlockSet::fillHaloBlock_ of every block at `level` by the reference itself.

    Returns (bids int32 [m], halo float32 [m][(bs+2h)^3])."""
    with tempfile.TemporaryDirectory() as td:
        jp, op = os.path.join(td, "job.bin"), os.path.join(td, "out.bin")
        write_halo_job(jp, sx, sy, sz, bsx, n_levels, chan, levels, states, payloads, level, halo, opt,
                       empty_value, full_value)
        r = subprocess.run([REF_DRIVER, jp, op], cwd=td, timeout=timeout,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        if r.returncode != 0:
            raise RuntimeError(f"reference halo job failed with status {r.returncode}")
        with open(op, "rb") as f:
            buf = f.read()
    hsz = struct.calcsize(_OUT_FMT)
    h = struct.unpack(_OUT_FMT, buf[:hsz])
    if h[0] != OUT_MAGIC:
        raise ValueError("bad oracle output")
    m = int(h[2])
    hs = (bsx >> level) + 2 * halo
    bids = np.frombuffer(buf, np.int32, m, hsz).copy()
    vals = np.frombuffer(buf, np.float32, m * hs ** 3, hsz + 4 * m).copy().reshape(m, hs ** 3)
    return bids, vals


# the demo's camera (src/msbg_demo.cpp:123-127) and surface colour (src/msbg_demo.cpp:150)
DEMO_CAMERA = {"pos": (0.5, 0.8, 0.7), "look_at": (0.5, 0.5, 0.5), "sun": (0.5, 5.0, 5.0),
               "color": (0.8, 0.6, 0.4), "zoom": 1.0}


def camera_array(cam: dict) -> np.ndarray:
    """The 5 float32 triples of a render job: position, look-at, sun, colour, (zoom, 0, 0)."""
    return np.array([*cam["pos"], *cam["look_at"], *cam["sun"], *cam["color"], cam["zoom"], 0.0, 0.0],
                    np.float32)


def run_reference_render(sx, sy, sz, bsx, active_bids, payload_u16, width, height, cam=None,
                         n_threads: int = 0, timeout: float = 1200):
    """RDR::RaymarchRenderer::render (src/render.cpp:20-101) of a uint16 payload.

    Returns (pixels int32 [height][width] as BMP_MKRGB, seconds, threads)."""
    cam = DEMO_CAMERA if cam is None else cam
    bids = np.ascontiguousarray(active_bids, dtype=np.int32).ravel()
    pay = np.ascontiguousarray(payload_u16, dtype=np.uint16)
    with tempfile.TemporaryDirectory() as td:
        jp, op = os.path.join(td, "job.bin"), os.path.join(td, "out.bin")
        hdr = struct.pack(_JOB_FMT, JOB_MAGIC, JOB_RENDER, sx, sy, sz, bsx, 3, CHAN_U16, width, height, 0,
                          n_threads, 0.0, 0.0, 0.0, 0.0, 0, 5, bids.size)
        with open(jp, "wb") as f:
            f.write(hdr)
            f.write(camera_array(cam).tobytes())
            f.write(bids.tobytes())
            f.write(pay.tobytes())
        r = subprocess.run([REF_DRIVER, jp, op], cwd=td, timeout=timeout,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        if r.returncode != 0:
            raise RuntimeError(f"reference render job failed with status {r.returncode}")
        with open(op, "rb") as f:
            buf = f.read()
    hsz = struct.calcsize(_OUT_FMT)
    h = struct.unpack(_OUT_FMT, buf[:hsz])
    if h[0] != OUT_MAGIC:
        raise ValueError("bad oracle output")
    px = np.frombuffer(buf, np.int32, width * height, hsz).copy().reshape(height, width)
    return px, float(h[17]), int(h[19])


def run_reference_morton(sx, sy, sz, bsx, bids, timeout: float = 600) -> np.ndarray:
    """MultiresSparseGrid::sortBlockListMorton (src/msbg2.cpp:46-58) of a block-id list."""
    bids = np.ascontiguousarray(bids, dtype=np.int32).ravel()
    with tempfile.TemporaryDirectory() as td:
        jp, op = os.path.join(td, "job.bin"), os.path.join(td, "out.bin")
        hdr = struct.pack(_JOB_FMT, JOB_MAGIC, JOB_MORTON, sx, sy, sz, bsx, 3, 0, 0, 0, 0, 0,
                          0.0, 0.0, 0.0, 0.0, 0, 0, bids.size)
        with open(jp, "wb") as f:
            f.write(hdr)
            f.write(bids.tobytes())
        r = subprocess.run([REF_DRIVER, jp, op], cwd=td, timeout=timeout,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        if r.returncode != 0:
            raise RuntimeError(f"reference morton job failed with status {r.returncode}")
        with open(op, "rb") as f:
            buf = f.read()
    hsz = struct.calcsize(_OUT_FMT)
    return np.frombuffer(buf, np.int32, bids.size, hsz).copy()


def read_result(path: str, bsx: int, surface: bool = True) -> OracleResult:
    with open(path, "rb") as f:
        buf = f.read()
    hsz = struct.calcsize(_OUT_FMT)
    h = struct.unpack(_OUT_FMT, buf[:hsz])
    if h[0] != OUT_MAGIC:
        raise ValueError("bad oracle output")
    n_blocks, n_active, n_act = h[1], h[2], h[3]
    per_level = np.array(h[4:12], dtype=np.int64)
    tnames = ["mark", "levels", "alloc", "splat", "final", "pde"]
    times = dict(zip(tnames, h[12:18]))
    elem, threads = h[18], h[19]
    off = hsz
    levels = np.frombuffer(buf, np.int8, n_blocks, off); off += n_blocks
    flags = np.frombuffer(buf, np.uint16, n_blocks, off); off += 2 * n_blocks
    if not surface:
        z = np.zeros((0, bsx ** 3), np.float32)
        return OracleResult(n_blocks, 0, 0, per_level, times, levels.copy(), flags.copy(),
                            np.zeros(0, np.int32), z, z, threads)
    bids = np.frombuffer(buf, np.int32, n_active, off); off += 4 * n_active
    dt = np.float32 if elem == 4 else np.uint16
    nv = bsx ** 3
    a = np.frombuffer(buf, dt, n_active * nv, off).reshape(n_active, nv); off += elem * n_active * nv
    b = np.frombuffer(buf, dt, n_active * nv, off).reshape(n_active, nv)
    return OracleResult(n_blocks, n_active, n_act, per_level, times, levels.copy(), flags.copy(),
                        bids.copy(), a.copy(), b.copy(), threads)


def ref_available() -> bool:
    return os.path.isfile(REF_DRIVER) and os.access(REF_DRIVER, os.X_OK)


def run_reference_surface(job: SurfaceJob, timeout: float = 600) -> OracleResult:
    """Run the compiled reference library on a surface job."""
    with tempfile.TemporaryDirectory() as td:
        jp, op = os.path.join(td, "job.bin"), os.path.join(td, "out.bin")
        write_surface_job(jp, job)
        subprocess.run([REF_DRIVER, jp, op], check=True, cwd=td, timeout=timeout,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        return read_result(op, job.bsx, surface=True)


def run_reference_levels(sx, sy, sz, bsx, n_levels, levels, timeout: float = 600) -> OracleResult:
    """Run the reference regularizeRefinementMap + setRefinementMap on a level map."""
    with tempfile.TemporaryDirectory() as td:
        jp, op = os.path.join(td, "job.bin"), os.path.join(td, "out.bin")
        write_levels_job(jp, sx, sy, sz, bsx, n_levels, levels)
        subprocess.run([REF_DRIVER, jp, op], check=True, cwd=td, timeout=timeout,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        return read_result(op, bsx, surface=False)


JOB_SOLVER, JOB_DOWNSAMPLE, JOB_HALO3, JOB_LAYOUT = 7, 8, 9, 10


def run_reference_solver(sx, sy, sz, bsx, bids, x, b, q, p, cx, cy, cz, d, a: float = 0.5,
                         bcoef: float = -2.0, relax_passes: int = 1, reverse: bool = False,
                         n_threads: int = 0, timeout: float = 600) -> dict:
    """The reference's solver building blocks on the value blocks `bids` of a single-resolution
    layout (src/msbg3.cpp:1756-1912, 2170-2369; src/msbg.cpp:4524-4768).  Every array is a
    payload [n][bsx^3]; cx, cy, cz are the lower-face coefficients and d the diagonal (the job
    stores 1/d in CH_DIAGONAL, as the reference's operator expects).  Returns the dots and
    the arrays described in oracle_common.h."""
    bids = np.ascontiguousarray(bids, np.int32).ravel()
    n, nv = bids.size, bsx ** 3
    dinv = (1.0 / np.asarray(d, np.float32)).astype(np.float32)
    arrs = [np.ascontiguousarray(v, np.float32).reshape(n, nv) for v in (x, b, q, p, cx, cy, cz, dinv)]
    with tempfile.TemporaryDirectory() as td:
        jp, op = os.path.join(td, "job.bin"), os.path.join(td, "out.bin")
        hdr = struct.pack(_JOB_FMT, JOB_MAGIC, JOB_SOLVER, sx, sy, sz, bsx, 3, CHAN_F32, relax_passes, 0,
                          int(reverse), n_threads, a, bcoef, 0.0, 0.0, 0, 0, n)
        with open(jp, "wb") as f:
            f.write(hdr)
            f.write(bids.tobytes())
            for v in arrs:
                f.write(v.tobytes())
        r = subprocess.run([REF_DRIVER, jp, op], cwd=td, timeout=timeout,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        if r.returncode != 0:
            raise RuntimeError(f"reference solver job failed with status {r.returncode}")
        with open(op, "rb") as f:
            buf = f.read()
    hsz = struct.calcsize(_OUT_FMT)
    h = struct.unpack(_OUT_FMT, buf[:hsz])
    if h[0] != OUT_MAGIC:
        raise ValueError("bad oracle output")
    dots = np.frombuffer(buf, np.float64, 2, hsz)
    off = hsz + 16
    out = {"dot_ax_x": float(dots[0]), "dot_x_b": float(dots[1]), "dot_error": int(h[3])}
    for name in ("ax", "residual", "axpby_x", "axpby_p", "relaxed"):
        out[name] = np.frombuffer(buf, np.float32, n * nv, off).copy().reshape(n, nv)
        off += 4 * n * nv
    return out


def run_reference_downsample(sx, sy, sz, bsx, n_levels, levels, states, payloads, simple_average=False,
                             empty_value=0.0, full_value=1.0, timeout: float = 600):
    """downsampleFloatChannelNew (src/msbg4.cpp:1035-1379) to multigrid level 1 of an FP32
    multi-level channel given as the halo job's level states and payloads.

    Returns (bids int32 [m] of the level-0 blocks, coarse float32 [m][(bsx/2)^3])."""
    with tempfile.TemporaryDirectory() as td:
        jp, op = os.path.join(td, "job.bin"), os.path.join(td, "out.bin")
        write_halo_job(jp, sx, sy, sz, bsx, n_levels, CHAN_F32, levels, states, payloads, 0, 1,
                       int(simple_average), empty_value, full_value)
        with open(jp, "r+b") as f:  # the same layout under the downsample job type
            f.seek(8)
            f.write(struct.pack("<i", JOB_DOWNSAMPLE))
        r = subprocess.run([REF_DRIVER, jp, op], cwd=td, timeout=timeout,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        if r.returncode != 0:
            raise RuntimeError(f"reference downsample job failed with status {r.returncode}")
        with open(op, "rb") as f:
            buf = f.read()
    hsz = struct.calcsize(_OUT_FMT)
    h = struct.unpack(_OUT_FMT, buf[:hsz])
    if h[0] != OUT_MAGIC:
        raise ValueError("bad oracle output")
    m = int(h[2])
    nvc = (bsx // 2) ** 3
    bids = np.frombuffer(buf, np.int32, m, hsz).copy()
    vals = np.frombuffer(buf, np.float32, m * nvc, hsz + 4 * m).copy().reshape(m, nvc)
    return bids, vals


def run_reference_halo3(sx, sy, sz, bsx, n_levels, levels, states, payloads, flag_states, flag_payloads,
                        domain_bc, empty_value=0.0, full_value=1.0, empty_flags=0, full_flags=0,
                        timeout: float = 600):
    """HaloBlockSet::fillHaloBlock3 (src/halo.cpp:536-738) of every level-0 block by the
    reference itself: FP32 level grids, uint16 cell flags per level, domain boundary types
    (-x,+x,-y,+y,-z,+z; 0 = DBC_OPEN, 1 = DBC_SOLID).  Returns (bids, float32 [m][(bsx+2)^3])."""
    with tempfile.TemporaryDirectory() as td:
        jp, op = os.path.join(td, "job.bin"), os.path.join(td, "out.bin")
        write_halo_job(jp, sx, sy, sz, bsx, n_levels, CHAN_F32, levels, states, payloads, 0, 1, 0,
                       empty_value, full_value)
        with open(jp, "r+b") as f:
            f.seek(8)
            f.write(struct.pack("<i", JOB_HALO3))
            f.seek(struct.calcsize("<8s11i4f"))
            f.write(struct.pack("<i", (int(empty_flags) & 0xffff) | ((int(full_flags) & 0xffff) << 16)))
        with open(jp, "ab") as f:
            for l in range(n_levels):
                f.write(np.ascontiguousarray(flag_states[l], dtype=np.int32).tobytes())
            for l in range(n_levels):
                n = int(np.max(flag_states[l])) + 1 if len(flag_states[l]) else 0
                bs = bsx >> l
                f.write(np.ascontiguousarray(flag_payloads[l], dtype=np.uint16).reshape(-1)[: n * bs ** 3].tobytes())
            f.write(np.asarray(domain_bc, np.int32).tobytes())
        r = subprocess.run([REF_DRIVER, jp, op], cwd=td, timeout=timeout,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        if r.returncode != 0:
            raise RuntimeError(f"reference halo3 job failed with status {r.returncode}")
        with open(op, "rb") as f:
            buf = f.read()
    hsz = struct.calcsize(_OUT_FMT)
    h = struct.unpack(_OUT_FMT, buf[:hsz])
    if h[0] != OUT_MAGIC:
        raise ValueError("bad oracle output")
    m = int(h[2])
    hs = bsx + 2
    bids = np.frombuffer(buf, np.int32, m, hsz).copy()
    vals = np.frombuffer(buf, np.float32, m * hs ** 3, hsz + 4 * m).copy().reshape(m, hs ** 3)
    return bids, vals


def run_reference_layout(sx, sy, sz, bsx, n_levels, levels, timeout: float = 600) -> dict:
    """setRefinementMap's block lists and fine-coarse distance channel (src/msbg.cpp:1428-2165)
    by the reference itself: {"existing": ids, "fine_coarse": [ids per level], "dist": [per
    level {"value_bids", "value" uint16 [n][(bsx>>l)^3], "full_bids", "full_value"}]}."""
    lv = np.ascontiguousarray(levels, dtype=np.int32).ravel()
    with tempfile.TemporaryDirectory() as td:
        jp, op = os.path.join(td, "job.bin"), os.path.join(td, "out.bin")
        hdr = struct.pack(_JOB_FMT, JOB_MAGIC, JOB_LAYOUT, sx, sy, sz, bsx, n_levels, 0, 0, 0, 0, 1,
                          0.0, 0.0, 0.0, 0.0, 0, 0, lv.size)
        with open(jp, "wb") as f:
            f.write(hdr)
            f.write(lv.tobytes())
        r = subprocess.run([REF_DRIVER, jp, op], cwd=td, timeout=timeout,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        if r.returncode != 0:
            raise RuntimeError(f"reference layout job failed with status {r.returncode}")
        with open(op, "rb") as f:
            buf = f.read()
    off = struct.calcsize(_OUT_FMT)
    if buf[:8] != OUT_MAGIC:
        raise ValueError("bad oracle output")

    def lst():
        nonlocal off
        n = int(np.frombuffer(buf, np.int32, 1, off)[0])
        v = np.frombuffer(buf, np.int32, n, off + 4).copy()
        off += 4 + 4 * n
        return v

    out = {"existing": lst(), "fine_coarse": [lst() for _ in range(n_levels)], "dist": []}
    for l in range(n_levels):
        vb = lst()
        nv = (bsx >> l) ** 3
        val = np.frombuffer(buf, np.uint16, len(vb) * nv, off).copy().reshape(len(vb), nv)
        off += 2 * len(vb) * nv
        fb = lst()
        fv = int(np.frombuffer(buf, np.uint16, 1, off)[0])
        off += 2
        out["dist"].append({"value_bids": vb, "value": val, "full_bids": fb, "full_value": fv})
    return out


JOB_MULTIRES = 11


def run_reference_multires(sx, sy, sz, bsx, n_levels, levels, x, b, dinv, relax_passes: int = 0,
                           reverse: bool = False, timeout: float = 600) -> dict:
    """multiplyLaplacianMatrixOpt (src/msbg3.cpp:1756-1912) by the reference itself on a
    multi-resolution layout: every block of the (regular) level map `levels` is a fluid block
    at its level, with unit face areas and fluid cells, so neighbouring levels meet through
    procNeighMixedRes2 (src/msbg3.cpp:46-161).  x, b, dinv: float32 over the blocks of level 0,
    then level 1, ..., ascending bid, (bsx>>l)^3 values per block of level l; dinv is what
    CH_DIAGONAL holds (the operator multiplies by 1/dinv).  Returns {"dot": sum(Y X),
    "y": A X, "r": B - A X} in the same order, and with relax_passes > 0 "relaxed": X after
    that many passes of relaxBlockList (src/msbg3.cpp:2170-2239) from x."""
    lv = np.ascontiguousarray(levels, np.int32).ravel()
    arrs = [np.ascontiguousarray(v, np.float32).ravel() for v in (x, b, dinv)]
    total = sum(int((lv == l).sum()) * (bsx >> l) ** 3 for l in range(n_levels))
    if any(a.size != total for a in arrs):
        raise ValueError("array sizes do not match the level map")
    with tempfile.TemporaryDirectory() as td:
        jp, op = os.path.join(td, "job.bin"), os.path.join(td, "out.bin")
        hdr = struct.pack(_JOB_FMT, JOB_MAGIC, JOB_MULTIRES, sx, sy, sz, bsx, n_levels, CHAN_F32, relax_passes, 0,
                          int(reverse), 1, 0.0, 0.0, 0.0, 0.0, 0, 0, lv.size)
        with open(jp, "wb") as f:
            f.write(hdr)
            f.write(lv.tobytes())
            for a in arrs:
                f.write(a.tobytes())
        r = subprocess.run([REF_DRIVER, jp, op], cwd=td, timeout=timeout,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        if r.returncode != 0:
            raise RuntimeError(f"reference multires job failed with status {r.returncode}")
        with open(op, "rb") as f:
            buf = f.read()
    hsz = struct.calcsize(_OUT_FMT)
    if buf[:8] != OUT_MAGIC:
        raise ValueError("bad oracle output")
    dot = float(np.frombuffer(buf, np.float64, 1, hsz)[0])
    y = np.frombuffer(buf, np.float32, total, hsz + 8).copy()
    res = np.frombuffer(buf, np.float32, total, hsz + 8 + 4 * total).copy()
    out = {"dot": dot, "y": y, "r": res}
    if relax_passes > 0:
        out["relaxed"] = np.frombuffer(buf, np.float32, total, hsz + 8 + 8 * total).copy()
    return out


JOB_DENSE = 12


def run_reference_dense(sx0, sy0, sz0, bsx, n_levels, flags, x, b, dinv, area_x, area_y, area_z,
                        relax_iter: int = 0, timeout: float = 600) -> dict:
    """multiplyLaplacianMatrixOpt by the reference itself at the first dense multigrid level
    (levelMg = n_levels) of a grid sx0 x sy0 x sz0 with block edge bsx: the masked 7-point
    operator of ImultiplyLaplacianMatrixProcessSliceDenseLevel (src/msbg3.cpp:166-403).
    flags (cell flags, uint16) and the float32 arrays are [sz][sy][sx] of that level (x
    fastest); dinv is what CH_DIAGONAL holds, area_* the lower-face areas.  Returns
    {"y": A X, "r": B - A X} in the same layout, and with relax_iter > 0 "relaxed": X after
    relax() with that many iterations at the level (omega-Jacobi, src/msbg3.cpp:1917-2165)."""
    fl = np.ascontiguousarray(flags, np.uint16)
    shape = fl.shape
    arrs = [np.ascontiguousarray(v, np.float32).reshape(shape) for v in (x, b, dinv, area_x, area_y, area_z)]
    n = fl.size
    with tempfile.TemporaryDirectory() as td:
        jp, op = os.path.join(td, "job.bin"), os.path.join(td, "out.bin")
        hdr = struct.pack(_JOB_FMT, JOB_MAGIC, JOB_DENSE, sx0, sy0, sz0, bsx, n_levels, CHAN_F32, relax_iter, 0, 0,
                          1, 0.0, 0.0, 0.0, 0.0, 0, 0, n)
        with open(jp, "wb") as f:
            f.write(hdr)
            f.write(fl.astype(np.int32).tobytes())
            for a in arrs:
                f.write(a.tobytes())
        r = subprocess.run([REF_DRIVER, jp, op], cwd=td, timeout=timeout,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        if r.returncode != 0:
            raise RuntimeError(f"reference dense job failed with status {r.returncode}")
        with open(op, "rb") as f:
            buf = f.read()
    hsz = struct.calcsize(_OUT_FMT)
    h = struct.unpack(_OUT_FMT, buf[:hsz])
    if h[0] != OUT_MAGIC or (int(h[3]), int(h[2]), int(h[1])) != (shape[0], shape[1], shape[2]):
        raise ValueError("bad oracle output or level size")
    y = np.frombuffer(buf, np.float32, n, hsz).copy().reshape(shape)
    res = np.frombuffer(buf, np.float32, n, hsz + 4 * n).copy().reshape(shape)
    out = {"y": y, "r": res}
    if relax_iter > 0:
        out["relaxed"] = np.frombuffer(buf, np.float32, n, hsz + 8 * n).copy().reshape(shape)
    return out
