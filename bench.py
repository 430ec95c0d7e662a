"""Benchmark of the MSBG hot path on GB300.

Workload (default): the 4096^3 surface reconstruction -- 1,024 seeded ellipsoid
clusters x 32,000 points, base block 32^3, three resolution levels by distance
to the points (level 0 within 8 voxels, level 1 within 16), FP16 storage with
FP32 arithmetic, 8-color in-place mean-curvature-flow sweeps (laplTyp 4).

* ``value``: voxel-updates/s of one step = applyChannelPdeFast with 50 MCF
  iterations over every level-0 voxel, field resident in HBM.  The field
  (~9.4 GB) is far larger than L2, so no flush is needed between steps.
* ``e2e``: the same metric through the public entry point msbg_gpu_surface_job
  with host buffers: pinned host points in, layout + splat + finalize + 50
  sweeps on the device, the level-0 payload back to pinned host memory.
* ``roofline``: the sweep kernel's algorithmic bytes (read + write of every
  updated voxel, 2 x 2 B) per launch over its average launch time, against the
  measured HBM copy bandwidth in MEASURED_PEAKS.json.
* ``cpu_baseline``: the CPU restatement (oracle/msbg_oracle.c, OpenMP) on a
  bounded sample of the same workload.

``--impl reference`` times the reference's CPU implementation of the path on
the host cores instead: the reference library built from its sources where it
compiles (x86-64), else the CPU restatement of it (aarch64 hosts).
Multi-GPU: the path does not shard here ("replicas only"); N ranks each run the
full workload and ``value`` is the sum over ranks.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from msbg_gb300 import gpu as G  # noqa: E402
from msbg_gb300 import poisson_workload as PW  # noqa: E402
from msbg_gb300 import workloads as W  # noqa: E402

OPT8 = 1 << 29
MCF8 = -(4 + OPT8)
JAC8 = -(17 + OPT8)  # Jacobi diffusion (phi + dt sum f_i) / (1 + 6 dt), 8-colour in place
# DRAM bytes (read + write) of one sweep launch of the 4096^3 workload, from an ncu
# capture of the sweep kernel on this workload (mean of 8 launches)
SWEEP_TRAFFIC_4096 = 2.63e9


# ------------------------------------------------------------------------------------
# helpers
# ------------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int = 0):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.gpu)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks() -> tuple[dict, str]:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.isfile(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class Dist:
    """torch.distributed only for barrier / max over ranks when WORLD_SIZE > 1."""

    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.dist = None
        if self.world > 1:
            import torch
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            if torch.cuda.is_available():
                torch.cuda.set_device(self.local)
            dist.init_process_group("gloo")
            self.dist = dist
            self.torch = torch

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, v: float) -> float:
        if not self.dist:
            return v
        t = self.torch.tensor([v], dtype=self.torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()


# ------------------------------------------------------------------------------------
# CPU baseline: the oracle on a bounded sample of the workload
# ------------------------------------------------------------------------------------
def cpu_sample(spec: dict, pts: np.ndarray, target_sec: float = 10.0, max_blocks: int = 0):
    """MCF sweeps of the CPU restatement on a crop of the level-0 blocks.

    Returns (updates/s, sample description, threads).  The crop is the first
    ``n`` level-0 blocks in bid order (a contiguous slab of the volume) with the
    rest of the grid empty; sweeps run with the same 8-color schedule and FP16
    storage as the GPU."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import port as P  # test/bench infrastructure only: the timed CPU baseline
    res, bsx = spec["res"], spec["bsx"]
    storage = {"f16": P.F16, "f32": P.F32}[spec["storage"]]
    g = P.grid(res, res, res, bsx, storage)
    nb = g.nbx * g.nby * g.nbz
    cnt, valid, nv = P.mark_blocks(g, pts, 0.0)
    lv = np.zeros(nb, np.int32)
    if "fine_band" in spec:
        rb = np.array([spec["fine_band"], spec["mid_band"]], np.float32)
        P.lib().orc_band_levels(C.byref(g), P._p(pts), len(pts), P._p(valid), P._p(rb), 2, 3, P._p(lv))
    else:
        cnt, valid, nv = P.mark_blocks(g, pts, 4.0)
        lv = np.where(cnt > 0, 0, 2).astype(np.int32)
    lv, _ = P.regularize(lv, g.nbx, g.nby, g.nbz, 3)
    act = np.nonzero(lv == 0)[0]
    n_take = max_blocks or min(len(act), 2048)
    keep = np.full(nb, 2, np.int32)
    keep[act[:n_take]] = 0
    slot = np.empty(nb, np.int32)
    bids = np.empty(nb, np.int32)
    n_act = P.lib().orc_build_slots(P._p(keep), nb, P._p(slot), P._p(bids))
    bids = bids[:n_act].copy()
    vox = n_act * bsx ** 3
    rng = np.random.Generator(np.random.PCG64(7))
    field = rng.random(vox).astype(np.float32)
    payload = field.astype(np.float16).view(np.uint16) if storage == P.F16 else field
    # one iteration first to size the sample to ~target_sec
    t0 = time.perf_counter()
    P.pde(g, slot, bids, payload, MCF8, 1, 2, 0.1)
    t2 = time.perf_counter() - t0
    per_iter = t2 / 2
    n_iter = max(2, int(target_sec / max(per_iter, 1e-6)) // 2 * 2)
    t0 = time.perf_counter()
    P.pde(g, slot, bids, payload, MCF8, 1, n_iter, 0.1)
    dt = time.perf_counter() - t0
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    desc = (f"{n_iter} MCF 8-color iterations of the CPU restatement over {n_act} level-0 "
            f"blocks ({vox / 1e6:.1f} M voxels, {spec['storage']}) cropped from the workload")
    return vox * n_iter / dt, desc, threads


# ------------------------------------------------------------------------------------
# reference arm
# ------------------------------------------------------------------------------------
def run_reference(args, spec, dist: Dist):
    if dist.rank != 0:
        return
    pts = W.make_points(spec, 1 if spec is W.SURFACE_512 else 2)
    arch = platform.machine()
    ref_driver = os.path.join(ROOT, "oracle", "_ref", "msbg_ref_driver")
    kind = "port"
    vals = []
    desc = ""
    threads = os.cpu_count() or 1
    if arch in ("x86_64", "AMD64") and os.path.isfile(ref_driver):
        # the reference library itself on a cropped sample (its MCF sweep timing)
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle_io as O
        kind = "reference"
        res = 1024 if spec["res"] > 1024 else spec["res"]
        sub = pts[(pts < res - 1).all(axis=1)]
        for _ in range(args.warmup + args.steps):
            job = O.SurfaceJob(res, res, res, spec["bsx"], sub, chan=O.CHAN_U16, n_iter=4, dt=0.1,
                               n_threads=threads)
            r = O.run_reference_surface(job)
            vals.append(r.n_active * spec["bsx"] ** 3 * 4 / r.times["pde"])
        vals = vals[args.warmup:]
        desc = (f"reference applyChannelPdeFast<uint16> MCF, 4 iterations over the level-0 blocks of "
                f"the workload's points inside a {res}^3 crop")
        dtype = "u16 storage / f32 math"
    else:
        for i in range(args.warmup + args.steps):
            v, desc, threads = cpu_sample(spec, pts, target_sec=8.0)
            vals.append(v)
        vals = vals[args.warmup:]
        desc = "reference CPU path unavailable on this host (x86 SIMD); " + desc
        dtype = "f16 storage / f32 math" if spec["storage"] == "f16" else "f32"
    value = float(np.median(vals))
    line = {
        "impl": "reference", "metric": "voxel-updates/s (MCF sweeps)", "value": value,
        "unit": "voxel-updates/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "higher_is_better": True, "dtype": dtype, "data": "synthetic",
        "config": {"workload": spec["name"]},
        "cpu_baseline": {"value": value, "unit": "voxel-updates/s", "cores": threads, "kind": kind,
                         "sample": desc},
        "e2e": {"value": value, "unit": "voxel-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------------
# GB300 arm
# ------------------------------------------------------------------------------------
def run_gpu(args, spec, dist: Dist):
    storage = {"f16": G.F16, "f32": G.F32}[spec["storage"]]
    elem = 2 if storage == G.F16 else 4
    variant = G.SWEEP_FAST if args.variant == "fast" else G.SWEEP_EXACT
    n_iter = spec["n_iter"]
    pts = W.make_points(spec, 1 if spec is W.SURFACE_512 else 2)
    bands = (spec["fine_band"], spec["mid_band"]) if "fine_band" in spec else None
    res, bsx = spec["res"], spec["bsx"]

    g = G.MultiresSparseGrid(res, res, res, bsx, spec["n_levels"], storage)
    d = g.to_device(pts)
    n = len(pts)
    if bands:
        g.levels_from_bands(d, n, bands)
    else:
        g.mark_points(d, n, 4.0)
        g.levels_from_marks()
    g.regularizeRefinementMap()
    g.setRefinementMap(1.0)
    g.splat(d, n, 2.0, 2.0)
    g.splat_finalize(2.0, 2.0)
    g.synchronize()
    # the splat alone (each call rebuilds its particle lists and rewrites every value
    # block's minimum); the finalize after it restores the same field for the sweeps
    g.event_record(12)
    for _ in range(3):
        g.splat(d, n, 2.0, 2.0)
    g.event_record(13)
    g.splat_finalize(2.0, 2.0)
    g.synchronize()
    splat_ms = dist.max(g.event_elapsed_ms(12, 13)) / 3
    info = g.info()
    n_act = info.nActive
    vox = n_act * bsx ** 3
    updates_per_step = vox * (n_iter + (n_iter & 1))

    for _ in range(args.warmup):
        g.applyChannelPdeFast(0, laplTyp=MCF8, doConstrZeroOne=1, numIter=n_iter, timeStep=spec["dt"], variant=variant)
    g.synchronize()
    dist.barrier()
    clocks = ClockSampler(dist.local)
    clocks.start()
    l0 = g.launch_count()
    g.event_record(0)
    for _ in range(args.steps):
        g.applyChannelPdeFast(0, laplTyp=MCF8, doConstrZeroOne=1, numIter=n_iter, timeStep=spec["dt"], variant=variant)
    g.event_record(1)
    g.synchronize()
    ms = g.event_elapsed_ms(0, 1)
    launches = g.launch_count() - l0
    clk = clocks.stop()
    dist.barrier()
    ms_max = dist.max(ms)
    value = updates_per_step * args.steps * dist.world / (ms_max / 1e3)

    # roofline of the sweep kernel: every launch of the timed region is a color pass
    peaks, peak_kind = measured_peaks()
    bytes_per_update = 2 * elem
    per_launch_bytes = updates_per_step * bytes_per_update / (launches / args.steps)
    per_launch_s = (ms / 1e3) / launches
    achieved = per_launch_bytes / per_launch_s / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"],
                "traffic": args.traffic_per_launch if args.traffic_per_launch is not None
                else (SWEEP_TRAFFIC_4096 if spec is W.SURFACE_4096 and args.variant == "fast" else None),
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback"}

    # the same sweep machinery with the cheap Jacobi stencil (same layout and field)
    jacobi = None
    if not args.no_jacobi:
        for _ in range(max(1, args.warmup)):
            g.applyChannelPdeFast(0, laplTyp=JAC8, doConstrZeroOne=1, numIter=n_iter, timeStep=spec["dt"], variant=variant)
        g.synchronize()
        lj = g.launch_count()
        g.event_record(2)
        for _ in range(args.steps):
            g.applyChannelPdeFast(0, laplTyp=JAC8, doConstrZeroOne=1, numIter=n_iter, timeStep=spec["dt"], variant=variant)
        g.event_record(3)
        g.synchronize()
        msj = dist.max(g.event_elapsed_ms(2, 3))
        nlj = g.launch_count() - lj
        vj = updates_per_step * args.steps * dist.world / (msj / 1e3)
        achj = (updates_per_step * bytes_per_update / (nlj / args.steps)) / ((msj / 1e3) / nlj) / 1e9
        jacobi = {"laplTyp": 17, "value": vj, "unit": "voxel-updates/s", "ms_per_step": msj / args.steps,
                  "roofline": {"bound": "hbm", "achieved": achj, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                               "frac": achj / peaks["hbm_gbs"]}}

    # restriction of the swept field to the next coarser level (downsampleFloatChannelNew):
    # S bytes read per fine voxel, 4 bytes written per coarse cell (one per 8 fine voxels)
    restriction = None
    if not args.no_jacobi:
        cb3 = (bsx // 2) ** 3
        dst = G.DeviceBuffer.alloc(n_act * cb3 * 4)
        for _ in range(max(3, args.warmup)):
            g._check(g.L.msbg_gpu_downsample_channel(g.h, 0, C.c_void_p(dst.ptr), 0))
        g.synchronize()
        lr = g.launch_count()
        g.event_record(4)
        for _ in range(args.steps):
            g._check(g.L.msbg_gpu_downsample_channel(g.h, 0, C.c_void_p(dst.ptr), 0))
        g.event_record(5)
        g.synchronize()
        msr = dist.max(g.event_elapsed_ms(4, 5)) / args.steps
        dst.free()
        nbytes = vox * elem + n_act * cb3 * 4
        restriction = {"kernel": "kDownsample (4^3 Gauss-like weights)", "ms_per_call": msr,
                       "fine_voxels_per_s": vox * dist.world / (msr / 1e3),
                       "launches_per_call": (g.launch_count() - lr) // args.steps,
                       "roofline": {"bound": "hbm", "achieved": nbytes / (msr / 1e3) / 1e9,
                                    "peak": peaks["hbm_gbs"], "unit": "GB/s",
                                    "frac": nbytes / (msr / 1e3) / 1e9 / peaks["hbm_gbs"]}}

    # grid-to-particle interpolation of the swept field at every particle
    # (interpolateFloatFast / interpolateUint16ToFloatFast per point): 12 bytes of position
    # read and 4 bytes written per point; the 8 corner reads are gathers served by L1/L2
    g2p = None
    if not args.no_jacobi:
        dout = G.DeviceBuffer.alloc(max(n, 1) * 4)
        for _ in range(max(3, args.warmup)):
            g.interpolate_device(0, d, n, dout, 0)
        g.synchronize()
        lg = g.launch_count()
        g.event_record(6)
        for _ in range(args.steps):
            g.interpolate_device(0, d, n, dout, 0)
        g.event_record(7)
        g.synchronize()
        msg = dist.max(g.event_elapsed_ms(6, 7)) / args.steps
        dout.free()
        gbs = n * 16 / (msg / 1e3) / 1e9
        g2p = {"kernel": "kInterpolate (trilinear)", "points": int(n), "ms_per_call": msg,
               "particles_per_s": n * dist.world / (msg / 1e3),
               "launches_per_call": (g.launch_count() - lg) // args.steps,
               "roofline": {"bound": "l2/latency (gathers)", "achieved": gbs, "peak": peaks["hbm_gbs"],
                            "unit": "GB/s", "frac": gbs / peaks["hbm_gbs"],
                            "algorithmic_bytes_per_point": 16}}

    # e2e through the host-buffer entry point
    e2e = None
    if not args.no_e2e:
        hp = C.c_void_p()
        G.load_library().msbg_gpu_host_alloc(C.byref(hp), pts.nbytes)
        hpts = np.ctypeslib.as_array(C.cast(hp, C.POINTER(C.c_float)), shape=(pts.size,))
        hpts[:] = pts.ravel()
        out_bytes = vox * elem
        ho = C.c_void_p()
        G.load_library().msbg_gpu_host_alloc(C.byref(ho), out_bytes)
        times = []
        e2e_steps = max(1, min(args.steps, 3))
        b = np.asarray(bands, np.float32) if bands else None
        n_act_out = C.c_int64()
        gpu_times, stage_runs = [], []
        for i in range(1 + e2e_steps):
            dist.barrier()
            g.event_record(14)
            t0 = time.perf_counter()
            rc = g.L.msbg_gpu_surface_job(g.h, hp, n, 2.0, 2.0, G._ptr(b), 0 if b is None else len(b),
                                          MCF8, n_iter, spec["dt"], variant, ho, out_bytes,
                                          C.byref(n_act_out))
            dt_s = time.perf_counter() - t0
            g._check(rc)
            g.event_record(15)
            if i > 0:
                times.append(dt_s)
                gpu_times.append(g.event_elapsed_ms(14, 15) / 1e3)
            if i > 0:
                stage_runs.append(g.surface_job_stages())
        t_e2e = dist.max(float(np.median(times)))
        stages = {k: float(np.median([r[k] for r in stage_runs])) for k in stage_runs[0]}
        serial = {"api": "msbg_gpu_surface_job (one job at a time)",
                  "value": updates_per_step * dist.world / t_e2e, "seconds_per_step": t_e2e,
                  "stream_seconds_per_step": float(np.median(gpu_times)),
                  "stage_ms": stages, "stage_ms_sum": float(sum(stages.values())),
                  "d2h_gb_per_s": out_bytes / (stages["download"] / 1e3) / 1e9 if stages.get("download") else None}
        # the streaming form: jobs queued back to back, each with its own upload of the points
        # and download of the payload, which overlap the neighbouring jobs' compute
        submit = lambda: g._check(g.L.msbg_gpu_surface_job_submit(
            g.h, hp, n, 2.0, 2.0, G._ptr(b), 0 if b is None else len(b), MCF8, n_iter, spec["dt"], variant, ho,
            out_bytes, C.byref(n_act_out)))
        submit()
        g._check(g.L.msbg_gpu_surface_job_wait(g.h))  # warm-up: staging buffers
        k_jobs = max(3, min(args.steps, 6))
        dist.barrier()
        t0 = time.perf_counter()
        for _ in range(k_jobs):
            submit()
        g._check(g.L.msbg_gpu_surface_job_wait(g.h))
        t_pipe = dist.max((time.perf_counter() - t0) / k_jobs)
        e2e = {"value": updates_per_step * dist.world / t_pipe, "unit": "voxel-updates/s",
               "h2d_bytes_per_step": int(pts.nbytes), "d2h_bytes_per_step": int(out_bytes),
               "seconds_per_step": t_pipe,
               "api": f"msbg_gpu_surface_job_submit, {k_jobs} jobs queued back to back, then "
                      "msbg_gpu_surface_job_wait (wall clock over all of them)",
               "serial": serial}
        G.load_library().msbg_gpu_host_free(hp)
        G.load_library().msbg_gpu_host_free(ho)

    # cross-resolution halo fill (HaloBlockSet::fillHaloBlock_, OPT_BC_COARSE_LEVEL, halo 1)
    # of every level-0 block of the swept field: level 0 of a level channel bound to the
    # value-block slab (states: slots, "no block" off level 0), level 1 the level-1
    # blocks.  Algorithmic bytes per block: the (bs+2)^3 box read once at S bytes per
    # value and written once as FP32.
    halo, bound = None, []
    if not args.no_jacobi:
        halo = halo_measure(g, info, storage, elem, bsx, args.steps, dist, peaks, bound)

    # ray-march render of the iso-0.5 surface (RaymarchRenderer::render) of the swept field
    render = None
    if not args.no_jacobi:
        render = render_measure(g, args.steps, dist, cpu=dist.rank == 0 and not args.no_cpu_baseline)

    cpu = None
    if dist.rank == 0 and not args.no_cpu_baseline:
        v, desc, threads = cpu_sample(spec, pts, target_sec=args.cpu_seconds)
        cpu = {"value": v, "unit": "voxel-updates/s", "cores": threads, "kind": "port",
               "sample": desc}

    # the workload's field error against an FP64 GPU run of the same algorithm
    field_error = None
    if args.fp64_check:
        field_error = fp64_field_error(g, d, n, spec, bands, variant)

    d.free()
    g.close()
    for b in bound:  # device arrays a level channel of g was bound to: free after g
        b.free()
    poisson = poisson_crop = poisson_batch = None
    if not args.no_poisson and spec is W.SURFACE_4096:
        # the stated Poisson workload: every level-0 block of the layout; then the learned
        # warm start, which does not fit beside the solver at that size, on a crop of it;
        # then the 256-volume batch
        poisson = poisson_full_measure(1, 1)
        poisson_crop = poisson_measure(96, max(1, min(args.steps, 3)), 1)
        from msbg_gb300 import batch_workload as BW
        poisson_batch = BW.run_batch(max(1, min(args.steps, 3)), 1, WARMNET)
    if dist.rank != 0:
        return
    line = {
        "metric": "voxel-updates/s (MCF sweeps)", "value": value, "unit": "voxel-updates/s",
        "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f16 storage / f32 math" if storage == G.F16 else "f32",
        "data": "synthetic",
        "config": {"workload": spec["name"], "points": int(n), "level0_blocks": int(n_act),
                   "blocks_per_level": [int(x) for x in info.blocksPerLevel[:3]],
                   "voxel_updates_per_step": int(updates_per_step), "mcf_iterations": n_iter,
                   "sweep_variant": args.variant, "l2": "inputs larger than L2 (no flush)",
                   "parallelism": f"replicas x{dist.world}"},
        "gpu_launches": int(launches),
        "roofline": roofline,
        "clocks": clk,
        "e2e": e2e,
        "cpu_baseline": cpu,
        "jacobi_sweeps": jacobi,
        "restriction": restriction,
        "g2p": g2p,
        "field_error_vs_fp64": field_error,
        "splat": {"kernel": "kSplatCount + kSplatScatter + kSplatBlock (particles sorted into per-block "
                            "lists; blocks of 32^3 split into two CTAs by z-half, smaller blocks one CTA; "
                            "minimum in shared memory)", "ms_per_call": splat_ms,
                  "particles_per_s": n * dist.world / (splat_ms / 1e3)},
        "halo_fill": halo,
        "render": render,
        "poisson": poisson,
        "poisson_crop96": poisson_crop,
        "poisson_batch": poisson_batch,
    }
    print(json.dumps(line), flush=True)


def halo_measure(g, info, storage, elem, bsx, steps, dist, peaks, bound: list, batch=16384) -> dict:
    lv = g.levels()
    slot = g.slots()
    st0 = np.where(lv == 0, slot, G.LBLK_NONE).astype(np.int32)
    n1 = int((lv == 1).sum())
    st1 = np.full(lv.size, G.LBLK_NONE, np.int32)
    st1[lv == 1] = np.arange(n1, dtype=np.int32)
    d_st0 = g.to_device(st0)
    bound.append(d_st0)  # the context keeps this binding until it is destroyed
    g.level_grid_bind(0, 0, storage, d_st0.ptr, g.payload_ptr(0), 0.0, 1.0)
    g.level_grid_set(0, 1, storage, st1, np.zeros((max(n1, 1), (bsx // 2) ** 3), G.NP_STORAGE[storage]),
                     0.0, 1.0)
    bids = np.nonzero(lv == 0)[0].astype(np.int32)
    d_bids = g.to_device(bids)
    hs = bsx + 2
    nb = min(batch, len(bids))
    d_out = G.DeviceBuffer.alloc(nb * hs ** 3 * 4)

    def one_pass():
        for k0 in range(0, len(bids), nb):
            m = min(nb, len(bids) - k0)
            g._check(g.L.msbg_gpu_fill_halo_blocks(g.h, 0, 0, C.c_void_p(d_bids.ptr + 4 * k0), m, 1,
                                                   G.BC_COARSE_LEVEL, C.c_void_p(d_out.ptr), None))

    for _ in range(3):
        one_pass()
    g.synchronize()
    l0 = g.launch_count()
    g.event_record(8)
    for _ in range(steps):
        one_pass()
    g.event_record(9)
    g.synchronize()
    ms = dist.max(g.event_elapsed_ms(8, 9)) / steps
    launches = (g.launch_count() - l0) // steps
    sk = g.fill_halo_blocks_device(0, 0, d_bids, nb, 1, G.BC_COARSE_LEVEL, d_out, count_skipped=True)
    d_out.free()
    d_bids.free()
    nbytes = len(bids) * hs ** 3 * (elem + 4)
    gbs = nbytes / (ms / 1e3) / 1e9
    return {"kernel": "kFillHalo (OPT_BC_COARSE_LEVEL, halo 1)", "blocks": int(len(bids)),
            "level1_blocks": n1, "ms_per_pass": ms, "blocks_per_s": len(bids) * dist.world / (ms / 1e3),
            "launches_per_pass": int(launches), "skipped": int(sk),
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "frac": gbs / peaks["hbm_gbs"],
                         "algorithmic_bytes_per_block": hs ** 3 * (elem + 4)}}


def fp64_field_error(g, d_pts, n, spec, bands, variant, chunk=4096) -> dict:
    """The workload's pipeline (splat, finalize, spec['n_iter'] MCF sweeps) once more on g in
    its storage, and on a second grid with FP64 storage and FP64 arithmetic (the sweep's
    exact form, reference operation order): relative L2 and max error of the first against
    the second over every level-0 voxel, compared chunk by chunk on the host."""
    res, bsx, n_iter = spec["res"], spec["bsx"], spec["n_iter"]
    t0 = time.perf_counter()
    g.setRefinementMap(1.0)
    g.splat(d_pts, n, 2.0, 2.0)
    g.splat_finalize(2.0, 2.0)
    g.applyChannelPdeFast(0, laplTyp=MCF8, doConstrZeroOne=1, numIter=n_iter, timeStep=spec["dt"], variant=variant)
    g.synchronize()
    g64 = G.MultiresSparseGrid(res, res, res, bsx, spec["n_levels"], G.F64)
    try:
        if bands:
            g64.levels_from_bands(d_pts, n, bands)
        else:
            g64.mark_points(d_pts, n, 4.0)
            g64.levels_from_marks()
        g64.regularizeRefinementMap()
        g64.setRefinementMap(1.0)
        g64.splat(d_pts, n, 2.0, 2.0)
        g64.splat_finalize(2.0, 2.0)
        t1 = time.perf_counter()
        g64.applyChannelPdeFast(0, laplTyp=MCF8, doConstrZeroOne=1, numIter=n_iter, timeStep=spec["dt"], variant=G.SWEEP_EXACT)
        g64.synchronize()
        t64 = time.perf_counter() - t1
        same_layout = bool(np.array_equal(g.active_blocks(), g64.active_blocks()))
        n_act = g.info().nActive
        vpb = bsx ** 3
        dt_lo = G.NP_STORAGE[g.storage[0]]
        p_lo, p_hi = g.payload_ptr(0), g64.payload_ptr(0)
        esz = np.dtype(dt_lo).itemsize
        se = sr = 0.0
        mx = 0.0
        for k0 in range(0, n_act, chunk):
            m = min(chunk, n_act - k0)
            lo = np.empty(m * vpb, dt_lo)
            hi = np.empty(m * vpb, np.float64)
            g._check(g.L.msbg_gpu_copy_d2h(g.h, G._ptr(lo), C.c_void_p(p_lo + k0 * vpb * esz), lo.nbytes))
            g64._check(g64.L.msbg_gpu_copy_d2h(g64.h, G._ptr(hi), C.c_void_p(p_hi + k0 * vpb * 8), hi.nbytes))
            g.synchronize()
            g64.synchronize()
            e = lo.astype(np.float64) - hi
            se += float(np.dot(e, e))
            sr += float(np.dot(hi, hi))
            mx = max(mx, float(np.abs(e).max()))
        return {"reference": "same pipeline on the GPU with FP64 storage and FP64 arithmetic (exact form)",
                "tested": f"{spec['storage']} storage, FP32 arithmetic, {'fast' if variant == G.SWEEP_FAST else 'exact'} form",
                "same_active_blocks": same_layout, "voxels": int(n_act * vpb),
                "rel_l2": (se / sr) ** 0.5 if sr > 0 else None, "max_abs": mx,
                "fp64_sweep_seconds": t64, "seconds": time.perf_counter() - t0}
    finally:
        g64.close()


def render_measure(g, steps, dist, cpu: bool, width=1920, height=1080) -> dict:
    """RaymarchRenderer::render of channel 0 from the demo's camera at width x height;
    with cpu, the CPU restatement renders 1/64 of the pixels (the same view at width/8 x
    height/8) on all host cores."""
    d_rgb = G.DeviceBuffer.alloc(width * height * 3)
    g.render_device(0, width, height, G.DEMO_CAMERA, d_rgb)
    g.synchronize()
    l0 = g.launch_count()
    g.event_record(10)
    n = max(1, min(steps, 3))
    for _ in range(n):
        g.render_device(0, width, height, G.DEMO_CAMERA, d_rgb)
    g.event_record(11)
    g.synchronize()
    ms = dist.max(g.event_elapsed_ms(10, 11)) / n
    img = np.empty((height, width, 3), np.uint8)
    g._check(g.L.msbg_gpu_copy_d2h(g.h, G._ptr(img), C.c_void_p(d_rgb.ptr), img.nbytes))
    g.synchronize()
    d_rgb.free()
    out = {"kernel": "kRender (FP64 ray march, cubic B-spline normal)", "width": width, "height": height,
           "camera": "demo (src/msbg_demo.cpp:123-127)", "ms_per_frame": ms,
           "pixels_per_s": width * height * dist.world / (ms / 1e3), "hit_pixels": int(img.any(-1).sum()),
           "launches_per_frame": (g.launch_count() - l0) // n,
           "bound": "FP64 pipe (3 adds + 3 conversions per ray step) and gathers near the surface"}
    if cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import port as P  # the oracle, as the CPU baseline
        info = g.info()
        og = P.grid(g.sx, g.sy, g.sz, g.bsx, {G.F32: P.F32, G.F16: P.F16, G.U16: P.U16}[g.storage[0]])
        pay = g.payload(0)
        host = pay.view(np.uint16) if pay.dtype == np.float16 else pay
        w8, h8 = width // 8, height // 8
        t0 = time.perf_counter()
        P.render(og, g.slots(), host, w8, h8, G.DEMO_CAMERA)
        sec = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": w8 * h8 / sec, "unit": "pixels/s", "cores": os.cpu_count(),
                               "kind": "port", "sample": f"{w8}x{h8} pixels of the same view, all host threads",
                               "value_blocks": int(info.nActive)}
        del pay, host
    return out


WARMNET = os.path.join(ROOT, "msbg_gb300", "data", "warmnet_c3.npz")


def poisson_measure(n_objects: int, steps: int, warmup: int,
                    modes=("plain", "mixed", "learned", "learned_mixed")) -> dict:
    """Time-to-1e-6 of the sparse Poisson solve on the level-0 blocks of the 4096^3
    layout (first n_objects clusters): plain FP32 MG-PCG and FP16-storage / FP32
    iterative refinement from X = 0, and both from the learned warm start (trained
    weights in msbg_gb300/data, forward pass inside the timed region); median over
    `steps` solves."""
    g, spec = PW.surface_layout_grid(n_objects)
    try:
        bs = spec["bsx"]
        PW.setup_problem(g, bs)
        if any(m.startswith("learned") for m in modes):
            W_, c_ = PW.load_warmnet(WARMNET)
            g.warmnet_set(W_, c_)
        cells = int(g.info().nActive) * bs ** 3
        out = {"workload": f"poisson-4096^3-bs32-crop{n_objects}", "cells": cells,
               "mg_levels": [int(v) for v in g.mg_info()], "tolerance": 1e-6,
               "rhs": "N(0,1) per cell, zero mean per 6-connected component",
               "coefficients": "face coefficients U[0.5,2], Dirichlet 0 outside"}
        for kind in modes:
            for _ in range(warmup):
                PW.timed_solve(g, kind)
            runs = [PW.timed_solve(g, kind) for _ in range(steps)]
            med = sorted(runs, key=lambda r: r["ms"])[len(runs) // 2]
            out[kind] = med
        for m in modes:
            if m != "plain" and "plain" in out:
                out[f"{m}_speedup_vs_plain"] = out["plain"]["ms"] / out[m]["ms"]
        return out
    finally:
        g.close()


def poisson_full_measure(steps: int, warmup: int) -> dict:
    """Time-to-1e-6 on the stated Poisson workload: every level-0 block of the 4096^3
    three-level layout (144,191 blocks, 4.72 G cells), plain FP32 MG-PCG and FP16-storage /
    FP32 iterative refinement from X = 0.  The two run in turn on one context, whose work
    vectors are released in between (both together need more than the GPU's memory)."""
    g, spec = PW.surface_layout_grid(None)
    try:
        bs = spec["bsx"]
        t0 = time.perf_counter()
        PW.setup_problem(g, bs)
        setup_s = time.perf_counter() - t0
        cells = int(g.info().nActive) * bs ** 3
        out = {"workload": "poisson-4096^3-bs32-full", "cells": cells,
               "mg_levels": [int(v) for v in g.mg_info()], "tolerance": 1e-6,
               "rhs": "N(0,1) per cell, zero mean per 6-connected component",
               "coefficients": "face coefficients U[0.5,2], Dirichlet 0 outside",
               "host_setup_s": setup_s}
        for kind in ("plain", "mixed"):
            for _ in range(warmup):
                PW.timed_solve(g, kind)
            runs = [PW.timed_solve(g, kind) for _ in range(steps)]
            out[kind] = sorted(runs, key=lambda r: r["ms"])[len(runs) // 2]
            g.poisson_release_work()
        out["mixed_speedup_vs_plain"] = out["plain"]["ms"] / out["mixed"]["ms"]
        # the operator launch shapes the autotuner picked (level, bytes per value, mode,
        # cells per thread, grid), during the warm-up solves
        out["operator_shapes"] = [list(t) for t in g.poisson_tuning()]
        n1 = cells // 8
        out["learned"] = (f"not run at this size: the network's level-1 buffers ({n1 * (52 + 32 + 2) * 4 / 1e9:.0f} GB "
                          f"of activations and gradients, {cells * 8 / 1e9:.0f} GB of level-0 staging) do not fit "
                          f"beside the solver's arrays; see poisson_crop96")
        return out
    finally:
        g.close()


def run_poisson(args, dist):
    if args.workload == "poisson-batch256":
        from msbg_gb300 import batch_workload as BW
        res = BW.run_batch(args.steps, args.warmup, WARMNET)
        if dist.rank != 0:
            return
        pl = res["plain"]
        line = {
            "metric": "batched Poisson solves/s (256 volumes, 1e-6)", "value": pl["solves_per_s"], "unit": "solves/s",
            "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": pl["batch_ms"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 (f64 dots)",
            "data": "synthetic", "config": {"workload": res["workload"], "cells": res["cells"],
                                            "l2": "inputs larger than L2 (no flush)"},
            "poisson_batch": res,
        }
        print(json.dumps(line), flush=True)
        return
    n_obj = {"poisson-crop96": 96, "poisson-crop12": 12}[args.workload]
    res = poisson_measure(n_obj, args.steps, args.warmup)
    if dist.rank != 0:
        return
    plain = res["plain"]
    line = {
        "metric": "time-to-1e-6 relative residual (plain FP32 MG-PCG)", "value": plain["ms"], "unit": "ms",
        "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": plain["ms"],
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32 (f64 dots)",
        "data": "synthetic", "config": {"workload": res["workload"], "cells": res["cells"],
                                        "l2": "inputs larger than L2 (no flush)"},
        "gpu_launches": plain["gpu_launches"], "poisson": res,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="surface4096",
                    choices=["surface4096", "surface4096-crop", "surface512", "poisson-crop96", "poisson-crop12",
                             "poisson-batch256"])
    ap.add_argument("--no-jacobi", action="store_true", help="skip the Jacobi-sweep throughput of the default run")
    ap.add_argument("--no-poisson", action="store_true",
                    help="skip the sparse Poisson time-to-1e-6 measurement of the default run")
    ap.add_argument("--variant", default="fast", choices=["fast", "exact"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--fp64-check", action=argparse.BooleanOptionalAction, default=True,
                    help="field error of the workload against an FP64 GPU run of the same algorithm")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--traffic-per-launch", type=float, default=None,
                    help="DRAM bytes per sweep launch from an ncu capture (reported as roofline.traffic)")
    args = ap.parse_args()
    dist = Dist()
    try:
        if args.workload.startswith("poisson"):
            if args.impl == "reference":
                if dist.rank == 0:
                    print(json.dumps({"impl": "reference", "unavailable":
                                      "the reference release has no Poisson solver driver"}), flush=True)
            else:
                run_poisson(args, dist)
            return
        spec = {"surface4096": W.SURFACE_4096, "surface4096-crop": W.SURFACE_4096_CROP,
                "surface512": W.SURFACE_512}[args.workload]
        if args.impl == "reference":
            run_reference(args, spec, dist)
        else:
            run_gpu(args, spec, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
