"""The C++ binding a maintainer adds to the reference.

CPU: the header compiles as C11 and as C++17, and the code block of INTEGRATION.md section 2
(the demo's pipeline through the header-only facade msbg_gpu::MultiresSparseGrid, with the
reference's method names and argument order) compiles and links as one translation unit with
tests/cpp/facade_main.cpp.  GPU: that program runs and gives the same active blocks, the same
swept field bit for bit and the same dot products as the Python binding of the same calls.
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from msbg_gb300 import workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")
LIBDIR = os.path.join(ROOT, "msbg_gb300", "lib")
CUDA_LIB = "/usr/local/cuda/lib64"


def _snippet() -> str:
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    sec = text[text.index("## 2. Binding"):text.index("## 3.")]
    blocks = re.findall(r"```cpp\n(.*?)```", sec, re.S)
    assert len(blocks) == 1, "section 2 holds one C++ block"
    return blocks[0]


def _compile(out_dir: str) -> str:
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    if not os.path.isfile(os.path.join(LIBDIR, "libmsbg_gpu.so")):
        pytest.skip("libmsbg_gpu.so not built")
    src = os.path.join(out_dir, "facade_demo.cpp")
    with open(src, "w") as f:
        f.write(_snippet())
        f.write(open(os.path.join(ROOT, "tests", "cpp", "facade_main.cpp")).read())
    exe = os.path.join(out_dir, "facade_demo")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", INC, src, "-o", exe, "-L", LIBDIR,
           "-lmsbg_gpu", f"-Wl,-rpath,{LIBDIR}"]
    if os.path.isdir(CUDA_LIB):
        cmd += ["-L", CUDA_LIB, "-lcudart", f"-Wl,-rpath,{CUDA_LIB}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_header_compiles_as_c_and_cpp(tmp_path):
    if not shutil.which("gcc") or not shutil.which("g++"):
        pytest.skip("no host compiler")
    c = tmp_path / "h.c"
    c.write_text('#include "msbg_gpu.h"\nint main(void) { return MSBG_GPU_ABI_VERSION == 2 ? 0 : 1; }\n')
    r = subprocess.run(["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I", INC, str(c)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    cc = tmp_path / "h.cpp"
    cc.write_text('#include "msbg_gpu.hpp"\nint main() { return 0; }\n')
    r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I", INC, str(cc)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_integration_snippet_compiles_and_links(tmp_path):
    exe = _compile(str(tmp_path))
    assert os.access(exe, os.X_OK)


@pytest.mark.gpu
def test_integration_snippet_runs_like_the_python_binding(gpulib, tmp_path):
    G = gpulib
    exe = _compile(str(tmp_path))
    res, bsx, n_iter, dt = 128, 16, 4, 0.1
    pts = W.sphere_cloud(res, 6, 4000, seed=W.workload_seed(7, 1))
    pf = tmp_path / "pts.f32"
    pts.astype(np.float32).tofile(pf)
    out = tmp_path / "out.bin"
    r = subprocess.run([exe, str(pf), str(res), str(bsx), str(n_iter), str(dt), str(out)], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    buf = out.read_bytes()
    na = int(np.frombuffer(buf, np.int64, 1, 0)[0])
    act = np.frombuffer(buf, np.int32, na, 8)
    dens = np.frombuffer(buf, np.float32, na * bsx ** 3, 8 + 4 * na).reshape(na, bsx ** 3)
    dots = np.frombuffer(buf, np.float64, 3, 8 + 4 * na + 4 * na * bsx ** 3)

    g = G.MultiresSparseGrid(res, res, res, bsx, 3, G.F32)
    try:
        d = g.to_device(pts)
        g.mark_points(d, len(pts), 4.0)
        g.levels_from_marks()
        g.regularizeRefinementMap()
        g.setRefinementMap(1.0)
        g.splat(d, len(pts), 2.0, 2.0)
        g.splat_finalize(2.0, 2.0)
        want_act = g.active_blocks()
        g.applyChannelPdeFast(0, blockList=want_act, laplTyp=G.LAPL_MCF_8COLOR, doConstrZeroOne=1,
                              numIter=n_iter, timeStep=dt)
        want_dens = g.payload(0)
        assert np.array_equal(act, want_act)
        assert np.array_equal(dens.view(np.uint32), want_dens.view(np.uint32))
        for c in range(1, 8):
            g.channel_create(c, G.F32)
        g.poisson_procedural_coefficients(4242, 4, 5, 6, 7)
        g.upload_payload(want_dens, 1)
        g.upload_payload(want_dens, 2)
        dyx = g.multiplyLaplacianMatrixOpt(0, 0, 1, 2, 0.0, 3, withDotprod=True)
        half = want_act[::2]
        g.relax(0, 0, 0, 1, 2, 0, 1, blockList=half)
        want = [dyx, g.dotProdChannel(1, 2), g.dotProdChannel(1, 3, 0, half)]
        assert np.array_equal(dots, np.array(want)), (dots, want)
    finally:
        g.close()
