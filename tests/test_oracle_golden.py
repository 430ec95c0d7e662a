"""The CPU restatement (oracle/msbg_oracle.c) against golden vectors written by
the MSBG reference library itself (tests/golden/make_golden.py).

Integer outputs (levels, flags, active blocks, counts) must match bit for bit;
FP32 and uint16 fields within relative L2 1e-5 (uint16 compared as v/65535)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_l2

REL_TOL = 1e-5
NAMES = ["mcf8_f32", "mcf8_u16_odd", "jacobi_rb_f32", "jacobi_pp_f32_odd", "diff_pp_f32",
         "lapl8_f32", "pmj8_f32"]


def _run(port, golden, name):
    chan, lt, it, dt, al = golden[f"meta_{name}"]
    storage = port.F32 if int(chan) == 0 else port.U16
    return storage, port.surface_pipeline(golden["points"], int(golden["res"]), int(golden["bsx"]),
                                          storage=storage, n_iter=int(it), lapl_typ=int(lt),
                                          dt=float(dt), anis_alpha=float(al))


@pytest.mark.parametrize("name", NAMES)
def test_port_matches_reference_golden(port, golden, name):
    storage, r = _run(port, golden, name)
    assert np.array_equal(r.levels, golden["levels"])
    assert np.array_equal(r.flags, golden["flags"])
    assert np.array_equal(r.active_bids, golden["active_bids"])
    assert r.n_act_particles == int(golden["n_act_particles"])
    fin = golden["final_f32"] if storage == port.F32 else golden["final_u16"]
    want = golden[f"pde_{name}"]
    if storage == port.F32:
        assert rel_l2(r.after_finalize, fin) <= REL_TOL
        assert rel_l2(r.after_pde, want) <= REL_TOL
    else:
        # a one-quantum difference in the splat minimum grows through sqrt() near
        # the particle centre, hence a few quanta of slack on the max difference
        assert np.abs(r.after_finalize.astype(np.int64) - fin.astype(np.int64)).max() <= 8
        assert np.abs(r.after_pde.astype(np.int64) - want.astype(np.int64)).max() <= 8
        assert rel_l2(port.to_float(storage, r.after_finalize), port.to_float(storage, fin)) <= REL_TOL
        assert rel_l2(port.to_float(storage, r.after_pde), port.to_float(storage, want)) <= REL_TOL


def test_port_abort_rule_golden(port, golden):
    r = port.surface_pipeline(golden["points"], int(golden["res"]), int(golden["bsx"]),
                              storage=port.F32, n_iter=2, dt=0.1,
                              levels_in=golden["abort_levels_in"])
    assert r.n_aborted > 0
    assert np.array_equal(r.levels, golden["abort_levels"])
    assert np.array_equal(r.active_bids, golden["abort_active_bids"])
    assert rel_l2(r.after_finalize, golden["abort_final_f32"]) <= REL_TOL
    assert rel_l2(r.after_pde, golden["abort_pde_f32"]) <= REL_TOL


@pytest.mark.parametrize("nl", [3, 4])
def test_port_refinement_map_golden(port, golden, nl):
    lv, per = port.regularize(golden[f"lvl{nl}_in"], 8, 8, 8, nl)
    assert np.array_equal(lv, golden[f"lvl{nl}_out"])
    assert np.array_equal(per, golden[f"lvl{nl}_per_level"])
    assert np.array_equal(port.block_flags(lv, 8, 8, 8), golden[f"lvl{nl}_flags"])


def test_port_particles_per_block_golden(port, golden):
    """particlesPerBlock restated: the listed points are the demo's nActParticles (the
    reference's own count of the points its marking loop keeps), each in the list of the
    block that contains it."""
    res, bsx = int(golden["res"]), int(golden["bsx"])
    pts = golden["points"]
    g = port.grid(res, res, res, bsx, port.F32)
    off, idx = port.particles_per_block(g, pts)
    assert off[-1] == len(idx) == int(golden["n_act_particles"])
    nb = res // bsx
    ip = pts[idx].astype(np.int64)
    owner = ((ip[:, 2] // bsx) * nb + ip[:, 1] // bsx) * nb + ip[:, 0] // bsx
    assert np.array_equal(owner, np.repeat(np.arange(nb ** 3), np.diff(off)))
