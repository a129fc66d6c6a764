"""The drop-in seam: the reference's own solver driving the GPU energy/gradient unchanged.

The reference keeps its evaluation behind Objective Simulator::objective(z, top, trials)
(MC/include/sim.hpp:49), called by minimize (MC/src/sim.cpp:176,179,210) and gradientCheck
(:552,564-565).  The integration replaces only that member's body with a call to
mcg_objective and re-sends the base state after commit (MC/src/sim.cpp:212) with
mcg_set_state.  Here the CPU restatement of the reference (bit-identical to it,
tests/test_oracle.py) is patched exactly so: its objective hook is libmcg's mcg_objective
itself (same C signature, the GPU context as first argument) and its state hook is
mcg_set_state.  minimize, run, commit, the bisection and the checks are the restatement's
unchanged code.  The results must meet the same bars as the device-resident solver.
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden, rel_err
from test_gpu_solver import run_errors, short_run_cfg

pytestmark = pytest.mark.gpu


def seamed(fd, mco, cfg, lattice):
    """(restatement model whose objective is the GPU's, the GPU solver behind it)."""
    sol = fd.Solver(cfg, lattice)
    m = mco.Model("mco", cfg, lattice=lattice)
    m.set_objective_hook(sol.lib.mcg_objective, sol.lib.mcg_set_state, sol.h)
    return m, sol


def test_reference_minimize_over_the_gpu_objective(mcg, mco):
    g = golden("cubic6")
    m, sol = seamed(mcg, mco, g.cfg, g.lattice)
    top = float(g.d["min_top"][0])
    z, st, fe, fdg = m.minimize(top, np.zeros(6 * g.lattice.n_nodes))
    status, calls = m.hook_status()
    ref = g.d["min_stats"]
    print("seam minimize:", st, "GPU evaluations", calls)
    assert status == 0 and calls > st["iterations"]
    assert st["converged"] == 1 and st["iterations"] == int(ref[0])
    assert rel_err(z, g.d["min_z"]) <= 1e-8
    assert abs(fe - g.d["min_final"][0]) <= 1e-10 * abs(g.d["min_final"][0])
    sol.close()


def test_reference_run_over_the_gpu_objective(mcg, mco):
    """The 6x6x6 specimen's 200 + 200 increment run by the reference driver over the GPU
    objective, against the reference's own run, at the bars of the device-resident run."""
    g = golden("cubic6")
    run = np.load(os.path.join(GOLDEN, "cubic6_run.npz"))
    keys = [str(k) for k in run["frame_keys"]]
    ref = [dict(zip(keys, row)) for row in run["run_frames"]]
    m, sol = seamed(mcg, mco, g.cfg, g.lattice)
    rc, frames = m.run()
    status, calls = m.hook_status()
    assert status == 0 and rc == 0 and len(frames) == len(ref)
    errs = run_errors(frames, ref)
    print("seam run errors vs reference:", errs, "GPU evaluations", calls)
    assert errs["peak_force"] <= 1e-8 and errs["loading_work"] <= 1e-8, errs
    assert errs["dissipated_work"] <= 1e-6 and errs["permanent_set"] <= 1e-5, errs
    assert errs["curve"] <= 1e-5, errs
    # the GPU context holds the state the driver committed last
    bx, br, pl = sol.get_state()
    bxo, bro, plo = m.get_state()
    assert np.array_equal(bx, bxo) and np.array_equal(br, bro) and np.array_equal(pl, plo)
    sol.close()


def test_reference_bisection_over_the_gpu_objective(mcg, mco):
    """The reference driver's bisection of failed increments over the GPU objective takes the
    path it takes over its own objective."""
    g = golden("cubic6")
    for max_iterations, status in ((39, 0), (6, 5)):
        cfg = short_run_cfg(g, max_iterations)
        rc_o, fo = mco.Model("mco", cfg, lattice=g.lattice).run()
        m, sol = seamed(mcg, mco, cfg, g.lattice)
        rc, fr = m.run()
        assert m.hook_status()[0] == 0
        assert rc == rc_o == status and len(fr) == len(fo)
        assert [f["platen_y"] for f in fr] == [f["platen_y"] for f in fo]
        assert [f["refinement"] for f in fr] == [f["refinement"] for f in fo]
        sol.close()


def test_reference_gradient_check_over_the_gpu_objective(mcg, mco):
    """gradientCheck (sim.cpp:538-577) is a caller of objective: over the GPU objective it
    passes, as over the reference's (tests/golden/ref242.npz)."""
    g = golden("ref242")
    m, sol = seamed(mcg, mco, g.cfg, g.lattice)
    err = m.gradient_check_error()
    ref = float(g.d["fd_error"][0])
    print(f"seam gradient check: {err:.3e} (reference {ref:.3e})")
    assert m.hook_status()[0] == 0
    assert err < 0.075 and err <= max(10 * ref, 1e-4)
    sol.close()


def test_hook_errors_reach_the_driver_as_a_rejected_evaluation(mcg, mco):
    """A failing GPU call (here: a context without a topology) reads as a non-finite
    evaluation, which the reference driver rejects, and its status is kept."""
    g = golden("cubic6")
    lib = mcg.load()
    h = C.c_void_p()
    assert lib.mcg_create(C.byref(g.cfg), 0, C.byref(h)) == 0
    m = mco.Model("mco", g.cfg, lattice=g.lattice)
    m.set_objective_hook(lib.mcg_objective, None, h)
    e = m.objective(np.zeros(6 * g.lattice.n_nodes), g.lattice.geometry.top0)
    assert np.isinf(e["energy"]) and not np.any(e["grad"])
    assert m.hook_status()[0] == mcg.abi.MCG_ERR_STATE
    lib.mcg_destroy(h)
