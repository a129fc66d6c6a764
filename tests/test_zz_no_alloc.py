"""mcg_objective_noalloc: the evaluation for callers that cannot allocate device memory
while they evaluate (stream capture, fixed-budget loops, foreign allocators).  Its
self-contact scratch is a fixed __device__ array; its results must equal the allocating
entry point's, call after call, and lattices beyond the array's limits must be refused.

This file is collected last on purpose, so that a run stopping at its first failure has
already run every other test."""
import ctypes as C

import numpy as np
import pytest

from conftest import golden, rel_err
from falling_dice_gb300 import abi, workloads

pytestmark = pytest.mark.gpu

TOL = 1e-10


def noalloc(sol, z, top):
    z = np.ascontiguousarray(z, dtype=np.float64)
    e = C.c_double()
    grad = np.zeros(6 * sol.n_nodes)
    diag = abi.Diag()
    d = C.POINTER(C.c_double)
    rc = sol.lib.mcg_objective_noalloc(sol.h, z.ctypes.data_as(d), top, C.byref(e), grad.ctypes.data_as(d),
                                       C.byref(diag))
    return rc, e.value, grad, diag.as_dict()


def test_noalloc_matches_the_allocating_entry_point_on_consecutive_calls(mcg):
    g = golden("ref242")
    sol = mcg.Solver(g.cfg, g.lattice)
    for k in (3, 2, 3):  # consecutive calls reuse the array left by the previous one
        s = g.state(k)
        sol.set_state(plastic=s["plastic"])
        ref = sol.objective(s["z"], s["top"])
        rc, energy, grad, diag = noalloc(sol, s["z"], s["top"])
        assert rc == abi.MCG_OK, sol.lib.mcg_last_error(sol.h)
        assert abs(energy - ref["energy"]) <= TOL * abs(ref["energy"]), (k, energy, ref["energy"])
        assert rel_err(grad, ref["grad"]) <= TOL, (k, rel_err(grad, ref["grad"]))
        assert diag["contacts"] == ref["diag"]["contacts"] and diag["max_pen"] == ref["diag"]["max_pen"]
        assert abs(diag["reaction"] - ref["diag"]["reaction"]) <= TOL * max(abs(ref["diag"]["reaction"]), 1e-12)
        # and against the reference solver's own output for this state
        assert abs(energy - s["energy"]) <= TOL * abs(s["energy"])


def test_noalloc_refuses_lattices_beyond_its_scratch(mcg):
    cfg, spec = workloads.bcc((12, 12, 6))  # 2047 nodes, 10110 beams: more shapes than 8192
    lat = mcg.generate_lattice(spec, cfg)
    sol = mcg.Solver(cfg, lat)
    rc, _, _, _ = noalloc(sol, np.zeros(6 * lat.n_nodes), lat.geometry.top0)
    assert rc == abi.MCG_ERR_CAPACITY
    assert b"fixed scratch" in sol.lib.mcg_last_error(sol.h)
