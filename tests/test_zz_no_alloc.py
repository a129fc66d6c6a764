"""mcg_objective_noalloc: the evaluation for callers that cannot allocate device memory
while they evaluate (fixed device-memory budgets, hosts whose device memory belongs to
another allocator, schedulers that cannot wait for cudaFree).  Its self-contact scratch is
a fixed __device__ array; its results must equal the allocating entry point's, call after
call, in both precision forms, and lattices or states beyond the array's limits must be
refused with a message naming what overflowed.

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


def test_noalloc_mixed_form_matches_the_allocating_entry_point(mcg):
    g = golden("ref242")
    cfg = g.cfg
    cfg.precision = abi.MCG_MIXED
    sol = mcg.Solver(cfg, g.lattice)
    for k in (3, 2):
        s = g.state(k)
        sol.set_state(plastic=s["plastic"])
        ref = sol.objective(s["z"], s["top"])
        rc, energy, grad, diag = noalloc(sol, s["z"], s["top"])
        assert rc == abi.MCG_OK, sol.lib.mcg_last_error(sol.h)
        assert abs(energy - ref["energy"]) <= TOL * abs(ref["energy"]), (k, energy, ref["energy"])
        assert rel_err(grad, ref["grad"]) <= TOL
        assert diag["contacts"] == ref["diag"]["contacts"]


def squeezed(mcg, lat, cfg, squeeze, sigma):
    z, pl = mcg.random_state(lat, sigma, 0.1, 0.02, 77)
    y = lat.x0[1::3]
    z[1::6] += -squeeze * (y - y.min()) / cfg.translation_scale
    z[lat.locked.astype(bool)] = 0
    return z, pl, lat.geometry.top0 - squeeze * lat.geometry.height + 1e-3


def test_noalloc_refuses_a_state_that_overflows_the_scratch_and_recovers(mcg):
    """An 8x8x8 cubic+BCC lattice (1,241 nodes, 7,281 shapes: inside the size limits) with
    1 mm struts squeezed to 40 % of its height has ~17,000 contacting pairs, more than the
    scratch's 8,192 contacts.  The evaluation is refused with a message naming what
    overflowed; the allocating entry point evaluates the same state; the next call at a state
    that fits succeeds and matches it."""
    cfg, spec = workloads.bcc((8, 8, 8), r0=1.0e-3, r1=1.0e-3)
    lat = mcg.generate_lattice(spec, cfg)
    sol = mcg.Solver(cfg, lat)
    z, pl, top = squeezed(mcg, lat, cfg, 0.6, 0.2)
    sol.set_state(plastic=pl)
    rc, _, _, _ = noalloc(sol, z, top)
    msg = sol.lib.mcg_last_error(sol.h).decode()
    print("overflow:", msg)
    assert rc == abi.MCG_ERR_CAPACITY
    assert "contacts" in msg or "candidate pairs" in msg
    ref = sol.objective(z, top)
    assert ref["diag"]["contacts"] > 8192
    z1, _, top1 = squeezed(mcg, lat, cfg, 0.05, 0.02)
    ref1 = sol.objective(z1, top1)
    rc, energy, grad, diag = noalloc(sol, z1, top1)
    assert rc == abi.MCG_OK, sol.lib.mcg_last_error(sol.h)
    assert abs(energy - ref1["energy"]) <= TOL * abs(ref1["energy"])
    assert rel_err(grad, ref1["grad"]) <= TOL


def test_noalloc_refuses_a_grid_beyond_its_bins(mcg):
    """An 11x11x11 cubic lattice (1,728 nodes, 6,480 shapes) spans ~18 grid cells per axis at
    the reference's grid cell: more than the scratch's 4,096 bins."""
    cfg, spec = workloads.bcc((11, 11, 11))
    spec.kind = abi.MCG_LATTICE_CUBIC
    lat = mcg.generate_lattice(spec, cfg)
    assert lat.n_nodes <= 4096 and lat.n_nodes + lat.n_beams <= 8192
    sol = mcg.Solver(cfg, lat)
    rc, _, _, _ = noalloc(sol, np.zeros(6 * lat.n_nodes), lat.geometry.top0)
    msg = sol.lib.mcg_last_error(sol.h).decode()
    print("bins:", msg)
    assert rc == abi.MCG_ERR_CAPACITY and "grid bins" in msg


def test_contact_queries_refuse_after_a_noalloc_evaluation(mcg):
    g = golden("ref242")
    s = g.state(3)
    sol = mcg.Solver(g.cfg, g.lattice)
    sol.set_state(plastic=s["plastic"])
    sol.objective(s["z"], s["top"])
    assert np.array_equal(sol.contact_pairs(), s["pairs"])
    rc, _, _, _ = noalloc(sol, s["z"], s["top"])
    assert rc == abi.MCG_OK
    with pytest.raises(mcg.MCGError) as e:
        sol.contact_pairs()
    assert e.value.status == abi.MCG_ERR_STATE
    sol.objective(s["z"], s["top"])  # an allocating evaluation makes them current again
    assert np.array_equal(sol.contact_pairs(), s["pairs"])


def test_noalloc_runs_beside_a_graph_capture_and_adds_nothing_to_it(mcg):
    """A caller may evaluate while one of its streams captures a CUDA graph: in relaxed
    capture mode on the capturing thread, and in thread-local mode from another thread.  The
    evaluation runs at once with unchanged results, and the capture still ends in a graph
    that holds only the caller's own work."""
    torch = pytest.importorskip("torch")
    import threading

    g = golden("ref242")
    s = g.state(3)
    sol = mcg.Solver(g.cfg, g.lattice)
    sol.set_state(plastic=s["plastic"])
    rc, e0, g0, _ = noalloc(sol, s["z"], s["top"])  # sets up before any capture
    assert rc == abi.MCG_OK, sol.lib.mcg_last_error(sol.h)
    x = torch.zeros(256, device="cuda")
    got = []
    for mode in ("relaxed", "thread_local"):
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, capture_error_mode=mode):
            x.add_(1.0)
            if mode == "relaxed":
                got.append(noalloc(sol, s["z"], s["top"]))
            else:
                t = threading.Thread(target=lambda: got.append(noalloc(sol, s["z"], s["top"])))
                t.start()
                t.join()
            assert torch.cuda.is_current_stream_capturing()
            x.add_(1.0)
        x.zero_()
        graph.replay()
        torch.cuda.synchronize()
        assert torch.all(x == 2.0).item(), mode  # the graph holds the two additions only
    for rc, energy, grad, _ in got:
        assert rc == abi.MCG_OK, sol.lib.mcg_last_error(sol.h)
        assert abs(energy - e0) <= 1e-14 * abs(e0)
        assert rel_err(grad, g0) <= 1e-14
