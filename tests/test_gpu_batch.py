"""Batched contexts (mcg_upload_batch): lattices of different sizes and yield stresses in
one context, evaluated and solved in the same launches, against each lattice in a context
of its own.  An instance's arithmetic never mixes with another's (blocks never straddle two
lattices, per-instance reductions run in the same order, contact sums are ordered by shape
pair), so the results must agree bit for bit."""
import numpy as np
import pytest

from falling_dice_gb300 import abi, workloads

pytestmark = pytest.mark.gpu

SPECS = [((4, 4, 4), 40e6, 11), ((5, 3, 4), 55e6, 12), ((3, 5, 3), 30e6, 13), ((6, 4, 5), 65e6, 14)]


def make(mcg, load_steps=0, unload_steps=0, max_strain=0.2, precision=abi.MCG_FP64):
    cfg, _ = workloads.bcc((4, 4, 4), contact_stiffness=workloads.CONTACT_STIFF)
    cfg.load_steps, cfg.unload_steps, cfg.max_strain = load_steps, unload_steps, max_strain
    cfg.precision = precision
    lats = []
    for cells, _, seed in SPECS:
        _, spec = workloads.bcc(cells, 0.3e-3, 0.5e-3, 0.03, abi.MCG_RADIUS_GRADED_Y)
        spec.seed = seed
        lats.append(mcg.generate_lattice(spec, cfg))
    return cfg, lats, [y for _, y, _ in SPECS]


def single_cfg(cfg, y):
    c = abi.Config.from_buffer_copy(cfg)
    c.material.yield_ = y
    return c


@pytest.mark.parametrize("precision", [abi.MCG_FP64, abi.MCG_MIXED])
def test_batched_evaluation_is_bitwise_the_single_one(mcg, precision):
    cfg, lats, ys = make(mcg, precision=precision)
    states = [mcg.random_state(lat, 0.04, 0.08, 0.02, 1000 + k) for k, lat in enumerate(lats)]
    tops = [lat.geometry.top0 - 0.002 for lat in lats]
    batch = mcg.BatchSolver(cfg, lats, yields=ys)
    batch.set_state(plastic=np.concatenate([pl for _, pl in states]))
    got = batch.objective(np.concatenate([z for z, _ in states]), tops)
    off = batch.node_offsets
    for k, lat in enumerate(lats):
        sol = mcg.Solver(single_cfg(cfg, ys[k]), lat)
        sol.set_state(plastic=states[k][1])
        ref = sol.objective(states[k][0], tops[k])
        assert got["energy"][k] == ref["energy"], (k, got["energy"][k], ref["energy"])
        assert np.array_equal(got["grad"][6 * off[k]:6 * off[k + 1]], ref["grad"]), k
        assert got["diag"][k] == ref["diag"], k


def test_batched_run_is_bitwise_the_single_runs(mcg):
    cfg, lats, ys = make(mcg, load_steps=10, unload_steps=4, max_strain=0.25)
    batch = mcg.BatchSolver(cfg, lats, yields=ys)
    status, runs = batch.run()
    for k, lat in enumerate(lats):
        rc, ref = mcg.Solver(single_cfg(cfg, ys[k]), lat).run()
        assert status[k] == rc
        assert len(runs[k]) == len(ref) and len(ref) == 15
        keys = sorted(ref[0].keys())
        a = np.array([[f[q] for q in keys] for f in runs[k]])
        b = np.array([[f[q] for q in keys] for f in ref])
        assert np.array_equal(a, b), (k, np.argwhere(a != b)[:5])


def test_single_lattice_functions_refuse_a_batch(mcg):
    cfg, lats, ys = make(mcg)
    batch = mcg.BatchSolver(cfg, lats[:2], yields=ys[:2])
    assert batch.lib.mcg_instance_count(batch.h) == 2
    with pytest.raises(mcg.MCGError):
        mcg.Solver.objective(batch, np.zeros(6 * batch.n_nodes), 0.0)


def test_autotuned_shapes_leave_evaluations_and_runs_unchanged(mcg):
    """mcg_autotune times broad-phase cells and pair grids and keeps the fastest; the choice
    must not change an evaluation or a run by a bit (it checks its candidates itself)."""
    cfg, lats, ys = make(mcg, load_steps=6, unload_steps=2, max_strain=0.25)
    states = [mcg.random_state(lat, 0.04, 0.08, 0.02, 2000 + k) for k, lat in enumerate(lats)]
    z = np.concatenate([zz for zz, _ in states])
    tops = [lat.geometry.top0 - 0.003 for lat in lats]
    plain = mcg.BatchSolver(cfg, lats, yields=ys)
    ref = plain.objective(z, tops)
    _, ref_runs = plain.run()
    tuned = mcg.BatchSolver(cfg, lats, yields=ys)
    t = tuned.autotune(z, tops, reps=2)
    # the fastest, or within 1 % of it (the tie-break that keeps repeated tunings in agreement)
    assert t["tried"] >= 4 and t["ms_chosen"] <= t["ms_default"] * 1.0101
    assert t["cell"] > 0 and t["pair_blocks"] >= 1
    got = tuned.objective(z, tops)
    assert np.array_equal(got["energy"], ref["energy"])
    assert np.array_equal(got["grad"], ref["grad"])
    _, runs = tuned.run()
    for k in range(len(lats)):
        assert [f["reaction_force"] for f in runs[k]] == [f["reaction_force"] for f in ref_runs[k]], k
    with pytest.raises(ValueError):
        tuned.autotune(z[:-1])


def test_fixed_shapes_leave_evaluations_unchanged(mcg):
    """mcg_set_contact_shapes (a saved tuning, or shapes pinned for a profiler) changes how
    the broad phase splits its work, not an evaluation."""
    cfg, lats, ys = make(mcg)
    states = [mcg.random_state(lat, 0.04, 0.08, 0.02, 3000 + k) for k, lat in enumerate(lats)]
    z = np.concatenate([zz for zz, _ in states])
    tops = [lat.geometry.top0 - 0.003 for lat in lats]
    ref = mcg.BatchSolver(cfg, lats, yields=ys).objective(z, tops)
    for cell, blocks in ((0.0, 0), (0.004, 152), (0.0056, 1)):
        b = mcg.BatchSolver(cfg, lats, yields=ys)
        b.set_contact_shapes(cell, blocks)
        got = b.objective(z, tops)
        assert np.array_equal(got["energy"], ref["energy"]), (cell, blocks)
        assert np.array_equal(got["grad"], ref["grad"]), (cell, blocks)
    with pytest.raises(mcg.MCGError):
        b.set_contact_shapes(-1.0, 0)


@pytest.mark.parametrize("precision,beam_blocks", [(0, (1, 2, 3)), (1, (3, 4, 5, 6, -3, -4))])
def test_kernel_occupancy_variants_leave_evaluations_unchanged(mcg, precision, beam_blocks):
    """The beam kernel's and the gather's occupancy variants (CTAs per SM, which set their
    register budgets; mcg_set_kernel_shapes / mcg_autotune), and the mixed beam kernel with
    its records staged by bulk copies (-3, -4), do the same arithmetic: every variant gives the
    default's evaluation bit for bit, in both precision forms."""
    cfg, lats, ys = make(mcg)
    cfg.precision = precision
    states = [mcg.random_state(lat, 0.04, 0.08, 0.02, 4000 + k) for k, lat in enumerate(lats)]
    z = np.concatenate([zz for zz, _ in states])
    tops = [lat.geometry.top0 - 0.003 for lat in lats]
    ref = mcg.BatchSolver(cfg, lats, yields=ys).objective(z, tops)
    b = mcg.BatchSolver(cfg, lats, yields=ys)
    for bb in beam_blocks:
        for gb in (1, 2, 4):
            b.set_kernel_shapes(bb, gb)
            got = b.objective(z, tops)
            assert np.array_equal(got["energy"], ref["energy"]), (bb, gb)
            assert np.array_equal(got["grad"], ref["grad"]), (bb, gb)
    with pytest.raises(mcg.MCGError):
        b.set_kernel_shapes(7, 1)
    t = b.autotune(z, tops, reps=2)
    assert t["beam_blocks"] in beam_blocks and t["gather_blocks"] in (1, 2, 4)
    got = b.objective(z, tops)
    assert np.array_equal(got["grad"], ref["grad"])


def test_batched_run_is_the_same_with_host_stepped_rounds(mcg):
    """The batch run with its rounds in the device-resident graph loop (the default; the
    loop returns to the host whenever a lattice finishes an increment) and stepped from the
    host: the same frames bit for bit."""
    cfg, lats, ys = make(mcg, load_steps=10, unload_steps=4, max_strain=0.25)
    out = {}
    for device in (True, False):
        batch = mcg.BatchSolver(cfg, lats, yields=ys)
        batch.set_solver_loop(device)
        out[device] = batch.run()
        assert batch.solver_loop()[0] == device, batch.solver_loop()[1]
    (sa, ra), (sb, rb) = out[True], out[False]
    assert list(sa) == list(sb)
    for k in range(len(lats)):
        assert ra[k] == rb[k], k
