"""Pins the CPU restatement (oracle/mco_oracle.cpp) to the reference solver.

The golden fixtures were produced by the reference's own MC/src/sim.cpp (see
tests/golden/make_golden.py); the restatement must reproduce them bit for bit on the
machine they were made on (x86-64, g++ -O3, no FMA contraction).  Where the reference
sources are present the two are also compared live on fresh states.
"""
import numpy as np
import pytest

from conftest import golden
from falling_dice_gb300 import abi

GOLDEN_CASES = ["ref242", "cubic6", "bcc4"]


def model_for(orc, g):
    if g.name == "ref242":
        return orc.Model("mco", g.cfg)  # the restated builder must regenerate the lattice
    return orc.Model("mco", g.cfg, lattice=g.lattice)


def same_bits(a, b):
    a = np.ascontiguousarray(a, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


def test_restated_builder_reproduces_reference_lattice(mco):
    g = golden("ref242")
    m = mco.Model("mco", g.cfg)
    lat = m.export()
    for f in lat.FIELDS:
        ref = getattr(g.lattice, f)
        got = getattr(lat, f)
        assert got.shape == ref.shape and np.array_equal(got.view(np.uint8), ref.view(np.uint8)), f
    geo = [getattr(lat.geometry, n) for n, _ in abi.Geometry._fields_]
    assert same_bits(geo, g.d["lat_geometry"])
    assert (m.n_nodes, m.n_beams) == (365, 456)


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_restated_objective_bitwise(mco, case):
    g = golden(case)
    m = model_for(mco, g)
    for k in range(g.n_states):
        s = g.state(k)
        m.set_state(plastic=s["plastic"])
        r = m.objective(s["z"], s["top"], s["trials"])
        assert same_bits([r["energy"]], [s["energy"]]), (case, k)
        assert same_bits(r["grad"], s["grad"]), (case, k)
        d = r["diag"]
        got = [d["elastic"], d["plastic"], d["contact"], d["reaction"], d["max_pen"], d["contacts"]]
        assert same_bits(got, s["diag"]), (case, k)
        if s["trials"]:
            assert same_bits(r["trial_next"], s["trial_next"])
            assert same_bits(r["trial_aux"], s["trial_aux"])
            assert np.array_equal(r["trial_flags"], s["trial_flags"])
        if np.isfinite(s["energy"]):  # with a NaN coordinate the reference's grid cell is undefined
            assert np.array_equal(m.contact_pairs(s["z"]), s["pairs"]), (case, k)


@pytest.mark.parametrize("case", ["ref242", "cubic6"])
def test_restated_minimize_bitwise(mco, case):
    g = golden(case)
    m = model_for(mco, g)
    z, st, fe, fdg = m.minimize(float(g.d["min_top"][0]), np.zeros(6 * g.lattice.n_nodes))
    assert same_bits(z, g.d["min_z"])
    ref = g.d["min_stats"]
    assert [st["iterations"], st["backtracks"]] == [int(ref[0]), int(ref[1])]
    assert same_bits([st["rms"], st["max"], st["energy"]], ref[2:5])
    assert same_bits([fe, fdg["reaction"], fdg["max_pen"]], g.d["min_final"][[0, 4, 5]])


def test_restated_verification_checks(mco):
    g = golden("ref242")
    m = model_for(mco, g)
    assert same_bits([m.rigid_rotation_error()], g.d["rigid_error"])
    assert same_bits([m.gradient_check_error()], g.d["fd_error"])


def test_restated_run_reproduces_reference_and_published_numbers(mco):
    """Full 20/14 load/unload run of the reference specimen (about 45 s on one core)."""
    g = golden("ref242")
    m = model_for(mco, g)
    rc, frames = m.run()
    assert rc == 0
    ref = g.frames()
    assert len(frames) == len(ref) == 35
    for f, r in zip(frames, ref):
        for k in r:
            assert same_bits([f[k]], [r[k]]), k
    # published step-refinement row 20/14 (MC/docs/VALIDATION.md:47)
    peak = max(f["reaction_force"] for f in frames)
    last = frames[-1]
    assert round(peak, 3) == 79.482
    assert round(last["loading_work"], 3) == 0.667
    assert round(last["dissipated_work"], 3) == 0.137
    assert round(100 * last["permanent_set"], 2) == 10.71


def test_restatement_matches_reference_live(mco, ref_oracle):
    """Fresh random states on both solvers (skipped where the reference is absent)."""
    g = golden("ref242")
    a = mco.Model("mco", g.cfg)
    b = mco.Model("ref", g.cfg)
    rng = np.random.default_rng(99)
    lk = g.lattice.locked.astype(bool)
    for k in range(4):
        z = rng.normal(0, 0.03 * (k + 1), 6 * a.n_nodes)
        z[lk] = 0
        pl = rng.uniform(-0.01, 0.01, 7 * a.n_beams)
        a.set_state(plastic=pl)
        b.set_state(plastic=pl)
        top = g.lattice.geometry.top0 - 0.003 * k
        ra, rb = a.objective(z, top, True), b.objective(z, top, True)
        assert same_bits([ra["energy"]], [rb["energy"]])
        assert same_bits(ra["grad"], rb["grad"])
        assert same_bits(ra["trial_next"], rb["trial_next"])
        assert np.array_equal(a.contact_pairs(z), b.contact_pairs(z))


def test_oracle_flags_nonfinite_energy(mco):
    """A NaN coordinate gives energy = +inf and an all-zero gradient (sim.cpp:172)."""
    g = golden("ref242")
    s = g.state(5)
    assert np.isinf(s["energy"]) and not np.any(s["grad"])


@pytest.mark.parametrize("which", ["cubic6", "bcc32", "small_uniform"])
def test_specimen_restatement_reproduces_the_product_generator(mco, mcg, which):
    """The timed CPU baseline builds its inputs with the oracle's own restatement of the
    workload generator (oracle/specimens.cpp), so that it loads no product library; the
    arrays and the seeded deformed state must be the product's, bit for bit."""
    from falling_dice_gb300 import workloads
    if which == "small_uniform":
        cfg, spec = workloads.bcc((5, 4, 3))
    else:
        cfg, spec = getattr(workloads, which)()
    lat = mcg.generate_lattice(spec, cfg)
    got = mco.Model("mco", cfg, lattice=spec).export()
    for f in lat.FIELDS:
        a, b = getattr(lat, f), getattr(got, f)
        assert a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8)), f
    for n, _ in abi.Geometry._fields_:
        assert same_bits([getattr(lat.geometry, n)], [getattr(got.geometry, n)]), n
    z, pl = mcg.random_state(lat, **workloads.DEFORM)
    zo, plo = mco.random_state(lat.n_nodes, lat.n_beams, lat.locked, **workloads.DEFORM)
    assert same_bits(z, zo) and same_bits(pl, plo)


def test_objective_hook_is_transparent(mco):
    """The seam plumbing on the CPU: a restatement whose objective hook forwards to a second,
    plain restatement (through C callbacks with mcg_objective's and mcg_set_state's
    signatures) runs minimize and a short load/unload run bit for bit like the plain one, and
    keeps the plain one's state in step through the state hook."""
    import ctypes as C
    g = golden("cubic6")
    cfg = g.cfg
    cfg.load_steps, cfg.unload_steps = 6, 3
    inner = mco.Model("mco", cfg, lattice=g.lattice)
    dptr = C.POINTER(C.c_double)
    OBJ = C.CFUNCTYPE(C.c_int, C.c_void_p, dptr, C.c_double, C.c_int, dptr, dptr, C.POINTER(abi.Diag),
                      dptr, dptr, C.POINTER(C.c_uint8))
    ST = C.CFUNCTYPE(C.c_int, C.c_void_p, dptr, dptr, dptr)

    def objective(_ctx, z, top, trials, energy, grad, diag, nxt, aux, flags):
        energy[0] = inner.lib.orc_objective(inner.h, z, top, trials, grad, diag, nxt, aux, flags)
        return 0

    def state(_ctx, bx, br, pl):
        inner.lib.orc_set_state(inner.h, bx, br, pl)
        return 0
    obj_cb, st_cb = OBJ(objective), ST(state)
    hooked = mco.Model("mco", cfg, lattice=g.lattice)
    hooked.set_objective_hook(obj_cb, st_cb, None)
    plain = mco.Model("mco", cfg, lattice=g.lattice)
    top = float(g.d["min_top"][0])
    z0 = np.zeros(6 * g.lattice.n_nodes)
    a, b = hooked.minimize(top, z0), plain.minimize(top, z0)
    assert same_bits(a[0], b[0]) and a[1] == b[1] and a[2] == b[2]
    rc_a, fa = hooked.run()
    rc_b, fb = plain.run()
    assert rc_a == rc_b == 0 and fa == fb
    assert all(same_bits(x, y) for x, y in zip(inner.get_state(), plain.get_state()))
    status, calls = hooked.hook_status()
    assert status == 0 and calls > 100
