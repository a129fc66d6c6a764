"""The mixed-precision form (FP32 bulk arithmetic, FP64 base state and reductions)
against the plain FP64 form, which is itself pinned to the reference.

Bars: per evaluation, energy within 1e-6 and the gradient within 1e-5 relative (2-norm);
the 6x6x6 cubic run's peak force and absorbed energy within 1e-5 of the FP64 run."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden, rel_err
from falling_dice_gb300 import abi, workloads

pytestmark = pytest.mark.gpu


def mixed_cfg(cfg):
    cfg.precision = abi.MCG_MIXED
    return cfg


@pytest.mark.parametrize("case", ["ref242", "cubic6", "bcc4"])
def test_mixed_evaluation_matches_fp64(mcg, case):
    g = golden(case)
    f64 = mcg.Solver(g.cfg, g.lattice)
    mix = mcg.Solver(mixed_cfg(g.cfg), g.lattice)
    for k in range(g.n_states):
        s = g.state(k)
        if not np.isfinite(s["energy"]):
            continue
        if case == "ref242" and k == 4:
            continue  # a degenerate (zero-length) beam: below FP32 position resolution
        for sol in (f64, mix):
            sol.set_state(plastic=s["plastic"])
        a = f64.objective(s["z"], s["top"], True)
        b = mix.objective(s["z"], s["top"], True)
        e_err = abs(b["energy"] - a["energy"]) / abs(a["energy"])
        g_err = rel_err(b["grad"], a["grad"])
        print(case, k, "energy", e_err, "grad", g_err, "contacts", a["diag"]["contacts"], b["diag"]["contacts"])
        assert e_err <= 1e-6, (case, k, e_err)
        assert g_err <= 1e-5, (case, k, g_err)
        assert abs(b["diag"]["reaction"] - a["diag"]["reaction"]) <= 1e-5 * max(abs(a["diag"]["reaction"]), 1e-9)
        assert b["diag"]["contacts"] == a["diag"]["contacts"]
        assert np.array_equal(b["trial_flags"], a["trial_flags"]) or \
            np.mean(b["trial_flags"] != a["trial_flags"]) < 1e-3


def test_mixed_evaluation_at_full_size(mcg):
    """The 64x64x32 cubic+BCC workload state: mixed against FP64, and deterministic."""
    cfg, spec = workloads.bcc64()
    lat = mcg.generate_lattice(spec, cfg)
    z, pl = mcg.random_state(lat, **workloads.DEFORM)
    top = lat.geometry.top0 + 0.01
    f64 = mcg.Solver(cfg, lat)
    mix = mcg.Solver(mixed_cfg(workloads.bcc64()[0]), lat)
    for sol in (f64, mix):
        sol.set_state(plastic=pl)
    a = f64.objective(z, top)
    b = mix.objective(z, top)
    b2 = mix.objective(z, top)
    print("full size: energy", abs(b["energy"] - a["energy"]) / abs(a["energy"]), "grad", rel_err(b["grad"], a["grad"]))
    assert abs(b["energy"] - a["energy"]) <= 1e-6 * abs(a["energy"])
    assert rel_err(b["grad"], a["grad"]) <= 1e-5
    assert b2["energy"] == b["energy"] and np.array_equal(b2["grad"], b["grad"])


def summary(frames):
    return {"peak_force": max(f["reaction_force"] for f in frames), "loading_work": frames[-1]["loading_work"],
            "dissipated_work": frames[-1]["dissipated_work"], "permanent_set": frames[-1]["permanent_set"]}


def test_mixed_run_matches_fp64_on_the_cubic_specimen(mcg):
    """The 6x6x6 cubic specimen, 40 % strain in 200 + 200 increments, mixed against FP64.

    Loading: peak platen force and absorbed (loading) work within 1e-5 of the FP64 run.
    Unloading is ill-conditioned: the solver stops at a 1.5e-3 relative residual, and from
    about increment 209 a perturbation of the iterate grows ~30x per increment, so the
    recovered work -- and with it dissipated work and permanent set -- moves by ~1e-4 under
    any perturbation of FP32 size.  The mixed run must therefore lie inside the envelope
    of FP64 runs whose Young's modulus is perturbed by +-1e-7 and +-2e-7 (one FP32 rounding
    of the section constants), widened by the envelope's span."""
    g = golden("cubic6")
    base = mcg.Solver(g.cfg, g.lattice)
    rc, f64 = base.run()
    assert rc == 0
    ens = [summary(f64)]
    for d in (-2e-7, -1e-7, 1e-7, 2e-7):
        cfg = golden("cubic6").cfg
        cfg.material.young *= 1.0 + d
        rc, fr = mcg.Solver(cfg, g.lattice).run()
        assert rc == 0
        ens.append(summary(fr))
    rc, mix = mcg.Solver(mixed_cfg(golden("cubic6").cfg), g.lattice).run()
    assert rc == 0 and len(mix) == len(f64)
    got, ref = summary(mix), ens[0]
    errs = {k: abs(got[k] - ref[k]) / abs(ref[k]) for k in got}
    spread = {k: (max(e[k] for e in ens) - min(e[k] for e in ens)) / abs(ref[k]) for k in got}
    print("mixed cubic6 run vs FP64:", errs, "FP64 perturbation spread:", spread)
    assert errs["peak_force"] <= 1e-5 and errs["loading_work"] <= 1e-5, errs
    for k in ("dissipated_work", "permanent_set"):
        lo = min(e[k] for e in ens)
        hi = max(e[k] for e in ens)
        assert lo - (hi - lo) <= got[k] <= hi + (hi - lo), (k, got[k], lo, hi)
