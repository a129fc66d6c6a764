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


def test_mixed_run_matches_fp64_on_the_cubic_specimen(mcg):
    g = golden("cubic6")
    run = np.load(os.path.join(GOLDEN, "cubic6_run.npz"))
    keys = [str(k) for k in run["frame_keys"]]
    ref = [dict(zip(keys, row)) for row in run["run_frames"]]
    sol = mcg.Solver(mixed_cfg(g.cfg), g.lattice)
    rc, frames = sol.run()
    assert rc == 0 and len(frames) == len(ref)
    peak = max(f["reaction_force"] for f in frames)
    peak_ref = max(f["reaction_force"] for f in ref)
    errs = {"peak_force": abs(peak - peak_ref) / peak_ref,
            "loading_work": abs(frames[-1]["loading_work"] - ref[-1]["loading_work"]) / ref[-1]["loading_work"],
            "dissipated_work": abs(frames[-1]["dissipated_work"] - ref[-1]["dissipated_work"]) / ref[-1]["dissipated_work"],
            "permanent_set": abs(frames[-1]["permanent_set"] - ref[-1]["permanent_set"]) / ref[-1]["permanent_set"]}
    print("mixed cubic6 run vs reference:", errs)
    assert errs["peak_force"] <= 1e-5 and errs["loading_work"] <= 1e-5 and errs["dissipated_work"] <= 1e-5, errs
