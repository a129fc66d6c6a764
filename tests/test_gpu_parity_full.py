"""Parity of the FP64 GPU evaluation with the CPU restatement at the benchmark's own size and
in dense self-contact (Simulator::objective, MC/src/sim.cpp:138-172).

  64x64x32 cubic+BCC (270,497 nodes, 1,458,336 beams) at the benchmark's seeded deformed
      state: the broad phase runs on the grid shapes the benchmark uses (the full-size bin
      count, ~6 M candidate pairs), which the fixture sizes never reach; the state has no
      self-contact within the target distance (its 1,063 contacts are platen contacts), so
      the pair set to match is empty and the evaluation's sums are the other check;
  32x32x16 cubic+BCC squeezed to 40 % of its height with lateral noise: ~42,000 contacting
      shape pairs, the narrow phase and the per-node contact lists at high density.

Bars as for the fixtures: energy 1e-10 relative, gradient 1e-10 relative in the 2-norm,
diagnostics 1e-10 (maximum penetration and contact count exact), contact pair sets
bit-identical, trial plastic states and trial diagnostics within 1e-10 per column.  The CPU
restatement is bit-identical to the reference on every fixture (tests/test_oracle.py); one
evaluation of the 64x64x32 state takes it ~50 s on one core.
"""
import numpy as np
import pytest

from conftest import rel_err
from falling_dice_gb300 import workloads
from test_gpu_objective import check_eval, close_cols

pytestmark = pytest.mark.gpu


def compare(fd, mco, cfg, lat, z, pl, top, name):
    sol = fd.Solver(cfg, lat)
    sol.set_state(plastic=pl)
    r = sol.objective(z, top, True)
    gpu_pairs = sol.contact_pairs()
    sol.close()
    orc = mco.Model("mco", cfg, lattice=lat)
    orc.set_state(plastic=pl)
    orc.record_pairs(True)
    o = orc.objective(z, top, True)
    ref_pairs = orc.last_pairs()
    s = {"energy": o["energy"], "grad": o["grad"],
         "diag": np.array([o["diag"][k] for k in ("elastic", "plastic", "contact", "reaction", "max_pen", "contacts")])}
    print(f"{name}: {lat.n_beams} beams, {len(ref_pairs)} contact pairs, energy rel err "
          f"{abs(r['energy'] - o['energy']) / abs(o['energy']):.2e}, grad rel err {rel_err(r['grad'], o['grad']):.2e}")
    check_eval(r, s, name)
    assert gpu_pairs.shape == ref_pairs.shape and np.array_equal(gpu_pairs, ref_pairs), name
    ok, err = close_cols(r["trial_next"], o["trial_next"], np.zeros(7))
    assert ok, (name, err)
    ok, err = close_cols(r["trial_aux"], o["trial_aux"], np.zeros(7))
    assert ok, (name, err)
    assert np.array_equal(r["trial_flags"], o["trial_flags"]), name
    return len(ref_pairs)


def test_headline_specimen_matches_oracle(mcg, mco):
    cfg, spec = workloads.bcc64()
    lat = mcg.generate_lattice(spec, cfg)
    z, pl = mcg.random_state(lat, **workloads.DEFORM)
    top = lat.geometry.top0 + 0.01  # the benchmark's platen height
    compare(mcg, mco, cfg, lat, z, pl, top, "bcc64 benchmark state")


def test_dense_contact_state_matches_oracle(mcg, mco):
    cfg, spec = workloads.bcc32()
    lat = mcg.generate_lattice(spec, cfg)
    squeeze = 0.6
    z, pl = mcg.random_state(lat, 0.15, 0.1, 0.02, 77)
    y = lat.x0[1::3]
    z[1::6] += -squeeze * (y - y.min()) / cfg.translation_scale
    z[lat.locked.astype(bool)] = 0
    top = lat.geometry.top0 - squeeze * lat.geometry.height + 1e-3
    n = compare(mcg, mco, cfg, lat, z, pl, top, "bcc32 squeezed")
    assert n > 30000
