"""Generates the golden fixtures in tests/golden/ by running the reference solver itself.

    python tests/golden/make_golden.py [--run-cubic6]

Needs the reference sources (to build oracle/_ref/libmcref.so) and libmcg.so (only for the
synthetic lattice generator, which is host code).  Every output value comes from the
reference's own Simulator (MC/src/sim.cpp) through oracle/ref_harness.cpp:

  ref242.npz       the reference's own 2x4x2 graded-BCC specimen (its builder), seeded
                   states incl. plastic, degenerate and non-finite cases: energy, gradient,
                   diagnostics, trial states, contact pair sets; one minimize; the
                   rigid-rotation and finite-difference checks; the full 20/14 run.
  cubic6.npz       the 6x6x6 cubic specimen: seeded evaluations and one minimize.
  bcc4.npz         a 4x4x4 cubic+BCC specimen at the heavy deformation of the
                   single-evaluation workload (many self-contacts).
  cubic6_run.npz   (--run-cubic6) the 6x6x6 specimen's full 200/200 load/unload run.
  ref242_metrics.csv, ref242_summary.json  (--outputs) the reference CLI's own writers
                   (MC/src/main.cpp:112-155) applied to the ref242 20/14 run.
  ref242_ensemble.npz  (--ensemble) the 20/14 run of the reference specimen under the CPU
                   restatement's rounding-order variants 1..31: the same sums in other orders.
                   Their spread is how far rounding alone moves the run-level results.
"""
import argparse
import ctypes as C
import os
import sys
import time
import zlib

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from falling_dice_gb300 import abi, workloads  # noqa: E402
import falling_dice_gb300 as fd  # noqa: E402
from oracle import oracle as orc  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
FRAME_KEYS = abi.FRAME_DOUBLES + abi.FRAME_INTS[:-2]


def cfg_dict(cfg):
    d = {}
    for name, _ in abi.Config._fields_:
        v = getattr(cfg, name)
        if name == "material":
            for m, _ in abi.Material._fields_:
                d["material." + m] = getattr(v, m)
        else:
            d[name] = v
    return d


def pack_cfg(cfg):
    d = cfg_dict(cfg)
    keys = sorted(d)
    return np.array(keys), np.array([repr(d[k]) for k in keys])


def reference_config_242():
    return abi.default_config(cells_x=2, cells_y=4, cells_z=2, load_steps=20, unload_steps=14,
                              max_strain=0.5, max_iterations=800, contact_stiffness=1e6)


def eval_states(model, lat, states, out):
    """states: list of (z, top, plastic or None, trials)."""
    for k, (z, top, plastic, trials) in enumerate(states):
        if plastic is not None:
            model.set_state(plastic=plastic)
        else:
            model.set_state(plastic=np.zeros(7 * lat.n_beams))
        r = model.objective(z, top, trials)
        p = f"s{k}_"
        out[p + "z"] = z
        out[p + "top"] = np.array([top])
        out[p + "plastic"] = plastic if plastic is not None else np.zeros(7 * lat.n_beams)
        out[p + "trials"] = np.array([int(trials)])
        out[p + "energy"] = np.array([r["energy"]])
        out[p + "grad"] = r["grad"]
        d = r["diag"]
        out[p + "diag"] = np.array([d["elastic"], d["plastic"], d["contact"], d["reaction"],
                                    d["max_pen"], d["contacts"]])
        if trials:
            out[p + "trial_next"] = r["trial_next"]
            out[p + "trial_aux"] = r["trial_aux"]
            out[p + "trial_flags"] = r["trial_flags"]
        out[p + "pairs"] = model.contact_pairs(z)
        print(f"  state {k}: E={r['energy']:.6g} contacts={d['contacts']} pairs={len(out[p + 'pairs'])}")
    model.set_state(plastic=np.zeros(7 * lat.n_beams))
    out["n_states"] = np.array([len(states)])


def random_plastic(rng, B, scale=0.01):
    pl = np.zeros((B, 7))
    pl[:, 0] = rng.uniform(-scale, scale, B)
    pl[:, 1] = np.abs(pl[:, 0]) + rng.uniform(0, scale, B)
    pl[:, 2:5] = rng.uniform(-scale, scale, (B, 3))
    pl[:, 5] = rng.uniform(0, scale, B)
    pl[:, 6] = rng.uniform(0, scale, B)
    return pl.reshape(-1)


def save_lattice(out, lat):
    for f in lat.FIELDS:
        out["lat_" + f] = getattr(lat, f)
    g = lat.geometry
    out["lat_geometry"] = np.array([g.width, g.height, g.depth, g.area, g.mass, g.top0])


def minimize_case(model, top, out, prefix="min_"):
    z0 = np.zeros(6 * model.n_nodes)
    z, st, fe, fdg = model.minimize(top, z0)
    out[prefix + "top"] = np.array([top])
    out[prefix + "z"] = z
    out[prefix + "stats"] = np.array([st["iterations"], st["backtracks"], st["rms"], st["max"],
                                      st["energy"], st["converged"]])
    out[prefix + "final"] = np.array([fe, fdg["elastic"], fdg["plastic"], fdg["contact"],
                                      fdg["reaction"], fdg["max_pen"], fdg["contacts"]])
    print(f"  minimize: {st}")


def frames_array(frames):
    return np.array([[f[k] for k in FRAME_KEYS] for f in frames], dtype=np.float64)


def make_ref242():
    print("ref242")
    cfg = reference_config_242()
    m = orc.Model("ref", cfg)
    lat = m.export()
    out = {}
    keys, vals = pack_cfg(cfg)
    out["cfg_keys"], out["cfg_vals"] = keys, vals
    out["translation_scale"] = np.array([lat.translation_scale])
    save_lattice(out, lat)
    rng = np.random.default_rng(242)
    N, B = lat.n_nodes, lat.n_beams
    top0 = lat.geometry.top0
    lk = lat.locked.astype(bool)

    def rz(s):
        z = rng.normal(0, s, 6 * N)
        z[lk] = 0
        return z
    zdeg = np.zeros(6 * N)
    a, b = int(lat.beam_a[0]), int(lat.beam_b[0])
    zdeg[6 * b:6 * b + 3] = (lat.x0[3 * a:3 * a + 3] - lat.x0[3 * b:3 * b + 3]) / lat.translation_scale
    zdeg[lk] = 0
    znan = rz(0.01)
    znan[6 * 7 + 1] = np.nan
    states = [
        (np.zeros(6 * N), top0, None, True),
        (rz(0.02), top0 - 0.002, None, False),
        (rz(0.02), top0 - 0.006, random_plastic(rng, B), True),
        (rz(0.08), top0 - 0.010, random_plastic(rng, B, 0.03), True),
        (zdeg, top0 - 0.001, None, True),
        (znan, top0, None, False),
    ]
    eval_states(m, lat, states, out)
    out["rigid_error"] = np.array([m.rigid_rotation_error()])
    out["fd_error"] = np.array([m.gradient_check_error()])
    minimize_case(m, top0 - 0.001, out)
    m2 = orc.Model("ref", cfg)
    t = time.time()
    rc, frames = m2.run()
    print(f"  run rc={rc} frames={len(frames)} in {time.time() - t:.1f}s")
    out["run_rc"] = np.array([rc])
    out["run_frames"] = frames_array(frames)
    out["frame_keys"] = np.array(FRAME_KEYS)
    np.savez_compressed(os.path.join(OUT, "ref242.npz"), **out)


def make_synthetic(name, preset, deform_sigma, extra_plastic=True, minimize=True):
    print(name)
    cfg, spec = preset
    lat = fd.generate_lattice(spec, cfg)
    m = orc.Model("ref", cfg, lattice=lat)
    out = {}
    keys, vals = pack_cfg(cfg)
    out["cfg_keys"], out["cfg_vals"] = keys, vals
    out["translation_scale"] = np.array([cfg.translation_scale])
    save_lattice(out, lat)
    N, B = lat.n_nodes, lat.n_beams
    top0 = lat.geometry.top0
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    lk = lat.locked.astype(bool)

    def rz(s):
        z = rng.normal(0, s, 6 * N)
        z[lk] = 0
        return z
    zc, plc = fd.random_state(lat, deform_sigma[0], deform_sigma[1], 0.02, 7)
    states = [
        (np.zeros(6 * N), top0, None, False),
        (rz(0.01), top0 - 0.001, None, True),
        (zc, top0 + 0.01, plc, True),
    ]
    if extra_plastic:
        states.append((rz(0.03), top0 - 0.004, random_plastic(rng, B), True))
    # densified: heights compressed to 45 % plus noise, so that non-adjacent struts touch
    zd = rz(0.12)
    y = lat.x0[1::3]
    zd[1::6] += (-0.55 * (y - y.min())) / cfg.translation_scale
    zd[lk] = 0
    states.append((zd, top0 - 0.55 * lat.geometry.height, random_plastic(rng, B), True))
    eval_states(m, lat, states, out)
    if minimize:
        minimize_case(m, top0 - 0.0005, out)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **out)


def make_cubic6_run():
    print("cubic6_run")
    cfg, spec = workloads.cubic6()
    lat = fd.generate_lattice(spec, cfg)
    m = orc.Model("ref", cfg, lattice=lat)
    t = time.time()
    rc, frames = m.run()
    print(f"  run rc={rc} frames={len(frames)} in {time.time() - t:.1f}s")
    out = {"run_rc": np.array([rc]), "run_frames": frames_array(frames),
           "frame_keys": np.array(FRAME_KEYS), "seconds": np.array([time.time() - t])}
    np.savez_compressed(os.path.join(OUT, "cubic6_run.npz"), **out)


def _ensemble_run(v):
    cfg = reference_config_242()
    m = orc.Model("mco", cfg)
    m.set_variant(v)
    t = time.time()
    rc, frames = m.run()
    return v, rc, frames_array(frames), time.time() - t


def make_ensemble(variants=range(1, 32)):
    """The 20/14 run under every rounding-order variant, four processes at a time."""
    import multiprocessing as mp
    print("ref242_ensemble")
    orc.build("mco")
    out = {"frame_keys": np.array(FRAME_KEYS), "variants": np.array(list(variants))}
    with mp.get_context("spawn").Pool(min(8, os.cpu_count() or 1)) as pool:
        for v, rc, frames, sec in pool.imap(_ensemble_run, list(variants)):
            peak = frames[:, FRAME_KEYS.index("reaction_force")].max() if len(frames) else float("nan")
            print(f"  variant {v}: rc={rc} frames={len(frames)} peak={peak:.4f} in {sec:.1f}s", flush=True)
            out[f"v{v}_rc"] = np.array([rc])
            out[f"v{v}_frames"] = frames
    np.savez_compressed(os.path.join(OUT, "ref242_ensemble.npz"), **out)


def frames_from_array(rows):
    """abi.Frame structs from the rows of a fixture's frame table (exact doubles)."""
    arr = (abi.Frame * max(len(rows), 1))()
    for i, row in enumerate(rows):
        for k, v in zip(FRAME_KEYS, row):
            setattr(arr[i], k, int(v) if k in abi.FRAME_INTS else float(v))
    return arr


def make_outputs():
    """The reference CLI's own metrics CSV and summary JSON (MC/src/main.cpp:112-155,
    writeMetrics / writeSummary) of the reference specimen's 20/14 run in ref242.npz."""
    print("ref242_metrics.csv, ref242_summary.json")
    d = np.load(os.path.join(OUT, "ref242.npz"))
    rows = d["run_frames"]
    cfg = reference_config_242()
    lib = orc.load("ref")
    rc = lib.orc_ref_write_outputs(frames_from_array(rows), len(rows), C.byref(cfg), float(d["lat_geometry"][4]),
                                   os.path.join(OUT, "ref242_metrics.csv").encode(),
                                   os.path.join(OUT, "ref242_summary.json").encode())
    assert rc == 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--run-cubic6", action="store_true")
    ap.add_argument("--ensemble", action="store_true")
    ap.add_argument("--outputs", action="store_true", help="the reference CLI's CSV/JSON of the ref242 run")
    ap.add_argument("--only", default=None)
    a = ap.parse_args()
    if not orc.build("ref"):
        sys.exit("the reference sources are not available: fixtures cannot be generated here")
    fd.load()
    if a.only == "none":
        pass
    elif a.only in (None, "ref242"):
        make_ref242()
    if a.only in (None, "cubic6"):
        make_synthetic("cubic6", workloads.cubic6(), (0.05, 0.1))
    if a.only in (None, "bcc4"):
        make_synthetic("bcc4", workloads.bcc((4, 4, 4)), (0.05, 0.1), minimize=False)
    if a.run_cubic6:
        make_cubic6_run()
    if a.ensemble:
        make_ensemble()
    if a.outputs:
        make_outputs()


if __name__ == "__main__":
    main()
