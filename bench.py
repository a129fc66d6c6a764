"""Throughput of the beam-lattice energy/gradient evaluation on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl mcg|reference]
                    [--workload bcc64|cubic6|bcc32|bcc128]

A step is one full evaluation of the objective (energy + 6-DOF gradient: node state, beam
mechanics with return mapping, self-contact broad/narrow phase, platen contact, gather)
on the 64x64x32 cubic+BCC specimen at its seeded deformed state.  Metric: evaluations/s.
The headline is the mixed-precision form (FP32 bulk arithmetic, FP64 base state and
reductions), with its error against the plain FP64 form; the FP64 form is measured beside
it under "fp64".

value      device-resident: z already in HBM, result left in HBM (mcg_objective_resident).
e2e        the public C-ABI call mcg_objective with pinned host buffers: z host->device,
           energy + gradient device->host, every step.
roofline   the beam kernel (the dominant kernel): algorithmic bytes per launch (128 B per
           beam: end indices, L0, radius, area, I, J, e0 and the 7 plastic values, FP64)
           over its CUDA-event time, against the measured HBM copy bandwidth.
cpu_baseline  the CPU restatement of the reference objective (oracle/), one core, on a
           bounded sample of the same lattice family, scaled by beam count.

--impl reference times the reference's CPU implementation of the same evaluation (the
oracle port where the reference cannot be built, i.e. on the GPU machine) on all host cores,
one process per core, each evaluating a bounded sample, scaled by beam count.

Multi-GPU: replicas only (every rank evaluates its own copy; no collective), weak scaling.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

BEAM_BYTES = 128    # per beam, FP64: a, b (2 x 4 B) + 15 reals
NODE_BYTES = 166    # per node, FP64: z[6] + baseX[3] + baseR[4] + mass + grad[6], locked[6]
# DRAM bytes (read + write, ncu dram__bytes_read.sum + dram__bytes_write.sum) of one launch,
# captured with ncu on GB300 and scaled to the workload:
#   k_beams (FP64), 32x32x16 cubic+BCC: 40.35 MB for 184,400 beams, scaled by beam count;
#   k_beams_mixed, 64x64x32 cubic+BCC: 212.75 MB for 1,458,336 beams, scaled by beam count;
#   k_bin_pairs, 64x64x32 cubic+BCC at the tuned shapes (4.5 mm cell, 1216 blocks): 107.87 MB
#   where the algorithmic bytes below come to 123.55 MB, scaled by the algorithmic bytes.
BEAM_TRAFFIC_PER_BEAM = 40.348160e6 / 184400
BEAM_TRAFFIC_PER_BEAM_MIXED = 212.748800e6 / 1458336
PAIR_TRAFFIC_PER_ALGORITHMIC_BYTE = 107.870720e6 / 123.545196e6
BEAM_BYTES_MIXED = 68    # per beam, mixed: a, b (2 x 4 B) + 15 reals as FP32
NODE_BYTES_MIXED = 98    # per node, mixed: baseX (3 x 8 B) + 17 reals as FP32 + locked[6]
# Pair enumeration (k_bin_pairs), algorithmic bytes: every cell entry's shape id (4 B), each
# shape's pair-test record once (16 B box/cell record + 8 B nodes), each occupied bin's
# count, start and list slot (12 B), each candidate written (8 B).
PAIR_ENTRY_BYTES, PAIR_SHAPE_BYTES, PAIR_BIN_BYTES, PAIR_CAND_BYTES = 4, 24, 12, 8
# The pair enumeration is bound by instruction issue, not by memory: its second roofline is
# warp instructions per second against the issue peak of one warp instruction per clock on
# each of the 4 x 152 SM sub-partitions.  Instructions per launch from ncu
# (smsp__inst_executed.sum, profiles/k_bin_pairs_bcc64.md) at the benchmark state of the
# 64x64x32 specimen with the 4.5 mm cell and 1216 pair blocks; other shapes have no figure.
PAIR_WARP_INSTRUCTIONS = {("bcc64", 0.0045, 1216): 304137669}
SM_SUBPARTITIONS = 4 * 152


def pair_issue_roofline(workload, cell, pair_blocks, ms, sm_mhz):
    """Warp instructions/s of one k_bin_pairs launch against the issue peak, or None when no
    instruction count was measured for these shapes."""
    key = next((k for k in PAIR_WARP_INSTRUCTIONS
                if k[0] == workload and abs(k[1] - cell) < 1e-9 and k[2] == pair_blocks), None)
    if key is None or not ms or not sm_mhz:
        return None
    inst = PAIR_WARP_INSTRUCTIONS[key]
    ach = inst / (ms * 1e-3) / 1e9
    peak_issue = SM_SUBPARTITIONS * sm_mhz * 1e6 / 1e9
    return {"bound": "issue", "achieved": ach, "peak": peak_issue, "unit": "G warp-instructions/s",
            "frac": ach / peak_issue, "warp_instructions_per_launch": inst, "sm_mhz": sm_mhz,
            "source": "ncu smsp__inst_executed.sum of one launch with the same shapes"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="mcg", choices=["mcg", "reference"])
    ap.add_argument("--workload", default="bcc64")
    ap.add_argument("--shapes", default="",
                    help="CELL,PAIR_BLOCKS[,BEAM_BLOCKS,GATHER_BLOCKS]: fixed shapes instead of tuning "
                         "(broad-phase cell and pair grid; CTAs per SM of the beam kernel and the gather)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the load/unload (32x32x16) and batched-sweep (256 lattices) measurements")
    ap.add_argument("--largest-run", action="store_true",
                    help="only the 128x128x64 load run (50 %% strain, 100 increments), mixed against FP64")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(torch, x, pg, device):
    """The largest of the ranks' values of x (a time): every replica waits for the slowest."""
    if pg is None:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world, steps, ms):
    """Whole-job evaluations per second: `world` replicas each ran `steps` evaluations in at
    most `ms` milliseconds (the max over ranks)."""
    return world * 1e3 * steps / ms


def workload(name):
    from falling_dice_gb300 import workloads
    return getattr(workloads, name)()


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}",
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if not self.rows:
            return None
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[3 + k] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cpu_model():
    """The host CPU's model name and core count, for the CPU-baseline records."""
    name = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                name = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    return {"model": name or "unknown", "cores": os.cpu_count() or 1}


# -- the reference's CPU path (the oracle's restatement of it; test infrastructure) ----------
# Workers build the specimen and its seeded state with the oracle's own restatement of the
# workload generator (oracle/specimens.cpp), so the CPU legs load no product library.
_worker_model = None
_worker_args = None


def _worker_init(name):
    global _worker_model, _worker_args
    sys.path.insert(0, ROOT)
    from falling_dice_gb300 import workloads
    from oracle import oracle as orc
    cfg, spec = getattr(workloads, name)()
    m = orc.Model("mco", cfg, lattice=spec)
    lat = m.export()
    z, pl = orc.random_state(lat.n_nodes, lat.n_beams, lat.locked, **workloads.DEFORM)
    m.set_state(plastic=pl)
    _worker_model = m
    _worker_args = (z, lat.geometry.top0 + 0.01, lat.n_nodes, lat.n_beams)


def _worker_eval(_):
    """One full evaluation of the reference objective at the benchmark state; (seconds, E)."""
    z, top, _, _ = _worker_args
    t = time.perf_counter()
    e = _worker_model.objective(z, top)["energy"]
    return time.perf_counter() - t, e


def cpu_one_core(name):
    """One full-size evaluation of the reference objective (the oracle port) on one core."""
    from oracle import oracle as orc
    orc.build("mco")
    _worker_init(name)
    dt, e = _worker_eval(0)
    return dt, e, _worker_args[2], _worker_args[3]


def run_reference(a, rank, world):
    """--impl reference: the reference CPU objective (the oracle port of it) on all host
    cores, one process per core; every step is one full evaluation of the benchmark
    specimen at the benchmark state, and the steps are spread over the processes.  A full
    evaluation takes ~47 s of one core, so the arm runs at most two steps per process
    (the steps it ran are the line's "steps"; "steps_requested" is the count asked for),
    which keeps it within a few minutes at any --steps."""
    if rank != 0:
        return
    import multiprocessing as mp
    sys.path.insert(0, ROOT)
    from oracle import oracle as orc
    orc.build("mco")
    host = cpu_model()
    cores = host["cores"]
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores, initializer=_worker_init, initargs=(a.workload,)) as pool:
        pool.map(_worker_eval, range(max(1, min(a.warmup, cores))), chunksize=1)  # untimed
        steps = max(1, min(a.steps, 2 * cores))
        t0 = time.perf_counter()
        res = pool.map(_worker_eval, range(steps), chunksize=1)
        wall = time.perf_counter() - t0
        N, B = pool.apply(_counts)
    value = steps / wall
    energies = {r[1] for r in res}
    assert len(energies) == 1  # every process evaluated the same state
    kind = "port"  # the CPU restatement, bit-identical to the reference (tests/test_oracle.py)
    sample = (f"{steps} full evaluations of the {a.workload} specimen ({N} nodes, {B} beams) at the "
              f"benchmark state, spread over {cores} processes; no scaling")
    line = {"impl": "reference", "metric": "beam energy-grad evals/s", "value": value, "unit": "evals/s",
            "n_gpus": a.gpus, "steps": steps, "steps_requested": a.steps, "warmup": a.warmup,
            "ms_per_step": 1e3 / value, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"{a.workload}: {N} nodes, {B} beams, seeded deformed state",
                       "parallelism": f"{cores} CPU processes", "cpu": host["model"]},
            "cpu_baseline": {"value": value, "unit": "evals/s", "cores": cores, "kind": kind,
                             "sample": sample, "cpu": host["model"],
                             "seconds_per_eval_mean": float(np.mean([r[0] for r in res])),
                             "wall_s": wall, "energy": energies.pop()},
            "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _counts():
    return _worker_args[2], _worker_args[3]


def _sweep_cpu_run(k):
    """One lattice of the sweep solved by the reference's own run (the oracle port) on one
    core: (lattice index, beams, status, frames, seconds)."""
    sys.path.insert(0, ROOT)
    from falling_dice_gb300 import abi, workloads
    from oracle import oracle as orc
    cfg, specs, ys = workloads.sweep()
    c = abi.Config.from_buffer_copy(cfg)
    c.material.yield_ = ys[k]
    m = orc.Model("mco", c, lattice=specs[k])
    beams = m.export().n_beams
    t = time.perf_counter()
    rc, frames = m.run()
    return k, beams, int(rc), len(frames), time.perf_counter() - t


def sweep_cpu_reference(workloads, batched_rate):
    """The sweep's CPU reference (one reference process per host core): the reference's own
    run of the sweep's smallest lattices, one per core, on all cores at once.  A whole sweep
    on the CPU takes hours (its smallest lattice alone ~50 s of one core), so this times the
    cheapest lattices only; their rate bounds the CPU's sweep rate from above."""
    import multiprocessing as mp
    from oracle import oracle as orc
    orc.build("mco")
    cores = cpu_model()["cores"]
    cfg, specs, ys = workloads.sweep()
    order = sorted(range(len(specs)), key=lambda k: (specs[k].cells_x * specs[k].cells_y * specs[k].cells_z, k))
    pick = order[:cores]
    with mp.get_context("spawn").Pool(cores) as pool:
        t0 = time.perf_counter()
        res = pool.map(_sweep_cpu_run, pick, chunksize=1)
        wall = time.perf_counter() - t0
    secs = [r[4] for r in res]
    rate = len(pick) / wall
    return {"metric": "lattices/s", "cores": cores, "cpu": cpu_model()["model"], "kind": "port",
            "lattices": len(pick), "beams": [r[1] for r in res], "status": [r[2] for r in res],
            "wall_s": wall, "seconds_per_lattice_mean": float(np.mean(secs)),
            "all_cores_lattices_per_s": rate, "one_core_lattices_per_s": 1.0 / float(np.mean(secs)),
            "batched_gpu_over_all_cores": batched_rate / rate,
            "sample": f"the {len(pick)} smallest of the {len(specs)} lattices (by cell count), each solved "
                      f"by the reference's run in its own process; an upper bound of the CPU's sweep rate"}


def measure(fd, torch, cfg, lat, z, pl, top, steps, warmup, local, pg, world, shapes=None):
    """Times one precision form: device-resident evaluations, e2e through the C ABI, phases."""
    import ctypes as C
    from falling_dice_gb300 import abi
    N, B = lat.n_nodes, lat.n_beams
    sol = fd.Solver(cfg, lat, device=local)
    sol.set_contact_skin(0.0)  # a full evaluation: grid, pairs and narrow phase every step
    sol.set_state(plastic=pl)
    if shapes:  # fixed shapes (a saved tuning), e.g. for a profiler run
        sol.set_contact_shapes(shapes[0], shapes[1])
        kb = shapes[2:4] if len(shapes) >= 4 else (0, 0)
        try:
            sol.set_kernel_shapes(*kb)
        except fd.MCGError:  # the occupancy variants differ between the two forms
            kb = (0, 0)
            sol.set_kernel_shapes(*kb)
        tune = {"cell": shapes[0], "pair_blocks": shapes[1], "beam_blocks": kb[0], "gather_blocks": kb[1],
                "tried": 0}
    else:
        tune = sol.autotune(z, top, reps=3)  # broad-phase cell and pair grid, by measurement
    sol.upload_z(z)
    stream = torch.cuda.ExternalStream(sol.stream, device=local)

    def barrier():
        if pg is not None:
            pg.barrier()
        torch.cuda.synchronize()

    for _ in range(max(warmup, 3)):
        sol.objective_resident(top)
    res0 = sol.read_result(grad=True)  # also sizes the contact buffers before timing
    barrier()
    launches0 = sol.launch_count()
    clocks = Clocks(local)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    nvtx = "timed_mixed" if cfg.precision == abi.MCG_MIXED else "timed_fp64"
    torch.cuda.nvtx.range_push(nvtx)  # lets a profiler select the timed launches
    e0.record(stream)
    for _ in range(steps):
        sol.objective_resident(top)
    e1.record(stream)
    torch.cuda.nvtx.range_pop()
    barrier()
    ms = e0.elapsed_time(e1)
    launches = sol.launch_count() - launches0
    clk = clocks.stop()
    ms = max_over_ranks(torch, ms, pg, "cuda")
    res = sol.read_result(grad=False)
    # end to end through the public C ABI, pinned host buffers
    zh = torch.empty(6 * N, dtype=torch.float64, pin_memory=True)
    zh.numpy()[:] = z
    gh = torch.empty(6 * N, dtype=torch.float64, pin_memory=True)
    eout = C.c_double()
    diag = abi.Diag()
    zp = C.cast(zh.data_ptr(), C.POINTER(C.c_double))
    gp = C.cast(gh.data_ptr(), C.POINTER(C.c_double))
    for _ in range(max(warmup, 3)):
        sol.lib.mcg_objective(sol.h, zp, top, 0, C.byref(eout), gp, C.byref(diag), None, None, None)
    barrier()
    t0 = time.perf_counter()
    e0.record(stream)
    for _ in range(steps):
        rc = sol.lib.mcg_objective(sol.h, zp, top, 0, C.byref(eout), gp, C.byref(diag), None, None, None)
        assert rc == 0
    e1.record(stream)
    barrier()
    ms_e2e = max(e0.elapsed_time(e1), (time.perf_counter() - t0) * 1e3)
    ms_e2e = max_over_ranks(torch, ms_e2e, pg, "cuda")
    assert np.isfinite(eout.value) and eout.value == res["energy"]
    # per-phase timing for the roofline (a separate pass: it synchronises per evaluation)
    sol.set_timing(True)
    for _ in range(max(3, min(steps, 10))):
        sol.objective_resident(top)
    phases, nev = sol.phase_times()
    sol.set_timing(False)
    stats = sol.contact_stats()
    sol.close()
    return {"ms_step": ms / steps, "value": replica_throughput(world, steps, ms),
            "e2e": replica_throughput(world, steps, ms_e2e),
            "launches": launches, "clocks": clk, "energy": res["energy"], "grad": res0["grad"],
            "contacts": res["diag"]["contacts"], "phases": {k: v / nev for k, v in phases.items()},
            "contact_stats": stats, "tuning": tune}


def main():
    a = parse()
    rank, world, local = dist_info()
    if a.impl == "reference":
        run_reference(a, rank, world)
        return
    if a.largest_run:
        import falling_dice_gb300 as fd
        from falling_dice_gb300 import abi, workloads
        print(json.dumps(largest_run(fd, abi, workloads)), flush=True)
        return
    import torch
    import falling_dice_gb300 as fd
    from falling_dice_gb300 import abi, workloads
    if not os.path.exists(fd.LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()
    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        pg = dist
    cfg, spec = workload(a.workload)
    lat = fd.generate_lattice(spec, cfg)
    z, pl = fd.random_state(lat, **workloads.DEFORM)
    top = lat.geometry.top0 + 0.01
    N, B = lat.n_nodes, lat.n_beams
    cfg_mixed = workload(a.workload)[0]
    cfg_mixed.precision = abi.MCG_MIXED
    shapes = None
    if a.shapes:
        parts = a.shapes.split(",")
        shapes = (float(parts[0]),) + tuple(int(v) for v in parts[1:])
    mixed = measure(fd, torch, cfg_mixed, lat, z, pl, top, a.steps, a.warmup, local, pg, world, shapes)
    plain = measure(fd, torch, cfg, lat, z, pl, top, a.steps, a.warmup, local, pg, world, shapes)
    if rank != 0:
        return
    peak, peak_kind = measured_peaks()
    beam_bytes_f64 = BEAM_BYTES * B
    beam_bytes_mixed = BEAM_BYTES_MIXED * B

    def roofline(r, nbytes, traffic):
        ms = r["phases"]["beams"]
        ach = nbytes / (ms * 1e-3) / 1e9
        return {"bound": "hbm", "kernel": "k_beams_mixed" if r is mixed else "k_beams", "achieved": ach,
                "peak": peak, "unit": "GB/s", "frac": ach / peak, "peak_source": peak_kind,
                "traffic": traffic, "bytes_per_launch": nbytes, "ms_per_launch": ms}

    def roofline_pairs(r):
        st = r["contact_stats"]
        nbytes = (PAIR_ENTRY_BYTES * st["entries"] + PAIR_SHAPE_BYTES * (N + B) +
                  PAIR_BIN_BYTES * st["occupied_bins"] + PAIR_CAND_BYTES * st["candidates"])
        ms = r["phases"]["pairs"]
        ach = nbytes / (ms * 1e-3) / 1e9
        return {"bound": "hbm", "kernel": "k_bin_pairs", "achieved": ach, "peak": peak, "unit": "GB/s",
                "frac": ach / peak, "peak_source": peak_kind,
                "traffic": nbytes * PAIR_TRAFFIC_PER_ALGORITHMIC_BYTE, "bytes_per_launch": nbytes,
                "ms_per_launch": ms, "share_of_evaluation": ms / r["ms_step"],
                "counts": st, "note": "issue-bound integer work (pair tests); the fraction is of HBM",
                "issue": pair_issue_roofline(a.workload, r["tuning"].get("cell") or 0.0,
                                             r["tuning"].get("pair_blocks") or 0, ms,
                                             (r["clocks"] or {}).get("sm_mhz"))}
    cpu = None
    if not a.no_cpu_baseline:
        t_s, e_cpu, N_s, B_s = cpu_one_core(a.workload)
        cpu = {"value": 1.0 / t_s, "unit": "evals/s", "cores": 1, "kind": "port", "cpu": cpu_model()["model"],
               "sample": f"one full evaluation of the {a.workload} specimen ({N_s} nodes, {B_s} beams) at the "
                         f"benchmark state on one core, {t_s:.1f} s; no scaling",
               "seconds_per_eval": t_s,
               "energy_rel_err_vs_gpu_fp64": abs(e_cpu - plain["energy"]) / abs(e_cpu)}
    err_e = abs(mixed["energy"] - plain["energy"]) / abs(plain["energy"])
    err_g = float(np.linalg.norm(mixed["grad"] - plain["grad"]) / np.linalg.norm(plain["grad"]))
    eval_bytes_mixed = BEAM_BYTES_MIXED * B + NODE_BYTES_MIXED * N
    line = {
        "metric": "beam energy-grad evals/s", "value": mixed["value"], "unit": "evals/s",
        "n_gpus": world, "steps": a.steps, "warmup": a.warmup, "ms_per_step": mixed["ms_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 (f64 reductions)",
        "data": "synthetic",
        "config": {"workload": f"{a.workload}: cubic+BCC {spec.cells_x}x{spec.cells_y}x{spec.cells_z}, "
                               f"{N} nodes, {B} beams, seeded deformed state",
                   "precision": "mixed: FP32 bulk, FP64 base state and reductions",
                   "parallelism": "replicas" if world > 1 else "single",
                   "l2": "inputs larger than L2 (beam arrays alone exceed 129 MB)",
                   "contact_list": "rebuilt at every evaluation (grid, pairs, narrow phase)",
                   "shapes": {k: mixed["tuning"].get(k) for k in ("cell", "pair_blocks", "beam_blocks",
                                                                   "gather_blocks", "tried")},
                   "shapes_fp64": {k: plain["tuning"].get(k) for k in ("cell", "pair_blocks", "beam_blocks",
                                                                        "gather_blocks", "tried")}},
        "error_vs_fp64": {"energy_rel": err_e, "grad_rel_2norm": err_g},
        "hbm_gbs_algorithmic": eval_bytes_mixed * mixed["value"] / world / 1e9,
        "phase_ms": mixed["phases"],
        "roofline": roofline_pairs(mixed),
        "roofline_beams": roofline(mixed, beam_bytes_mixed, BEAM_TRAFFIC_PER_BEAM_MIXED * B),
        "fp64": {"value": plain["value"], "ms_per_step": plain["ms_step"], "e2e": plain["e2e"],
                 "phase_ms": plain["phases"], "gpu_launches": int(plain["launches"]),
                 "hbm_gbs_algorithmic": (BEAM_BYTES * B + NODE_BYTES * N) * plain["value"] / world / 1e9,
                 "roofline": roofline(plain, beam_bytes_f64, BEAM_TRAFFIC_PER_BEAM * B)},
        "cpu_baseline": cpu,
        "e2e": {"value": mixed["e2e"], "unit": "evals/s", "h2d_bytes_per_step": 8 * 6 * N,
                "d2h_bytes_per_step": 8 * 6 * N + 8},
        "gpu_launches": int(mixed["launches"]),
        "clocks": mixed["clocks"] or plain["clocks"],
        "energy": mixed["energy"], "contacts": mixed["contacts"],
    }
    if not a.no_extras and world == 1:
        line["dense_contact"] = dense_contact(fd, abi, workloads, torch)
        line["load_unload"] = load_unload(fd, abi, workloads)
        line["sweep"] = sweep(fd, abi, workloads)
    print(json.dumps(line), flush=True)


def run_summary(frames):
    return {"frames": len(frames), "iterations": int(sum(f["iterations"] for f in frames)),
            "peak_force": max(f["reaction_force"] for f in frames), "absorbed_energy": frames[-1]["loading_work"],
            "dissipated_work": frames[-1]["dissipated_work"], "permanent_set": frames[-1]["permanent_set"]}


def squeezed_state(fd, lat, cfg, squeeze=0.6):
    """The 32x32x16 specimen squeezed to 1 - squeeze of its height with lateral noise: the
    dense self-contact state of the full-size parity test (~42,000 contacting shape pairs)."""
    z, pl = fd.random_state(lat, 0.15, 0.1, 0.02, 77)
    y = lat.x0[1::3]
    z[1::6] += -squeeze * (y - y.min()) / cfg.translation_scale
    z[lat.locked.astype(bool)] = 0
    return z, pl, lat.geometry.top0 - squeeze * lat.geometry.height + 1e-3


def dense_contact(fd, abi, workloads, torch, steps=100):
    """Evaluations/s in dense self-contact, mixed and FP64: the squeezed 32x32x16 state, the
    contact list rebuilt at every evaluation, device-resident evaluations timed by CUDA events
    (its arrays fit in L2, so these are warm-cache figures), the phase split and the contact
    statistics.  The headline state has no self-contact within reach (its contacts are platen
    contacts); here the filter, the narrow phase and the per-node contact lists carry load."""
    out = {}
    for name, prec in (("mixed", abi.MCG_MIXED), ("fp64", abi.MCG_FP64)):
        cfg, spec = workloads.bcc32()
        cfg.precision = prec
        lat = fd.generate_lattice(spec, cfg)
        z, pl, top = squeezed_state(fd, lat, cfg)
        sol = fd.Solver(cfg, lat)
        sol.set_contact_skin(0.0)
        sol.set_state(plastic=pl)
        sol.upload_z(z)
        for _ in range(5):
            sol.objective_resident(top)
        res = sol.read_result(grad=False)
        stream = torch.cuda.ExternalStream(sol.stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(steps):
            sol.objective_resident(top)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        sol.set_timing(True)
        for _ in range(10):
            sol.objective_resident(top)
        phases, nev = sol.phase_times()
        sol.set_timing(False)
        st = sol.contact_stats()
        sol.close()
        out[name] = {"evals_per_s": 1e3 / ms, "ms_per_eval": ms, "contacts": int(res["diag"]["contacts"]),
                     "phase_ms": {k: v / nev for k, v in phases.items()}, "contact_stats": st}
    out["workload"] = (f"bcc32 squeezed to 40 % of its height: {lat.n_nodes} nodes, {lat.n_beams} beams, "
                       f"{out['fp64']['contact_stats']['contacts']} contacting shape pairs")
    return out


def load_unload(fd, abi, workloads):
    """The 32x32x16 cubic+BCC specimen, 60 % strain in 400 + 400 increments, mixed against
    FP64: wall time of the whole run (minimize rounds in the device-resident graph loop,
    commit and diagnostics on the device, the increment logic on the host) and the run-level
    figures, with their errors against FP64.  "split_ms" divides the run: device time of the
    loop's directions, evaluations and decisions/accept steps (global-timer stamps between
    the rounds' stage kernels), and the rest of the wall time (loop launches, commits,
    diagnostics, host increment logic)."""
    out = {}
    frames_of = {}
    for name, prec in (("mixed", abi.MCG_MIXED), ("fp64", abi.MCG_FP64)):
        cfg, spec = workloads.bcc32()
        cfg.precision = prec
        lat = fd.generate_lattice(spec, cfg)
        sol = fd.Solver(cfg, lat)
        t0 = time.perf_counter()
        rc, frames = sol.run()
        dt = time.perf_counter() - t0
        lt = sol.solver_times()
        loop_on, why = sol.solver_loop()
        builds = sol.contact_builds()
        sol.close()
        frames_of[name] = frames
        dev = lt["directions"] + lt["evaluations"] + lt["decisions_accept"]
        out[name] = dict(run_summary(frames), seconds=dt, status=int(rc),
                         iterations=int(sum(f["iterations"] for f in frames)), rounds=int(lt["rounds"]),
                         contact_list_builds=int(builds), device_loop=bool(loop_on), device_loop_error=why,
                         split_ms={"directions": lt["directions"], "evaluations": lt["evaluations"],
                                   "decisions_accept": lt["decisions_accept"], "rest": 1e3 * dt - dev})
    m, f = out["mixed"], out["fp64"]
    out["speedup_mixed_over_fp64"] = f["seconds"] / m["seconds"]
    out["rel_err_mixed_vs_fp64"] = {k: abs(m[k] - f[k]) / abs(f[k]) for k in
                                    ("peak_force", "absorbed_energy", "dissipated_work", "permanent_set")}
    out["curve_mixed_vs_fp64"] = curve_divergence(frames_of["mixed"], frames_of["fp64"])
    out["workload"] = "bcc32: cubic+BCC 32x32x16, radius 0.25->0.7 mm graded, 60 % strain, 400 + 400 increments"
    return out


def largest_run(fd, abi, workloads):
    """The largest single instance: 128x128x64 cubic+BCC (11.6 M beams), 50 % strain in 100
    increments with self-contact, mixed against FP64: wall time, run figures and their errors,
    per-increment curve error, and the mixed beam kernel's HBM fraction at this size."""
    out = {"workload": "bcc128: cubic+BCC 128x128x64, radii U[0.3, 0.6] mm, +/-2 % jitter, 50 % strain in "
                       "100 increments, self-contact on"}
    frames_of = {}
    peak, peak_kind = measured_peaks()
    for name, prec in (("mixed", abi.MCG_MIXED), ("fp64", abi.MCG_FP64)):
        cfg, spec = workloads.bcc128()
        cfg.precision = prec
        lat = fd.generate_lattice(spec, cfg)
        sol = fd.Solver(cfg, lat)
        t0 = time.perf_counter()
        rc, frames = sol.run()
        dt = time.perf_counter() - t0
        frames_of[name] = frames
        lt = sol.solver_times()
        out[name] = dict(run_summary(frames), seconds=dt, status=int(rc), beams=lat.n_beams, nodes=lat.n_nodes,
                         frames=len(frames), iterations=int(sum(f["iterations"] for f in frames)),
                         rounds=int(lt["rounds"]), contact_list_builds=int(sol.contact_builds()),
                         split_ms={"directions": lt["directions"], "evaluations": lt["evaluations"],
                                   "decisions_accept": lt["decisions_accept"]})
        # one evaluation at the final committed state, phases timed, for the beam kernel's roofline
        sol.upload_z(np.zeros(6 * lat.n_nodes))
        sol.set_timing(True)
        for _ in range(5):
            sol.objective_resident(lat.geometry.top0)
        ph, nev = sol.phase_times()
        sol.close()
        ms = ph["beams"] / nev
        nbytes = (BEAM_BYTES_MIXED if prec == abi.MCG_MIXED else BEAM_BYTES) * lat.n_beams
        out[name]["beam_kernel"] = {"ms": ms, "gbs_algorithmic": nbytes / (ms * 1e-3) / 1e9,
                                    "frac_of_hbm": nbytes / (ms * 1e-3) / 1e9 / peak, "peak_source": peak_kind}
        out[name]["eval_ms"] = sum(ph[k] for k in sol.PHASES) / nev
        print(json.dumps({name: out[name]}), file=sys.stderr, flush=True)  # progress of a long run
    m, f = out["mixed"], out["fp64"]
    out["speedup_mixed_over_fp64"] = f["seconds"] / m["seconds"]
    out["rel_err_mixed_vs_fp64"] = {k: abs(m[k] - f[k]) / abs(f[k]) for k in
                                    ("peak_force", "absorbed_energy", "permanent_set")}
    out["curve_mixed_vs_fp64"] = curve_divergence(frames_of["mixed"], frames_of["fp64"])
    return out


def curve_divergence(a, b, bar=1e-5):
    """Reaction-force curves of two runs compared at the schedule's own increments (frames
    that were not bisected, matched by platen position): relative error against b's peak per
    increment, its maximum and mean, and the first increment (with its strain) past `bar`."""
    peak = max(f["reaction_force"] for f in b)
    fb = {f["platen_y"]: f for f in b if f["refinement"] == 0}
    errs = []
    for k, f in enumerate(x for x in a if x["refinement"] == 0):
        g = fb.get(f["platen_y"])
        if g is not None and f["loading"] == g["loading"]:
            errs.append((k, f["engineering_strain"], abs(f["reaction_force"] - g["reaction_force"]) / peak))
    first = next(((k, s_) for k, s_, e in errs if e > bar), None)
    return {"increments_compared": len(errs), "max_rel": max((e for _, _, e in errs), default=0.0),
            "mean_rel": float(np.mean([e for _, _, e in errs])) if errs else 0.0,
            "first_increment_beyond_1e-5": None if first is None else {"increment": first[0], "strain": first[1]},
            "rel_by_increment_every_40": [round(e, 9) for _, _, e in errs[::40]]}


def sweep(fd, abi, workloads, sample=32):
    """The batched sweep: 256 lattices (4-16 cells per side) solved together in FP64, against
    the same lattices solved one after another.  The sequential figure comes from a systematic
    sample of `sample` lattices spread over the sweep's cost range (lattices ordered by beam
    count, every 256/sample-th timed): mean time per lattice with its standard error, so the
    sequential throughput and the speed-up carry an error bar."""
    cfg, specs, ys = workloads.sweep()
    lats = [fd.generate_lattice(s, cfg) for s in specs]
    b = fd.BatchSolver(cfg, lats, yields=ys)
    t0 = time.perf_counter()
    tune = b.autotune(reps=3)  # inside the timed region: part of the job
    status, runs = b.run()
    dt = time.perf_counter() - t0
    b.close()
    order = np.argsort([l.n_beams for l in lats], kind="stable")
    step = len(lats) / sample
    idx = [int(order[int((j + 0.5) * step)]) for j in range(sample)]
    times = []
    same = True
    for k in idx:
        c = abi.Config.from_buffer_copy(cfg)
        c.material.yield_ = ys[k]
        s = fd.Solver(c, lats[k])
        t0 = time.perf_counter()
        rc, fr = s.run()
        times.append(time.perf_counter() - t0)
        s.close()
        same &= [x["reaction_force"] for x in fr] == [x["reaction_force"] for x in runs[k]]
    mean_t = float(np.mean(times))
    se_t = float(np.std(times, ddof=1) / np.sqrt(len(times)))
    batched, seq = len(lats) / dt, 1.0 / mean_t
    try:
        cpu_ref = sweep_cpu_reference(workloads, batched)
    except Exception as e:  # the CPU leg never costs the GPU figures
        cpu_ref = {"error": f"{type(e).__name__}: {e}"}
    return {"metric": "lattices/s", "batched_fp64": batched, "sequential_fp64": seq, "speedup": batched / seq,
            "speedup_range_1se": [batched * (mean_t - se_t), batched * (mean_t + se_t)],
            "batched_seconds": dt,
            "sequential_sample": f"{sample} of {len(lats)} lattices, every {step:g}-th by beam count; "
                                 f"{mean_t:.3f} +/- {se_t:.3f} s per lattice (standard error), {sum(times):.1f} s",
            "completed": int((np.asarray(status) == 0).sum()), "lattices": len(lats),
            "beams": int(sum(l.n_beams for l in lats)), "sample_frames_identical_to_batch": bool(same),
            "broad_phase": tune, "cpu_reference": cpu_ref,
            "workload": "256 cubic+BCC lattices, 4-16 cells per side, radius 0.3 mm + U[0, 0.1] mm/cell "
                        "(capped 0.7 mm), yield U[30, 70] MPa, 30 % strain in 100 increments"}


if __name__ == "__main__":
    main()
