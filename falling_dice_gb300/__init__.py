"""GB300-native beam-lattice energy/gradient and L-BFGS solver (libmcg.so, include/mcg.h).

The compute path is the CUDA library; this module is the Python-side binding of its C ABI,
with the same operations as the reference solver's Simulator (objective, minimize, commit,
run) in projects/metamaterial-compression/industry-grade/src/sim.cpp.  There is no CPU
fallback: without the built library every entry point raises.
"""
import ctypes as C
import os

import numpy as np

from . import abi
from .lattice import LatticeArrays

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmcg.so")

_lib = None

_d = C.POINTER(C.c_double)
_i32 = C.POINTER(C.c_int32)
_u8 = C.POINTER(C.c_uint8)
_u64 = C.POINTER(C.c_uint64)
_P = C.c_void_p

SIGNATURES = {
    "mcg_abi_version": (C.c_int, []),
    "mcg_config_defaults": (None, [C.POINTER(abi.Config)]),
    "mcg_status_string": (C.c_char_p, [C.c_int]),
    "mcg_create": (C.c_int, [C.POINTER(abi.Config), C.c_int, C.POINTER(_P)]),
    "mcg_destroy": (None, [_P]),
    "mcg_last_error": (C.c_char_p, [_P]),
    "mcg_upload_topology": (C.c_int, [_P, C.POINTER(abi.Topology), C.POINTER(abi.Geometry), _d, _d]),
    "mcg_set_state": (C.c_int, [_P, _d, _d, _d]),
    "mcg_get_state": (C.c_int, [_P, _d, _d, _d]),
    "mcg_objective": (C.c_int, [_P, _d, C.c_double, C.c_int, _d, _d, C.POINTER(abi.Diag), _d, _d, _u8]),
    "mcg_objective_noalloc": (C.c_int, [_P, _d, C.c_double, _d, _d, C.POINTER(abi.Diag)]),
    "mcg_upload_z": (C.c_int, [_P, _d]),
    "mcg_objective_resident": (C.c_int, [_P, C.c_double, C.c_int]),
    "mcg_read_result": (C.c_int, [_P, _d, _d, C.POINTER(abi.Diag)]),
    "mcg_contact_pairs": (C.c_int, [_P, _u64, C.c_int64, C.POINTER(C.c_int64)]),
    "mcg_minimize": (C.c_int, [_P, C.c_double, _d, C.POINTER(abi.OptStats), _d, C.POINTER(abi.Diag)]),
    "mcg_commit": (C.c_int, [_P]),
    "mcg_run": (C.c_int, [_P, C.POINTER(abi.Frame), C.c_int32, _i32, C.c_int]),
    "mcg_stream": (_P, [_P]),
    "mcg_launch_count": (C.c_int64, [_P]),
    "mcg_set_timing": (C.c_int, [_P, C.c_int]),
    "mcg_set_contact_capacity": (C.c_int, [_P, C.c_int64, C.c_int64, C.c_int64, C.c_int64]),
    "mcg_set_contact_skin": (C.c_int, [_P, C.c_double]),
    "mcg_contact_stats": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "mcg_set_contact_cell": (C.c_int, [_P, C.c_double]),
    "mcg_autotune": (C.c_int, [_P, _d, _d, C.c_int32, C.POINTER(abi.Tuning)]),
    "mcg_set_contact_shapes": (C.c_int, [_P, C.c_double, C.c_int32]),
    "mcg_set_kernel_shapes": (C.c_int, [_P, C.c_int32, C.c_int32]),
    "mcg_contact_builds": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "mcg_set_solver_loop": (C.c_int, [_P, C.c_int]),
    "mcg_solver_loop": (C.c_int, [_P, C.POINTER(C.c_int32)]),
    "mcg_solver_times": (C.c_int, [_P, _d, C.POINTER(C.c_int64)]),
    "mcg_upload_batch": (C.c_int, [_P, C.c_int32, C.POINTER(abi.Topology), C.POINTER(abi.Geometry),
                                   C.POINTER(_d), C.POINTER(_d), _d]),
    "mcg_instance_count": (C.c_int32, [_P]),
    "mcg_batch_objective": (C.c_int, [_P, _d, _d, _d, _d, C.POINTER(abi.Diag)]),
    "mcg_batch_run": (C.c_int, [_P, C.POINTER(abi.Frame), C.c_int32, _i32, _i32]),
    "mcg_phase_times": (C.c_int, [_P, _d, C.c_int32, C.POINTER(C.c_int64)]),
    "mcg_lattice_generate": (C.c_int, [C.POINTER(abi.LatticeSpec), C.POINTER(abi.Config), C.POINTER(_P)]),
    "mcg_lattice_view_of": (C.c_int, [_P, C.POINTER(abi.LatticeView)]),
    "mcg_lattice_free": (None, [_P]),
    "mcg_lattice_topology": (C.c_int, [_P, C.POINTER(abi.Topology)]),
    "mcg_random_state": (C.c_int, [C.c_int32, C.c_int32, _u8, C.c_double, C.c_double, C.c_double,
                                   C.c_uint64, _d, _d]),
    "mcg_write_metrics_csv": (C.c_int, [C.POINTER(abi.Frame), C.c_int32, C.c_char_p]),
    "mcg_write_summary_json": (C.c_int, [C.POINTER(abi.Frame), C.c_int32, C.POINTER(abi.Config), C.c_double,
                                         C.c_char_p, C.c_char_p]),
}


class MCGError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{message} (status {status})")
        self.status = status


def load(path=LIB_PATH):
    """Loads libmcg.so and binds every exported entry point; raises if it is not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError(
            f"{path} is not built: run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _ptr(a, t=_d):
    return None if a is None else a.ctypes.data_as(t)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def generate_lattice(spec, cfg):
    """Builds a synthetic lattice (mcg_lattice_generate) and copies it into numpy arrays."""
    lib = load()
    h = _P()
    rc = lib.mcg_lattice_generate(C.byref(spec), C.byref(cfg), C.byref(h))
    if rc:
        raise MCGError(rc, "mcg_lattice_generate failed")
    try:
        v = abi.LatticeView()
        lib.mcg_lattice_view_of(h, C.byref(v))
        N, B, nc = v.n_nodes, v.n_beams, v.n_connected

        def arr(p, n, dt):
            return np.ctypeslib.as_array(p, shape=(n,)).astype(dt, copy=True)
        a = LatticeArrays()
        a.x0, a.r0 = arr(v.x0, 3 * N, np.float64), arr(v.r0, 4 * N, np.float64)
        a.layer, a.mass = arr(v.layer, N, np.int32), arr(v.mass, N, np.float64)
        a.locked = arr(v.locked, 6 * N, np.uint8)
        a.beam_a, a.beam_b = arr(v.beam_a, B, np.int32), arr(v.beam_b, B, np.int32)
        for f in ("L0", "radius", "area", "I", "J"):
            setattr(a, f, arr(getattr(v, f), B, np.float64))
        a.e0 = arr(v.e0, 3 * B, np.float64)
        a.connected = arr(v.connected, nc, np.uint64) if nc else np.zeros(0, np.uint64)
        g = v.geometry
        a.geometry = abi.Geometry(g.width, g.height, g.depth, g.area, g.mass, g.top0)
        a.translation_scale = cfg.translation_scale
        return a
    finally:
        lib.mcg_lattice_free(h)


def random_state(lattice, sigma_t, sigma_r, epsp_max, seed):
    """Seeded deformed state (mcg_random_state): returns (z, plastic)."""
    lib = load()
    z = np.zeros(6 * lattice.n_nodes)
    pl = np.zeros(7 * lattice.n_beams)
    rc = lib.mcg_random_state(lattice.n_nodes, lattice.n_beams, _ptr(lattice.locked, _u8), sigma_t,
                              sigma_r, epsp_max, seed, _ptr(z), _ptr(pl))
    if rc:
        raise MCGError(rc, "mcg_random_state failed")
    return z, pl


def _frames_array(frames):
    arr = (abi.Frame * max(len(frames), 1))()
    for i, f in enumerate(frames):
        for k, v in f.items():
            setattr(arr[i], k, v)
    return arr


def write_metrics_csv(frames, path):
    """The reference CLI's per-increment metrics CSV of a run's frames (mcg_write_metrics_csv)."""
    rc = load().mcg_write_metrics_csv(_frames_array(frames), len(frames), os.fsencode(path))
    if rc:
        raise MCGError(rc, f"cannot write {path}")


def write_summary_json(frames, cfg, mass_kg, path, material=abi.REFERENCE_MATERIAL_NAME):
    """The reference CLI's summary.json of a run (mcg_write_summary_json)."""
    rc = load().mcg_write_summary_json(_frames_array(frames), len(frames), C.byref(cfg), float(mass_kg),
                                       material.encode(), os.fsencode(path))
    if rc:
        raise MCGError(rc, f"cannot write {path}")


class Solver:
    """One device context holding one lattice: the reference Simulator's energy/gradient,
    minimize, commit and run, on the GPU."""

    def __init__(self, cfg, lattice, device=0):
        self.lib = load()
        self.cfg = cfg
        self.h = _P()
        self._check(self.lib.mcg_create(C.byref(cfg), device, C.byref(self.h)), "mcg_create", ctx=False)
        self.lattice = lattice
        topo, geom = lattice.topology()
        self._check(self.lib.mcg_upload_topology(self.h, C.byref(topo), C.byref(geom),
                                                 _ptr(lattice.x0), _ptr(lattice.r0)),
                    "mcg_upload_topology")
        self.n_nodes, self.n_beams = lattice.n_nodes, lattice.n_beams

    def _check(self, rc, what, ctx=True):
        if rc:
            msg = self.lib.mcg_last_error(self.h).decode() if ctx and self.h else \
                self.lib.mcg_status_string(rc).decode()
            raise MCGError(rc, f"{what}: {msg}")

    def close(self):
        if getattr(self, "h", None):
            self.lib.mcg_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def set_state(self, base_x=None, base_r=None, plastic=None):
        self._check(self.lib.mcg_set_state(self.h, _ptr(_f64(base_x)), _ptr(_f64(base_r)),
                                           _ptr(_f64(plastic))), "mcg_set_state")

    def get_state(self):
        bx = np.zeros(3 * self.n_nodes)
        br = np.zeros(4 * self.n_nodes)
        pl = np.zeros(7 * self.n_beams)
        self._check(self.lib.mcg_get_state(self.h, _ptr(bx), _ptr(br), _ptr(pl)), "mcg_get_state")
        return bx, br, pl

    def objective(self, z, top, trials=False):
        z = _f64(z)
        e = C.c_double()
        grad = np.zeros(6 * self.n_nodes)
        diag = abi.Diag()
        nxt = aux = flags = None
        if trials:
            nxt = np.zeros(7 * self.n_beams)
            aux = np.zeros(7 * self.n_beams)
            flags = np.zeros(3 * self.n_beams, np.uint8)
        self._check(self.lib.mcg_objective(self.h, _ptr(z), top, int(trials), C.byref(e), _ptr(grad),
                                           C.byref(diag), _ptr(nxt), _ptr(aux), _ptr(flags, _u8)),
                    "mcg_objective")
        out = {"energy": e.value, "grad": grad, "diag": diag.as_dict()}
        if trials:
            out.update(trial_next=nxt, trial_aux=aux, trial_flags=flags)
        return out

    def upload_z(self, z):
        self._check(self.lib.mcg_upload_z(self.h, _ptr(_f64(z))), "mcg_upload_z")

    def objective_resident(self, top, trials=False):
        self._check(self.lib.mcg_objective_resident(self.h, top, int(trials)), "mcg_objective_resident")

    def read_result(self, grad=True):
        e = C.c_double()
        g = np.zeros(6 * self.n_nodes) if grad else None
        diag = abi.Diag()
        self._check(self.lib.mcg_read_result(self.h, C.byref(e), _ptr(g), C.byref(diag)), "mcg_read_result")
        return {"energy": e.value, "grad": g, "diag": diag.as_dict()}

    def contact_pairs(self):
        n = C.c_int64()
        rc = self.lib.mcg_contact_pairs(self.h, None, 0, C.byref(n))
        if rc not in (abi.MCG_OK, abi.MCG_ERR_CAPACITY):
            self._check(rc, "mcg_contact_pairs")
        keys = np.zeros(max(n.value, 1), np.uint64)
        self._check(self.lib.mcg_contact_pairs(self.h, _ptr(keys, _u64), n.value, C.byref(n)),
                    "mcg_contact_pairs")
        return keys[:n.value]

    def minimize(self, top, z):
        z = np.array(z, dtype=np.float64, copy=True)
        st = abi.OptStats()
        fe = C.c_double()
        fd = abi.Diag()
        self._check(self.lib.mcg_minimize(self.h, top, _ptr(z), C.byref(st), C.byref(fe), C.byref(fd)),
                    "mcg_minimize")
        return z, st.as_dict(), fe.value, fd.as_dict()

    def commit(self):
        self._check(self.lib.mcg_commit(self.h), "mcg_commit")

    def run(self, verbose=False):
        cap = self.cfg.load_steps + self.cfg.unload_steps + 1 + 4096
        frames = (abi.Frame * cap)()
        count = C.c_int32()
        rc = self.lib.mcg_run(self.h, frames, cap, C.byref(count), int(verbose))
        if rc not in (abi.MCG_OK, abi.MCG_ERR_EQUILIBRIUM):
            self._check(rc, "mcg_run")
        return rc, [frames[i].as_dict() for i in range(min(count.value, cap))]

    @property
    def stream(self):
        return self.lib.mcg_stream(self.h)

    def launch_count(self):
        return self.lib.mcg_launch_count(self.h)

    def contact_stats(self):
        """Entries, occupied bins, candidates, filtered candidates and contacts of the last list
        build / evaluation."""
        out = (C.c_int64 * 5)()
        self._check(self.lib.mcg_contact_stats(self.h, out), "mcg_contact_stats")
        return dict(zip(("entries", "occupied_bins", "candidates", "filtered", "contacts"), list(out)))

    def set_solver_loop(self, device):
        """Solver rounds as a device-resident graph loop (True, the default) or stepped from the
        host (False); mcg_set_solver_loop."""
        self._check(self.lib.mcg_set_solver_loop(self.h, int(bool(device))), "mcg_set_solver_loop")

    def solver_times(self):
        """Device-resident loop time by stage (ms) and rounds (mcg_solver_times)."""
        ms = np.zeros(4)
        n = C.c_int64()
        self._check(self.lib.mcg_solver_times(self.h, _ptr(ms), C.byref(n)), "mcg_solver_times")
        return {"directions": ms[0], "evaluations": ms[1], "decisions_accept": ms[2], "loop_wall": ms[3],
                "rounds": n.value}

    def solver_loop(self):
        """(device loop in use, why not when it was switched off)."""
        v = C.c_int32()
        self._check(self.lib.mcg_solver_loop(self.h, C.byref(v)), "mcg_solver_loop")
        return bool(v.value), ("" if v.value else self.lib.mcg_last_error(self.h).decode())

    def contact_builds(self):
        """Candidate-list builds since the upload (mcg_contact_builds)."""
        n = C.c_int64()
        self._check(self.lib.mcg_contact_builds(self.h, C.byref(n)), "mcg_contact_builds")
        return n.value

    def set_contact_cell(self, cell):
        """Contact-grid cell size in metres (0: the reference's)."""
        self._check(self.lib.mcg_set_contact_cell(self.h, float(cell)), "mcg_set_contact_cell")

    def autotune(self, z=None, tops=None, reps=3):
        """Times the broad-phase shape candidates (grid cell, pair-enumeration grid) at z
        (None: 0) and platen heights tops (None: each lattice's top0), keeps the fastest and
        returns the choice; the candidates must agree bit for bit (mcg_autotune)."""
        zp = None if z is None else np.ascontiguousarray(z, np.float64)
        if zp is not None and zp.size != 6 * self.n_nodes:
            raise ValueError("z must hold 6 values per node")
        tp = None if tops is None else np.ascontiguousarray(np.atleast_1d(tops), np.float64)
        if tp is not None and tp.size != getattr(self, "count", 1):
            raise ValueError("tops must hold one platen height per lattice")
        t = abi.Tuning()
        self._check(self.lib.mcg_autotune(self.h, _ptr(zp), _ptr(tp), int(reps), C.byref(t)),
                    "mcg_autotune")
        return {"cell": t.cell, "pair_blocks": t.pair_blocks, "tried": t.tried,
                "ms_chosen": t.ms_chosen, "ms_default": t.ms_default,
                "beam_blocks": t.beam_blocks, "gather_blocks": t.gather_blocks}

    def set_kernel_shapes(self, beam_blocks, gather_blocks):
        """Occupancy of the beam kernel and the gather (CTAs per SM, 0: default), as autotune()
        reports them."""
        self._check(self.lib.mcg_set_kernel_shapes(self.h, int(beam_blocks), int(gather_blocks)),
                    "mcg_set_kernel_shapes")

    def set_contact_shapes(self, cell, pair_blocks):
        """Grid cell (m, 0: the reference's) and pair-enumeration blocks (0: default), as
        autotune() reports them."""
        self._check(self.lib.mcg_set_contact_shapes(self.h, float(cell), int(pair_blocks)),
                    "mcg_set_contact_shapes")

    def set_contact_skin(self, skin):
        """Candidate-list reuse distance in metres (0: rebuild at every evaluation)."""
        self._check(self.lib.mcg_set_contact_skin(self.h, float(skin)), "mcg_set_contact_skin")

    def set_contact_capacity(self, entries, candidates, contacts, bins):
        self._check(self.lib.mcg_set_contact_capacity(self.h, entries, candidates, contacts, bins),
                    "mcg_set_contact_capacity")

    PHASES = ("state", "beams", "grid", "pairs", "narrow", "gather", "finalize")

    def set_timing(self, on):
        self._check(self.lib.mcg_set_timing(self.h, int(on)), "mcg_set_timing")

    def phase_times(self):
        """Summed milliseconds per evaluation phase since timing was switched on; "contacts"
        is grid + pairs + narrow."""
        ms = np.zeros(len(self.PHASES))
        n = C.c_int64()
        self._check(self.lib.mcg_phase_times(self.h, _ptr(ms), len(ms), C.byref(n)), "mcg_phase_times")
        out = dict(zip(self.PHASES, ms))
        out["contacts"] = out["grid"] + out["pairs"] + out["narrow"]
        return out, n.value


class BatchSolver(Solver):
    """One device context holding many lattices (mcg_upload_batch): every evaluation,
    minimizer step and load/unload increment of all of them runs in the same launches.
    `yields` gives each lattice's yield stress (default: the configuration's)."""

    def __init__(self, cfg, lattices, yields=None, device=0):
        self.lib = load()
        self.cfg = cfg
        self.h = _P()
        self._check(self.lib.mcg_create(C.byref(cfg), device, C.byref(self.h)), "mcg_create", ctx=False)
        self.lattices = list(lattices)
        k = len(self.lattices)
        topos = (abi.Topology * k)()
        geoms = (abi.Geometry * k)()
        x0 = (_d * k)()
        r0 = (_d * k)()
        for i, lat in enumerate(self.lattices):
            t, g = lat.topology()
            topos[i], geoms[i] = t, g
            x0[i], r0[i] = _ptr(lat.x0), _ptr(lat.r0)
        self._keep = (topos, geoms, x0, r0, [lat.topology() for lat in self.lattices])
        y = None if yields is None else np.ascontiguousarray(yields, dtype=np.float64)
        self._check(self.lib.mcg_upload_batch(self.h, k, topos, geoms, x0, r0, _ptr(y)), "mcg_upload_batch")
        self.count = k
        self.node_offsets = np.cumsum([0] + [lat.n_nodes for lat in self.lattices])
        self.n_nodes = int(self.node_offsets[-1])
        self.n_beams = sum(lat.n_beams for lat in self.lattices)

    def objective(self, z, tops):
        z = _f64(z)
        tops = _f64(tops)
        e = np.zeros(self.count)
        grad = np.zeros(6 * self.n_nodes)
        diags = (abi.Diag * self.count)()
        self._check(self.lib.mcg_batch_objective(self.h, _ptr(z), _ptr(tops), _ptr(e), _ptr(grad), diags),
                    "mcg_batch_objective")
        return {"energy": e, "grad": grad, "diag": [diags[i].as_dict() for i in range(self.count)]}

    def run(self, verbose=False):
        cap = self.cfg.load_steps + self.cfg.unload_steps + 1 + 4096
        frames = (abi.Frame * (cap * self.count))()
        counts = np.zeros(self.count, np.int32)
        status = np.zeros(self.count, np.int32)
        self._check(self.lib.mcg_batch_run(self.h, frames, cap, _ptr(counts, _i32), _ptr(status, _i32)),
                    "mcg_batch_run")
        return status, [[frames[i * cap + f].as_dict() for f in range(counts[i])] for i in range(self.count)]
