"""TEST INFRASTRUCTURE ONLY: Python access to the CPU oracles (oracle/oracle.h).

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs, always as the
checker or the timed CPU baseline, never as the measured product path.

  load("mco")  the CPU restatement (oracle/_build/libmco.so), available everywhere;
  load("ref")  the reference's own solver (oracle/_ref/libmcref.so), only where the
               reference sources were present to build it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from falling_dice_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
PATHS = {"mco": os.path.join(HERE, "_build", "libmco.so"),
         "ref": os.path.join(HERE, "_ref", "libmcref.so")}
REF_ROOT = "/root/reference/projects/metamaterial-compression/industry-grade"

_libs = {}

_d = C.POINTER(C.c_double)
_i32 = C.POINTER(C.c_int32)
_u8 = C.POINTER(C.c_uint8)
_u64 = C.POINTER(C.c_uint64)


def build(which="mco", quiet=True):
    """Builds an oracle library with oracle/Makefile (the reference one needs its sources)."""
    if which == "ref" and not os.path.isdir(REF_ROOT):
        return False
    cmd = ["make", "-s", "-C", HERE, which] + ([f"REF_ROOT={REF_ROOT}"] if which == "ref" else [])
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError(f"oracle build ({which}) failed:\n{out.stdout}\n{out.stderr}")
    return True


def available(which):
    return os.path.exists(PATHS[which])


def load(which="mco"):
    if which in _libs:
        return _libs[which]
    path = PATHS[which]
    if not os.path.exists(path):
        raise FileNotFoundError(f"oracle library {path} is not built")
    lib = C.CDLL(path)
    P = C.c_void_p
    sig = {
        "orc_is_reference": (C.c_int, []),
        "orc_create_builder": (P, [C.POINTER(abi.Config)]),
        "orc_create_injected": (P, [C.POINTER(abi.Config), C.POINTER(abi.Topology),
                                    C.POINTER(abi.Geometry), _d, _d, _i32]),
        "orc_free": (None, [P]),
        "orc_counts": (None, [P, _i32, _i32, C.POINTER(C.c_int64)]),
        "orc_export": (None, [P, _d, _d, _i32, _d, _u8, _i32, _i32, _d, _d, _d, _d, _d, _d,
                              _u64, C.POINTER(abi.Geometry), _d]),
        "orc_set_state": (None, [P, _d, _d, _d]),
        "orc_get_state": (None, [P, _d, _d, _d]),
        "orc_objective": (C.c_double, [P, _d, C.c_double, C.c_int, _d, C.POINTER(abi.Diag),
                                       _d, _d, _u8]),
        "orc_contact_pairs": (C.c_int64, [P, _d, _u64, C.c_int64]),
        "orc_minimize": (C.c_int, [P, C.c_double, _d, C.POINTER(abi.OptStats), _d,
                                   C.POINTER(abi.Diag)]),
        "orc_commit": (C.c_int, [P]),
        "orc_run": (C.c_int, [P, C.POINTER(abi.Frame), C.c_int32, _i32, C.c_int]),
        "orc_rigid_rotation_error": (C.c_double, [P]),
        "orc_gradient_check_error": (C.c_double, [P]),
        "orc_beam_potential": (C.c_double, [P, _d, _d]),
        "orc_top_y": (C.c_double, [P, C.c_double, C.c_int]),
        "orc_set_variant": (C.c_int, [P, C.c_int]),
    }
    # restatement only
    sig_mco = {
        "orc_set_objective_hook": (None, [P, P, P, P]),
        "orc_hook_status": (C.c_int, [P, C.POINTER(C.c_int64)]),
        "orc_record_pairs": (None, [P, C.c_int]),
        "orc_last_pairs": (C.c_int64, [P, _u64, C.c_int64]),
        "orc_create_specimen": (P, [C.POINTER(abi.Config), C.POINTER(abi.LatticeSpec)]),
        "orc_random_state": (None, [C.c_int32, C.c_int32, _u8, C.c_double, C.c_double, C.c_double,
                                    C.c_uint64, _d, _d]),
    }
    if which == "mco":
        sig.update(sig_mco)
    else:
        sig["orc_ref_write_outputs"] = (C.c_int, [C.POINTER(abi.Frame), C.c_int32, C.POINTER(abi.Config),
                                                  C.c_double, C.c_char_p, C.c_char_p])
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _libs[which] = lib
    return lib


def ptr(a, t=_d):
    return None if a is None else a.ctypes.data_as(t)


class Model:
    """One solver model inside an oracle library (a reference Simulator or its restatement).

    lattice: None (the reference's own builder), a LatticeArrays to inject, or a
    LatticeSpec of a synthetic specimen built by the restatement itself (libmco only)."""

    def __init__(self, which, cfg, lattice=None):
        self.lib = load(which)
        self.which = which
        self.cfg = cfg
        if isinstance(lattice, abi.LatticeSpec):
            if which != "mco":
                raise ValueError("synthetic specimens are built by the restatement only")
            self.h = self.lib.orc_create_specimen(C.byref(cfg), C.byref(lattice))
            if not self.h:
                raise ValueError("invalid specimen")
        elif lattice is None:
            self.h = self.lib.orc_create_builder(C.byref(cfg))
        else:
            topo, geom = lattice.topology()
            self.h = self.lib.orc_create_injected(C.byref(cfg), C.byref(topo), C.byref(geom),
                                                  ptr(lattice.x0), ptr(lattice.r0),
                                                  ptr(lattice.layer, _i32))
        n, b, nc = C.c_int32(), C.c_int32(), C.c_int64()
        self.lib.orc_counts(self.h, C.byref(n), C.byref(b), C.byref(nc))
        self.n_nodes, self.n_beams, self.n_connected = n.value, b.value, nc.value

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_free(self.h)
            self.h = None

    def export(self):
        """The model arrays as a LatticeArrays (same fields as a generated lattice)."""
        from falling_dice_gb300.lattice import LatticeArrays
        N, B = self.n_nodes, self.n_beams
        a = LatticeArrays.empty(N, B, self.n_connected)
        geom = abi.Geometry()
        ts = C.c_double()
        self.lib.orc_export(self.h, ptr(a.x0), ptr(a.r0), ptr(a.layer, _i32), ptr(a.mass),
                            ptr(a.locked, _u8), ptr(a.beam_a, _i32), ptr(a.beam_b, _i32),
                            ptr(a.L0), ptr(a.radius), ptr(a.area), ptr(a.I), ptr(a.J),
                            ptr(a.e0), ptr(a.connected, _u64), C.byref(geom), C.byref(ts))
        a.geometry = geom
        a.translation_scale = ts.value
        return a

    def set_state(self, base_x=None, base_r=None, plastic=None):
        self.lib.orc_set_state(self.h, ptr(_f64(base_x)), ptr(_f64(base_r)), ptr(_f64(plastic)))

    def get_state(self):
        bx = np.zeros(3 * self.n_nodes)
        br = np.zeros(4 * self.n_nodes)
        pl = np.zeros(7 * self.n_beams)
        self.lib.orc_get_state(self.h, ptr(bx), ptr(br), ptr(pl))
        return bx, br, pl

    def objective(self, z, top, trials=False):
        z = _f64(z)
        grad = np.zeros(6 * self.n_nodes)
        diag = abi.Diag()
        out = {"grad": grad}
        nxt = aux = flags = None
        if trials:
            nxt = np.zeros(7 * self.n_beams)
            aux = np.zeros(7 * self.n_beams)
            flags = np.zeros(3 * self.n_beams, np.uint8)
        e = self.lib.orc_objective(self.h, ptr(z), top, int(trials), ptr(grad), C.byref(diag),
                                   ptr(nxt), ptr(aux), ptr(flags, _u8))
        out.update(energy=e, diag=diag.as_dict())
        if trials:
            out.update(trial_next=nxt, trial_aux=aux, trial_flags=flags)
        return out

    def contact_pairs(self, z):
        z = _f64(z)
        n = self.lib.orc_contact_pairs(self.h, ptr(z), None, 0)
        keys = np.zeros(max(n, 1), np.uint64)
        self.lib.orc_contact_pairs(self.h, ptr(z), ptr(keys, _u64), n)
        return keys[:n]

    def minimize(self, top, z):
        z = np.array(z, dtype=np.float64, copy=True)
        st = abi.OptStats()
        fe = C.c_double()
        fd = abi.Diag()
        self.lib.orc_minimize(self.h, top, ptr(z), C.byref(st), C.byref(fe), C.byref(fd))
        return z, st.as_dict(), fe.value, fd.as_dict()

    def commit(self):
        rc = self.lib.orc_commit(self.h)
        if rc:
            raise RuntimeError(f"orc_commit: status {rc}")

    def run(self, verbose=False):
        cap = self.cfg.load_steps + self.cfg.unload_steps + 1 + 4096
        frames = (abi.Frame * cap)()
        count = C.c_int32()
        rc = self.lib.orc_run(self.h, frames, cap, C.byref(count), int(verbose))
        return rc, [frames[i].as_dict() for i in range(min(count.value, cap))]

    def rigid_rotation_error(self):
        return self.lib.orc_rigid_rotation_error(self.h)

    def gradient_check_error(self):
        return self.lib.orc_gradient_check_error(self.h)

    def beam_potential(self, x, r):
        return self.lib.orc_beam_potential(self.h, ptr(_f64(x)), ptr(_f64(r)))

    def set_variant(self, v):
        if self.lib.orc_set_variant(self.h, int(v)) != 0:
            raise ValueError(f"variant {v} not supported by the {self.which} oracle")

    def top_y(self, s, loading):
        return self.lib.orc_top_y(self.h, s, int(loading))

    # -- restatement only ---------------------------------------------------------------
    def set_objective_hook(self, objective_fn, state_fn, ctx):
        """Forwards every evaluation to a C function with mcg_objective's signature (and the
        state after each commit / set_state to one with mcg_set_state's), e.g. libmcg's own
        entry points with a GPU context as ctx.  None removes the hook."""
        as_ptr = (lambda f: None if f is None else C.cast(f, C.c_void_p))
        self._hook_refs = (objective_fn, state_fn, ctx)  # keep them alive
        self.lib.orc_set_objective_hook(self.h, as_ptr(objective_fn), as_ptr(state_fn), ctx)

    def hook_status(self):
        calls = C.c_int64()
        rc = self.lib.orc_hook_status(self.h, C.byref(calls))
        return rc, calls.value

    def record_pairs(self, on=True):
        self.lib.orc_record_pairs(self.h, int(on))

    def last_pairs(self):
        n = self.lib.orc_last_pairs(self.h, None, 0)
        keys = np.zeros(max(n, 1), np.uint64)
        self.lib.orc_last_pairs(self.h, ptr(keys, _u64), n)
        return keys[:n]

    def locked(self):
        a = np.zeros(6 * self.n_nodes, np.uint8)
        self.lib.orc_export(self.h, *([None] * 4), ptr(a, _u8), *([None] * 11))
        return a


def random_state(n_nodes, n_beams, locked, sigma_t, sigma_r, epsp_max, seed):
    """The restatement of mcg_random_state: (z [6N], plastic [7B])."""
    lib = load("mco")
    z = np.zeros(6 * n_nodes)
    pl = np.zeros(7 * n_beams)
    lk = np.ascontiguousarray(locked, dtype=np.uint8)
    lib.orc_random_state(n_nodes, n_beams, ptr(lk, _u8), sigma_t, sigma_r, epsp_max,
                         seed & 0xFFFFFFFFFFFFFFFF, ptr(z), ptr(pl))
    return z, pl


def _f64(a):
    if a is None:
        return None
    return np.ascontiguousarray(a, dtype=np.float64)
