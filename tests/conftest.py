import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from falling_dice_gb300 import abi  # noqa: E402
from falling_dice_gb300.lattice import LatticeArrays  # noqa: E402

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the product kernels")


def config_from(keys, vals):
    cfg = abi.Config()
    for k, v in zip(keys, vals):
        k = str(k)
        v = str(v)
        if k.startswith("material."):
            setattr(cfg.material, k.split(".", 1)[1], float(v))
        else:
            ftype = dict(abi.Config._fields_)[k]
            setattr(cfg, k, int(v) if ftype in (abi.C.c_int32, abi.C.c_uint64) else float(v))
    return cfg


class Golden:
    """A fixture made by tests/golden/make_golden.py from the reference solver."""

    def __init__(self, name):
        self.name = name
        self.d = np.load(os.path.join(GOLDEN, name + ".npz"))
        d = self.d
        lat = LatticeArrays()
        for f in LatticeArrays.FIELDS:
            setattr(lat, f, np.ascontiguousarray(d["lat_" + f]))
        lat.geometry = abi.Geometry(*[float(v) for v in d["lat_geometry"]])
        lat.translation_scale = self.cfg.translation_scale
        self.lattice = lat
        self.n_states = int(d["n_states"][0]) if "n_states" in d else 0

    @property
    def cfg(self):
        """A fresh copy of the fixture's configuration (callers may modify it)."""
        cfg = config_from(self.d["cfg_keys"], self.d["cfg_vals"])
        cfg.translation_scale = float(self.d["translation_scale"][0])
        return cfg

    def state(self, k):
        p = f"s{k}_"
        d = self.d
        s = {"z": d[p + "z"], "top": float(d[p + "top"][0]), "plastic": d[p + "plastic"],
             "trials": bool(d[p + "trials"][0]), "energy": float(d[p + "energy"][0]),
             "grad": d[p + "grad"], "diag": d[p + "diag"], "pairs": d[p + "pairs"]}
        if s["trials"]:
            s.update(trial_next=d[p + "trial_next"], trial_aux=d[p + "trial_aux"],
                     trial_flags=d[p + "trial_flags"])
        return s

    def frames(self):
        keys = [str(k) for k in self.d["frame_keys"]]
        return [dict(zip(keys, row)) for row in self.d["run_frames"]]


_golden_cache = {}


def golden(name):
    if name not in _golden_cache:
        _golden_cache[name] = Golden(name)
    return _golden_cache[name]


@pytest.fixture(scope="session")
def mco():
    from oracle import oracle as orc
    orc.build("mco")
    orc.load("mco")
    return orc


@pytest.fixture(scope="session")
def ref_oracle():
    from oracle import oracle as orc
    if not orc.build("ref"):
        pytest.skip("reference sources not present on this machine")
    orc.load("ref")
    return orc


@pytest.fixture(scope="session")
def mcg():
    import falling_dice_gb300 as fd
    if not os.path.exists(fd.LIB_PATH):
        from falling_dice_gb300 import build
        build.build()
    fd.load()
    return fd


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = max(np.linalg.norm(b), 1e-300)
    return float(np.linalg.norm(a - b) / den)
