"""Lattice arrays on the host: the model the objective reads (Node/Beam in the reference,
projects/metamaterial-compression/industry-grade/include/sim.hpp:27-29) as numpy arrays.

Lattices come from the library's generator (mcg_lattice_generate, cubic and cubic+BCC
synthetic specimens) or from any other source that fills the same arrays.
"""
import ctypes as C

import numpy as np

from . import abi


class LatticeArrays:
    FIELDS = ("x0", "r0", "layer", "mass", "locked", "beam_a", "beam_b", "L0", "radius",
              "area", "I", "J", "e0", "connected")

    def __init__(self):
        self.geometry = abi.Geometry()
        self.translation_scale = None

    @classmethod
    def empty(cls, n_nodes, n_beams, n_connected):
        a = cls()
        N, B = n_nodes, n_beams
        a.x0 = np.zeros(3 * N)
        a.r0 = np.zeros(4 * N)
        a.layer = np.zeros(N, np.int32)
        a.mass = np.zeros(N)
        a.locked = np.zeros(6 * N, np.uint8)
        a.beam_a = np.zeros(B, np.int32)
        a.beam_b = np.zeros(B, np.int32)
        for f in ("L0", "radius", "area", "I", "J"):
            setattr(a, f, np.zeros(B))
        a.e0 = np.zeros(3 * B)
        a.connected = np.zeros(n_connected, np.uint64)
        return a

    @property
    def n_nodes(self):
        return len(self.mass)

    @property
    def n_beams(self):
        return len(self.L0)

    def topology(self):
        """(Topology, Geometry) ctypes structures pointing into these arrays."""
        t = abi.Topology()
        t.n_nodes, t.n_beams = self.n_nodes, self.n_beams
        d = C.POINTER(C.c_double)
        t.beam_a = self.beam_a.ctypes.data_as(C.POINTER(C.c_int32))
        t.beam_b = self.beam_b.ctypes.data_as(C.POINTER(C.c_int32))
        for f in ("L0", "radius", "area", "I", "J", "e0", "mass"):
            setattr(t, f, getattr(self, f).ctypes.data_as(d))
        t.locked = self.locked.ctypes.data_as(C.POINTER(C.c_uint8))
        t.n_connected = len(self.connected)
        t.connected = self.connected.ctypes.data_as(C.POINTER(C.c_uint64))
        t._keep = self  # keep the arrays alive with the structure
        return t, self.geometry

    def save(self, path):
        g = self.geometry
        np.savez_compressed(
            path, **{f: getattr(self, f) for f in self.FIELDS},
            geometry=np.array([g.width, g.height, g.depth, g.area, g.mass, g.top0]),
            translation_scale=np.array([self.translation_scale or 0.0]))

    @classmethod
    def load(cls, path):
        z = np.load(path)
        a = cls()
        for f in cls.FIELDS:
            setattr(a, f, np.ascontiguousarray(z[f]))
        g = z["geometry"]
        a.geometry = abi.Geometry(*[float(v) for v in g])
        a.translation_scale = float(z["translation_scale"][0]) or None
        return a

    def copy(self):
        b = LatticeArrays()
        for f in self.FIELDS:
            setattr(b, f, getattr(self, f).copy())
        b.geometry = abi.Geometry(*[getattr(self.geometry, n) for n, _ in abi.Geometry._fields_])
        b.translation_scale = self.translation_scale
        return b
