"""The synthetic specimens the throughput and parity workloads are defined on.

Each preset returns (cfg, spec): the solver configuration (abi.Config) and the lattice
spec (abi.LatticeSpec) for mcg_lattice_generate.  Inputs are seeded and synthetic; the
reference publishes no dataset for this path.

  cubic6          6x6x6 cubic lattice, 5 mm cells, +/-2 % jitter, radius graded 0.3->0.6 mm
                  in height, E 2 GPa, nu 0.35, yield 50 MPa, hardening 5 % of E; 40 % strain
                  in 200 loading + 200 unloading increments, L-BFGS history 10.
  bcc64           64x64x32 cubic+BCC lattice, radii uniform 0.3-0.6 mm, +/-2 % jitter; one
                  evaluation at a seeded deformed state (displacement N(0, 0.05 cell), rotation
                  angle N(0, 0.1 rad), plastic strain U[0, 0.02]).
  bcc32           32x32x16 cubic+BCC, radius graded 0.25->0.7 mm, +/-3 % jitter, 60 % strain,
                  400 loading + 400 unloading increments, penalty stiffness scaled to E.
  bcc128          128x128x64 cubic+BCC, radii uniform 0.3-0.6 mm, +/-2 % jitter, 50 % strain in
                  100 increments, penalty stiffness scaled to E.
  sweep           256 cubic+BCC lattices of 4-16 cells per side with per-lattice radius
                  grading and yield stress, 30 % strain in 100 increments (batched).
"""
from . import abi

CELL = 0.005
SEED = abi.REFERENCE_SEED

# material of the throughput specimens: E = 2.0 GPa, nu = 0.35, yield 50 MPa, H = 5 % E
MATERIAL = dict(young=2.0e9, nu=0.35, yield_=50e6, hardening=1.0e8)

# Penalty stiffness of the load/unload specimens: the reference's default (1.2e6 N/m) is
# sized for its own 26 MPa material; scaled by the modulus ratio it keeps platen
# penetration well inside the 0.12 mm tolerance at the forces a 2 GPa lattice carries.
CONTACT_STIFF = 1.2e6 * 2.0e9 / 26e6


def _cfg(r0, r1, **kw):
    base = dict(cell_size=CELL, min_radius=r0, max_radius=r1, history=10, max_iterations=800,
                **MATERIAL)
    base.update(kw)
    return abi.default_config(**base)


def _spec(kind, mode, cells, r0, r1, jitter, seed=SEED):
    s = abi.LatticeSpec()
    s.kind, s.radius_mode = kind, mode
    s.cells_x, s.cells_y, s.cells_z = cells
    s.cell_size, s.r0, s.r1, s.jitter, s.seed = CELL, r0, r1, jitter, seed
    return s


def cubic6():
    cfg = _cfg(0.3e-3, 0.6e-3, max_strain=0.4, load_steps=200, unload_steps=200)
    return cfg, _spec(abi.MCG_LATTICE_CUBIC, abi.MCG_RADIUS_GRADED_Y, (6, 6, 6), 0.3e-3, 0.6e-3, 0.02)


def bcc(cells, r0=0.3e-3, r1=0.6e-3, jitter=0.02, mode=abi.MCG_RADIUS_UNIFORM, **kw):
    cfg = _cfg(r0, r1, **kw)
    return cfg, _spec(abi.MCG_LATTICE_CUBIC_BCC, mode, cells, r0, r1, jitter)


def bcc64():
    return bcc((64, 64, 32))


def bcc32():
    return bcc((32, 32, 16), 0.25e-3, 0.7e-3, 0.03, abi.MCG_RADIUS_GRADED_Y, max_strain=0.6,
               load_steps=400, unload_steps=400, contact_stiffness=CONTACT_STIFF)


def bcc128():
    return bcc((128, 128, 64), max_strain=0.5, load_steps=100, unload_steps=0, contact_stiffness=CONTACT_STIFF)


# deformed state of the single-evaluation workload
DEFORM = dict(sigma_t=0.05, sigma_r=0.1, epsp_max=0.02, seed=SEED ^ 0xD3F0)


def sweep(count=256, seed=SEED ^ 0x5357):
    """The batched sweep: `count` cubic+BCC lattices with cells per side U{4..16} (cubic
    blocks), radius graded in height from 0.3 mm with a slope U[0, 0.1] mm per cell and
    capped at 0.7 mm (the largest radius of the other specimens; uncapped, a 16-cell lattice
    would reach 1.9 mm struts in 5 mm cells, overlapping at rest), yield stress U[30, 70] MPa,
    +/-2 % jitter, 30 % strain in 100 loading increments.  Returns (cfg, specs, yields); the
    configuration is shared, the yield is per lattice."""
    import numpy as np
    rng = np.random.default_rng(seed & 0xFFFFFFFFFFFFFFFF)
    cfg = _cfg(0.3e-3, 0.6e-3, max_strain=0.3, load_steps=100, unload_steps=0, contact_stiffness=CONTACT_STIFF)
    specs, yields = [], []
    for k in range(count):
        n = int(rng.integers(4, 17))
        slope = float(rng.uniform(0.0, 0.1e-3))
        r0 = 0.3e-3
        s = _spec(abi.MCG_LATTICE_CUBIC_BCC, abi.MCG_RADIUS_GRADED_Y, (n, n, n), r0, min(r0 + slope * n, 0.7e-3), 0.02,
                  seed=(SEED + 7919 * (k + 1)) & 0xFFFFFFFFFFFFFFFF)
        specs.append(s)
        yields.append(float(rng.uniform(30e6, 70e6)))
    return cfg, specs, yields
