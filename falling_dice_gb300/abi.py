"""ctypes mirror of include/mcg.h (structures, enums and the reference defaults).

The layouts here must match include/mcg.h field for field; tests/test_abi.py checks the
sizes against the compiled library.  Defaults are SimulationConfig / MaterialConfig
(projects/metamaterial-compression/industry-grade/include/sim.hpp:16-26).
"""
import ctypes as C

MCG_OK = 0
MCG_ERR_INVALID = 1
MCG_ERR_CUDA = 2
MCG_ERR_NO_DEVICE = 3
MCG_ERR_STATE = 4
MCG_ERR_EQUILIBRIUM = 5
MCG_ERR_CAPACITY = 6
MCG_ERR_TIMEOUT = 7
MCG_ERR_MISMATCH = 8

MCG_FP64 = 0
MCG_MIXED = 1

MCG_LATTICE_CUBIC = 0
MCG_LATTICE_CUBIC_BCC = 1
MCG_LATTICE_REFERENCE_BCC = 2
MCG_RADIUS_GRADED_Y = 0
MCG_RADIUS_UNIFORM = 1

REFERENCE_SEED = 0x494E445553545259  # sim.hpp:25
REFERENCE_MATERIAL_NAME = "FFF TPU 95A provisional isotropic baseline"  # MaterialConfig::name, sim.hpp:16


class Material(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "density", "young", "nu", "yield_", "hardening", "bend_hardening",
        "torsion_hardening")]


class Config(C.Structure):
    _fields_ = [
        ("cells_x", C.c_int32), ("cells_y", C.c_int32), ("cells_z", C.c_int32),
        ("elements_per_strut", C.c_int32),
        ("cell_size", C.c_double), ("min_radius", C.c_double), ("max_radius", C.c_double),
        ("joint_scale", C.c_double), ("trigger_scale", C.c_double),
        ("imperfection", C.c_double), ("member_imperfection", C.c_double),
        ("material", Material),
        ("gravity", C.c_double), ("shear_correction", C.c_double),
        ("contact_stiffness", C.c_double), ("contact_margin", C.c_double),
        ("centering_stiffness", C.c_double),
        ("contact_samples", C.c_int32), ("load_steps", C.c_int32),
        ("unload_steps", C.c_int32), ("max_iterations", C.c_int32),
        ("history", C.c_int32), ("max_line_search", C.c_int32),
        ("max_strain", C.c_double), ("step_time", C.c_double),
        ("translation_scale", C.c_double), ("max_translation_step", C.c_double),
        ("max_rotation_step", C.c_double),
        ("gradient_rms_tolerance", C.c_double), ("gradient_max_tolerance", C.c_double),
        ("armijo", C.c_double), ("min_line_step", C.c_double),
        ("penetration_tolerance", C.c_double),
        ("max_adaptive_refinements", C.c_int32), ("fps", C.c_int32),
        ("frames", C.c_int32), ("threads", C.c_int32),
        ("seed", C.c_uint64),
        ("relative_gradient_tolerance", C.c_double),
        ("precision", C.c_int32), ("self_contact", C.c_int32),
        ("reaction_relative_tolerance", C.c_double),
    ]


def default_config(**overrides):
    """SimulationConfig defaults (sim.hpp:17-26), then keyword overrides.

    translation_scale is set to cell_size, as the reference constructor does
    (sim.cpp:49), unless given explicitly.
    """
    c = Config()
    c.cells_x, c.cells_y, c.cells_z = 4, 6, 4
    c.elements_per_strut = 3
    c.cell_size, c.min_radius, c.max_radius = 0.010, 0.00082, 0.00122
    c.joint_scale, c.trigger_scale = 1.18, 0.38
    c.imperfection, c.member_imperfection = 0.00022, 0.00022
    m = c.material
    m.density, m.young, m.nu, m.yield_, m.hardening = 1180.0, 26e6, 0.485, 5.2e6, 1.4e6
    m.bend_hardening, m.torsion_hardening = 0.06, 0.045
    c.gravity, c.shear_correction, c.contact_stiffness = 9.81, 0.62, 1.2e6
    c.contact_margin, c.centering_stiffness = 2e-5, 1.5
    c.contact_samples, c.load_steps, c.unload_steps = 3, 52, 30
    c.max_iterations, c.history, c.max_line_search = 130, 10, 22
    c.max_strain, c.step_time = 0.62, 0.06
    c.translation_scale, c.max_translation_step, c.max_rotation_step = 0.010, 0.0022, 0.30
    c.gradient_rms_tolerance, c.gradient_max_tolerance = 1.2e-3, 1.5e-2
    c.armijo, c.min_line_step, c.penetration_tolerance = 1e-4, 1e-9, 0.00012
    c.max_adaptive_refinements, c.fps, c.frames, c.threads = 7, 24, 83, 0
    c.seed = REFERENCE_SEED
    c.relative_gradient_tolerance = 0.0
    c.precision = MCG_FP64
    c.self_contact = 1
    c.reaction_relative_tolerance = 1.5e-3  # sim.cpp:177
    ts_given = "translation_scale" in overrides
    for k, v in overrides.items():
        if k in ("density", "young", "nu", "yield_", "hardening", "bend_hardening",
                 "torsion_hardening"):
            setattr(c.material, k, v)
        else:
            setattr(c, k, v)
    if not ts_given:
        c.translation_scale = c.cell_size
    return c


class Topology(C.Structure):
    _fields_ = [
        ("n_nodes", C.c_int32), ("n_beams", C.c_int32),
        ("beam_a", C.POINTER(C.c_int32)), ("beam_b", C.POINTER(C.c_int32)),
        ("L0", C.POINTER(C.c_double)), ("radius", C.POINTER(C.c_double)),
        ("area", C.POINTER(C.c_double)), ("I", C.POINTER(C.c_double)),
        ("J", C.POINTER(C.c_double)), ("e0", C.POINTER(C.c_double)),
        ("mass", C.POINTER(C.c_double)), ("locked", C.POINTER(C.c_uint8)),
        ("n_connected", C.c_int64), ("connected", C.POINTER(C.c_uint64)),
    ]


class Geometry(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("width", "height", "depth", "area", "mass", "top0")]


class Diag(C.Structure):
    _fields_ = [("elastic", C.c_double), ("plastic", C.c_double), ("contact", C.c_double),
                ("reaction", C.c_double), ("max_pen", C.c_double),
                ("contacts", C.c_int32), ("pad_", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k in
                ("elastic", "plastic", "contact", "reaction", "max_pen", "contacts")}


class Tuning(C.Structure):
    _fields_ = [("cell", C.c_double), ("pair_blocks", C.c_int32), ("tried", C.c_int32),
                ("ms_chosen", C.c_double), ("ms_default", C.c_double),
                ("beam_blocks", C.c_int32), ("gather_blocks", C.c_int32)]


class OptStats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("backtracks", C.c_int32),
                ("rms", C.c_double), ("max", C.c_double), ("energy", C.c_double),
                ("converged", C.c_int32), ("pad_", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k in
                ("iterations", "backtracks", "rms", "max", "energy", "converged")}


FRAME_DOUBLES = (
    "time", "platen_y", "displacement", "engineering_strain", "engineering_stress",
    "reaction_force", "loading_work", "recovered_work", "dissipated_work",
    "specific_energy_absorption", "elastic_energy", "plastic_dissipation", "contact_energy",
    "residual_rms", "residual_max", "max_penetration", "mean_plastic_strain",
    "max_plastic_strain", "mean_plastic_rotation", "max_plastic_rotation", "permanent_set")
FRAME_INTS = ("active_contacts", "plastic_beams", "plastic_hinges", "iterations",
              "converged", "loading", "refinement", "pad_")


class Frame(C.Structure):
    _fields_ = [(n, C.c_double) for n in FRAME_DOUBLES] + [(n, C.c_int32) for n in FRAME_INTS]

    def as_dict(self):
        return {k: getattr(self, k) for k in FRAME_DOUBLES + FRAME_INTS[:-1]}


class LatticeSpec(C.Structure):
    _fields_ = [("kind", C.c_int32), ("radius_mode", C.c_int32),
                ("cells_x", C.c_int32), ("cells_y", C.c_int32), ("cells_z", C.c_int32),
                ("pad_", C.c_int32),
                ("cell_size", C.c_double), ("r0", C.c_double), ("r1", C.c_double),
                ("jitter", C.c_double), ("seed", C.c_uint64)]


class LatticeView(C.Structure):
    _fields_ = [
        ("n_nodes", C.c_int32), ("n_beams", C.c_int32), ("n_connected", C.c_int64),
        ("x0", C.POINTER(C.c_double)), ("r0", C.POINTER(C.c_double)),
        ("layer", C.POINTER(C.c_int32)), ("mass", C.POINTER(C.c_double)),
        ("locked", C.POINTER(C.c_uint8)),
        ("beam_a", C.POINTER(C.c_int32)), ("beam_b", C.POINTER(C.c_int32)),
        ("L0", C.POINTER(C.c_double)), ("radius", C.POINTER(C.c_double)),
        ("area", C.POINTER(C.c_double)), ("I", C.POINTER(C.c_double)),
        ("J", C.POINTER(C.c_double)), ("e0", C.POINTER(C.c_double)),
        ("connected", C.POINTER(C.c_uint64)),
        ("geometry", Geometry),
    ]
