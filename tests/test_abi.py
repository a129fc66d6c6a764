"""The C ABI (include/mcg.h) without a GPU: exported symbols, struct layouts, defaults, the
lattice generators and the error path of context creation."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import ROOT
from falling_dice_gb300 import abi, workloads

HEADER = os.path.join(ROOT, "include", "mcg.h")


def declared_functions(path):
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*[\w\s\*]*?\b(mcg_\w+)\s*\(", text, flags=re.M)))


def test_every_declared_entry_point_is_exported(mcg):
    lib = mcg.load()
    names = declared_functions(HEADER)
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding covers them all
    assert set(names) <= set(mcg.SIGNATURES), set(names) - set(mcg.SIGNATURES)


def test_oracle_libraries_export_the_oracle_api(mco):
    names = [n for n in re.findall(r"\b(orc_\w+)\s*\(", open(os.path.join(ROOT, "oracle", "oracle.h")).read())]
    lib = mco.load("mco")
    assert all(hasattr(lib, n) for n in names)
    assert lib.orc_is_reference() == 0


STRUCTS = {"mcg_config": abi.Config, "mcg_material": abi.Material, "mcg_topology": abi.Topology,
           "mcg_geometry": abi.Geometry, "mcg_diag": abi.Diag, "mcg_optstats": abi.OptStats,
           "mcg_frame": abi.Frame, "mcg_lattice_spec": abi.LatticeSpec,
           "mcg_lattice_view": abi.LatticeView, "mcg_tuning": abi.Tuning}


def test_struct_layouts_match_the_header():
    src = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', 'int main(void) {']
    for cname, ct in STRUCTS.items():
        src.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in ct._fields_:
            cf = "yield" if fname == "yield_" else fname
            src.append(f'printf("{cname}.{fname} %zu\\n", offsetof({cname}, {cf}));')
    src.append("return 0; }")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "layout.c")
        exe = os.path.join(d, "layout")
        open(c, "w").write("\n".join(src))
        subprocess.run(["gcc", "-std=c11", c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    got = dict(line.rsplit(" ", 1) for line in out.strip().splitlines())
    for cname, ct in STRUCTS.items():
        assert int(got[cname]) == C.sizeof(ct), cname
        for fname, _ in ct._fields_:
            assert int(got[f"{cname}.{fname}"]) == getattr(ct, fname).offset, (cname, fname)


def test_config_defaults_are_the_reference_defaults(mcg):
    lib = mcg.load()
    c = abi.Config()
    lib.mcg_config_defaults(C.byref(c))
    d = abi.default_config()
    for name, _ in abi.Config._fields_:
        if name == "material":
            for m, _ in abi.Material._fields_:
                assert getattr(c.material, m) == getattr(d.material, m), m
        else:
            assert getattr(c, name) == getattr(d, name), name
    assert c.seed == 0x494E445553545259 and c.history == 10 and c.max_line_search == 22


def test_create_without_a_device_fails_cleanly(mcg):
    lib = mcg.load()
    h = C.c_void_p()
    cfg = abi.default_config()
    rc = lib.mcg_create(C.byref(cfg), 0, C.byref(h))
    if rc == abi.MCG_OK:
        lib.mcg_destroy(h)
        pytest.skip("a GPU is present")
    assert rc == abi.MCG_ERR_NO_DEVICE and not h.value
    bad = abi.default_config(precision=7)
    assert lib.mcg_create(C.byref(bad), 0, C.byref(h)) == abi.MCG_ERR_INVALID
    assert lib.mcg_status_string(abi.MCG_ERR_EQUILIBRIUM) == b"equilibrium failed"


def test_cubic_generator_counts_and_rules(mcg):
    from falling_dice_gb300 import workloads
    cfg, spec = workloads.cubic6()
    lat = mcg.generate_lattice(spec, cfg)
    assert lat.n_nodes == 343 and lat.n_beams == 3 * 6 * 7 * 7
    # section properties (sim.cpp:115)
    r = lat.radius
    assert np.allclose(lat.area, np.pi * r * r, rtol=0, atol=0)
    assert np.allclose(lat.I, .25 * np.pi * r ** 4, rtol=1e-15)
    assert np.array_equal(lat.J, 2 * lat.I)
    assert 0.3e-3 <= r.min() and r.max() <= 0.6e-3
    # directors and rest lengths from the jittered positions
    x = lat.x0.reshape(-1, 3)
    d = x[lat.beam_b] - x[lat.beam_a]
    assert np.allclose(np.linalg.norm(d, axis=1), lat.L0, rtol=1e-15)
    assert np.allclose(lat.e0.reshape(-1, 3), d / lat.L0[:, None], rtol=1e-14)
    # jitter bounded by 2 % of the cell, faces planar
    grid = np.stack(np.meshgrid(np.arange(7), np.arange(7), np.arange(7), indexing="ij"), -1)
    assert np.abs(x[:, 1] - x[:, 1].round(10)).max() < 1  # sanity
    y = x[:, 1].reshape(7, 7, 7)  # j, k, i
    jr = cfg.joint_scale * cfg.max_radius
    assert np.all(y[0] == jr) and np.allclose(y[6], jr + 6 * 0.005, rtol=0, atol=1e-15)
    assert grid.shape[0] == 7
    # exclusion pairs are the element end pairs; two anti-drift locks (sim.cpp:134)
    keys = (np.minimum(lat.beam_a, lat.beam_b).astype(np.uint64) << np.uint64(32)) | \
        np.maximum(lat.beam_a, lat.beam_b).astype(np.uint64)
    assert np.array_equal(np.sort(keys), lat.connected)
    assert lat.locked.sum() == 3
    # lumped mass: half of every element to each end plus the joint mass (sim.cpp:134)
    m = cfg.material.density * lat.area * lat.L0
    node = np.zeros(lat.n_nodes)
    np.add.at(node, lat.beam_a, .5 * m)
    np.add.at(node, lat.beam_b, .5 * m)
    jm = cfg.material.density * (4.0 / 3.0) * np.pi * jr ** 3 * .28
    assert np.allclose(lat.mass, node + jm, rtol=1e-14)
    assert lat.geometry.top0 == jr + 6 * 0.005 + jr


def test_cubic_bcc_generator_counts(mcg):
    from falling_dice_gb300 import workloads
    cfg, spec = workloads.bcc64()
    lat = mcg.generate_lattice(spec, cfg)
    nx, ny, nz = 64, 64, 32
    corners = (nx + 1) * (ny + 1) * (nz + 1)
    centres = nx * ny * nz
    edges = nx * (ny + 1) * (nz + 1) + (nx + 1) * ny * (nz + 1) + (nx + 1) * (ny + 1) * nz
    assert lat.n_nodes == corners + centres == 270497
    assert lat.n_beams == edges + 8 * centres == 1458336
    assert 0.3e-3 <= lat.radius.min() and lat.radius.max() <= 0.6e-3


def test_generator_rejects_bad_specs(mcg):
    from falling_dice_gb300 import workloads
    cfg, spec = workloads.cubic6()
    spec.cells_x = 0
    lib = mcg.load()
    h = C.c_void_p()
    assert lib.mcg_lattice_generate(C.byref(spec), C.byref(cfg), C.byref(h)) == abi.MCG_ERR_INVALID


def test_random_state_is_seeded_and_respects_locks(mcg):
    from falling_dice_gb300 import workloads
    cfg, spec = workloads.cubic6()
    lat = mcg.generate_lattice(spec, cfg)
    z1, p1 = mcg.random_state(lat, 0.05, 0.1, 0.02, 11)
    z2, p2 = mcg.random_state(lat, 0.05, 0.1, 0.02, 11)
    assert np.array_equal(z1, z2) and np.array_equal(p1, p2)
    assert not np.any(z1[lat.locked.astype(bool)])
    pl = p1.reshape(-1, 7)
    assert np.all((pl[:, 0] >= 0) & (pl[:, 0] <= 0.02)) and np.array_equal(pl[:, 0], pl[:, 1])
    assert abs(np.std(z1[0::6]) - 0.05) < 0.01


def test_sweep_workload_follows_its_specification():
    """The batched sweep's 256 lattices: cells per side U{4..16} (cubic blocks), radius graded
    from 0.3 mm with a slope up to 0.1 mm per cell and capped at 0.7 mm, yield U[30, 70] MPa,
    30 % strain in 100 loading increments; the same draw every time."""
    cfg, specs, ys = workloads.sweep()
    assert len(specs) == len(ys) == 256
    assert cfg.load_steps == 100 and cfg.unload_steps == 0 and abs(cfg.max_strain - 0.3) < 1e-12
    cells = [s.cells_x for s in specs]
    assert all(s.cells_x == s.cells_y == s.cells_z for s in specs)
    assert min(cells) >= 4 and max(cells) <= 16 and len(set(cells)) >= 10
    for s in specs:
        assert s.kind == abi.MCG_LATTICE_CUBIC_BCC
        assert abs(s.r0 - 0.3e-3) < 1e-15 and 0.3e-3 <= s.r1 <= 0.7e-3 + 1e-15
        assert s.r1 - s.r0 <= 0.1e-3 * s.cells_x + 1e-15
    assert all(30e6 <= y <= 70e6 for y in ys)
    cfg2, specs2, ys2 = workloads.sweep()
    assert ys2 == ys and [s.seed for s in specs2] == [s.seed for s in specs]


def test_run_outputs_match_the_reference_writers_byte_for_byte(mcg, tmp_path):
    """mcg_write_metrics_csv / mcg_write_summary_json on the reference's own 20/14 run frames
    (tests/golden/ref242.npz) write exactly the files the reference CLI's writeMetrics and
    writeSummary (MC/src/main.cpp:112-155) wrote for them (tests/golden/ref242_metrics.csv,
    ref242_summary.json, made by tests/golden/make_golden.py --outputs)."""
    from conftest import GOLDEN, golden
    g = golden("ref242")
    frames = g.frames()
    for f in frames:
        for k in abi.FRAME_INTS:
            if k in f:
                f[k] = int(f[k])
    csv = tmp_path / "metrics.csv"
    js = tmp_path / "summary.json"
    mcg.write_metrics_csv(frames, str(csv))
    mcg.write_summary_json(frames, g.cfg, float(g.d["lat_geometry"][4]), str(js))
    assert csv.read_bytes() == open(os.path.join(GOLDEN, "ref242_metrics.csv"), "rb").read()
    assert js.read_bytes() == open(os.path.join(GOLDEN, "ref242_summary.json"), "rb").read()
    with pytest.raises(mcg.MCGError):
        mcg.write_metrics_csv(frames, str(tmp_path / "no" / "such" / "dir.csv"))


def reference_spec():
    s = abi.LatticeSpec()
    s.kind = abi.MCG_LATTICE_REFERENCE_BCC
    return s


def same_arrays(a, b):
    return all(getattr(a, f).shape == getattr(b, f).shape and
               np.array_equal(getattr(a, f).view(np.uint8), getattr(b, f).view(np.uint8)) for f in a.FIELDS)


def test_reference_builder_reproduces_the_reference_specimen(mcg):
    """MCG_LATTICE_REFERENCE_BCC builds the reference's own 2x4x2 specimen
    (Simulator::build, MC/src/sim.cpp:51-134) bit for bit: the arrays of tests/golden/ref242.npz
    were exported from the reference's own Simulator."""
    from conftest import golden
    g = golden("ref242")
    lat = mcg.generate_lattice(reference_spec(), g.cfg)
    assert same_arrays(lat, g.lattice)
    for n, _ in abi.Geometry._fields_:
        assert getattr(lat.geometry, n) == getattr(g.lattice.geometry, n), n


@pytest.mark.parametrize("cells,elements", [((3, 4, 3), 3), ((5, 6, 4), 2), ((4, 4, 4), 5), ((6, 3, 2), 4)])
def test_reference_builder_matches_the_reference_live(mcg, ref_oracle, cells, elements):
    """Against the reference's builder compiled here, over cell counts and 2-5 elements per
    strut (3x4x3 with 3 elements is the reference's own ctest specimen: 788 nodes, 1008
    beams)."""
    cfg = abi.default_config(cells_x=cells[0], cells_y=cells[1], cells_z=cells[2], elements_per_strut=elements)
    cfg.translation_scale = cfg.cell_size
    lat = mcg.generate_lattice(reference_spec(), cfg)
    assert same_arrays(lat, ref_oracle.Model("ref", cfg).export())
    if cells == (3, 4, 3):
        assert (lat.n_nodes, lat.n_beams) == (788, 1008)
