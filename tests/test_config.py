"""The config.in front end (pt_config_load / pt_config_run_params): a config
in the reference's format, with binary STL files and an OPERA3D table beside
it, yields the same scene descriptor as the same scene built directly, and
the reference's parsing rules hold (comments, map order of keys, ambiguous
keys, materials_file, ignore times, constant [FORMULAS] scales, 3Dtable
units).  The last test tracks both scenes on the GPU."""
import numpy as np
import pytest

from pentrack_gb300 import _abi as A


CONFIG = """################ test config ###############
[GLOBAL]
simtime 2.5   # seconds
materials_file materials.in

[GEOMETRY]
#ID STLfile material ignore_times
1   ignored      default
2   cylinder.STL vacuum
10  block.STL    wall      0.5-1.0 2e-3-3e-3

[FIELDS]
1 OPERA3D table.tab  bramp  1  0  1
2 EDMStaticEField 0 0 1e5 escale

[FORMULAS]
bramp 0.75
escale 2

[PARTICLES]
tau 880
tmax 9e99
lmax 9e99
spintimes 0 1 2 3

[neutron]
tau 700
Bmax 0.1
"""

MATERIALS = """[MATERIALS]
#name FermiReal FermiImag Lambert Spinflip RMS CorrL Bint ModLambert Loss
default 250 0 0.05 0 0 0 0 0 1e-4
vacuum  0 0 0 0 0 0
wall    183 0.0852 0.1 1e-5 0 0 0 0 0
unused  54 0.003 0 1e-5 2.6e-9 20e-9 0 0 0
"""


def _write_case(d):
    from pentrack_gb300 import scenes, workloads
    (d / "config.in").write_text(CONFIG)
    (d / "materials.in").write_text(MATERIALS)
    cyl = scenes.cylinder_mesh(0.2, -0.05, 0.05, 64)
    blk = scenes.box_mesh((-0.05, -0.05, -0.02), (0.05, 0.05, 0.02))
    scenes.write_stl(d / "cylinder.STL", cyl)
    scenes.write_stl(d / "block.STL", blk)
    ax, comps = workloads.quadrupole_table(12)
    scenes.write_opera3d(d / "table.tab", ax, {"BX": comps[0], "BY": comps[1], "BZ": comps[2]})
    return cyl, blk, ax, comps


def _arr(ptr, n, dtype=np.float64):
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype).copy() if n else np.zeros(0, dtype)


def test_config_scene_matches_direct_construction(built, tmp_path):
    from pentrack_gb300 import ConfigScene, scenes
    cyl, blk, ax, comps = _write_case(tmp_path)
    cs = ConfigScene(tmp_path / "config.in")
    d, _ = cs.desc()
    # triangles: both STL files (map order of IDs "10" < "2"), float32 precision
    assert d.n_triangles == len(cyl) + len(blk)
    tris = _arr(d.triangles, 9 * d.n_triangles).reshape(-1, 9)
    sid = _arr(d.triangle_solid, d.n_triangles, np.int32)
    np.testing.assert_array_equal(tris, np.vstack([scenes.read_stl(tmp_path / "block.STL"), scenes.read_stl(tmp_path / "cylinder.STL")]))
    # solids: default first; block (ID 10) before cylinder (ID 2) in map order
    ids = [d.solids[k].id for k in range(d.n_solids)]
    assert ids == [1, 10, 2]
    assert np.all(sid[:len(blk)] == 1) and np.all(sid[len(blk):] == 2)
    blk_solid = d.solids[1]
    assert blk_solid.n_ignore == 2
    np.testing.assert_array_equal(_arr(blk_solid.ignore_times, 4), [0.5, 1.0, 2e-3, 3e-3])
    # materials: only the used ones, columns in order, defaults for missing ones
    mats = {k: d.materials[d.solids[k].material] for k in range(d.n_solids)}
    assert mats[0].fermi_real == 250 and mats[0].diff_prob == 0.05 and mats[0].loss_per_bounce == 1e-4
    assert mats[2].fermi_real == 0 and mats[2].loss_per_bounce == 0
    assert mats[1].fermi_imag == 0.0852 and mats[1].spinflip_prob == 1e-5
    assert d.n_materials == 3  # 'unused' (with micro-roughness) is not carried
    # fields: table with the [FORMULAS] scale and the table's extent as its box
    assert d.n_fields == 2
    f = d.fields[0]
    assert f.type == A.FIELD_TAB3D and f.b_scale == 0.75 and f.e_scale == 1.0 and f.boundary_width == 0
    assert (f.nx, f.ny, f.nz) == tuple(len(a) for a in ax)
    for k, a in enumerate(ax):
        np.testing.assert_allclose(_arr((f.x, f.y, f.z)[k], len(a)), a, rtol=0, atol=1e-15)
    np.testing.assert_allclose(_arr(f.bx, f.nx * f.ny * f.nz), comps[0].ravel(), rtol=0, atol=1e-15)
    assert (f.xmax, f.xmin) == (ax[0][-1], ax[0][0])
    e = d.fields[1]
    assert e.type == A.FIELD_UNIFORM_E and e.e_scale == 2.0 and e.b_scale == 0 and tuple(e.e) == (0, 0, 1e5)


def test_config_run_params_species_overrides(built, tmp_path):
    from pentrack_gb300 import config_run_params
    _write_case(tmp_path)
    p = config_run_params(tmp_path / "config.in", "neutron")
    assert p.species == A.NEUTRON and p.simtime == 2.5 and p.tau == 700 and p.bmax == 0.1
    assert p.n_spintimes == 4 and [p.spintimes[k] for k in range(4)] == [0, 1, 2, 3]
    q = config_run_params(tmp_path / "config.in", "proton")
    assert q.species == A.PROTON and q.tau == 880 and q.bmax == 0


def test_config_errors(built, tmp_path):
    from pentrack_gb300 import ConfigScene
    from pentrack_gb300.engine import EngineError
    _write_case(tmp_path)
    bad = tmp_path / "bad.in"
    bad.write_text(CONFIG.replace("2 EDMStaticEField 0 0 1e5 escale", "2 Conductor 1 0 0 0 0 0 1 1"))
    with pytest.raises(EngineError, match="Conductor") as ex:
        ConfigScene(bad)
    assert ex.value.status == A.PT_ERR_UNSUPPORTED
    bad.write_text(CONFIG.replace("bramp 0.75", "bramp 0.75*t"))
    with pytest.raises(EngineError, match="time-dependent") as ex:
        ConfigScene(bad)
    bad.write_text(CONFIG.replace("10  block.STL", "2  block.STL"))
    with pytest.raises(EngineError, match="ambiguous"):
        ConfigScene(bad)
    bad.write_text(CONFIG.replace("block.STL    wall", "missing.STL  wall"))
    with pytest.raises(EngineError) as ex:
        ConfigScene(bad)
    assert ex.value.status == A.PT_ERR_IO
    bad.write_text(CONFIG.replace("block.STL    wall", "block.STL    nosuch"))
    with pytest.raises(EngineError, match="not defined"):
        ConfigScene(bad)
    # at most one diffuse-reflection model per material (src/geometry.cpp:40-47)
    (tmp_path / "materials.in").write_text(MATERIALS.replace("wall    183 0.0852 0.1 1e-5 0 0 0 0 0",
                                                            "wall    183 0.0852 0.1 1e-5 0 0 0 0.2 0"))
    with pytest.raises(EngineError, match="more than one diffuse-reflection model") as ex:
        ConfigScene(tmp_path / "config.in")
    assert ex.value.status == A.PT_ERR_INVALID
    (tmp_path / "materials.in").write_text(MATERIALS.replace("wall    183 0.0852 0.1 1e-5 0 0 0 0 0",
                                                            "wall    183 0.0852 0.1 1e-5 0 0 0 1.5 0"))
    with pytest.raises(EngineError, match="outside range 0..1"):
        ConfigScene(tmp_path / "config.in")


@pytest.mark.parametrize("change,status,match", [
    ({"diff_prob": 0.1, "modified_lambert_prob": 0.2}, A.PT_ERR_INVALID, "more than one diffuse-reflection model"),
    ({"diff_prob": 0.1, "rms_roughness": 1e-9}, A.PT_ERR_INVALID, "more than one diffuse-reflection model"),
    ({"modified_lambert_prob": 1.5}, A.PT_ERR_INVALID, "outside 0..1"),
    ({"modified_lambert_prob": -0.1}, A.PT_ERR_INVALID, "outside 0..1"),
    ({"rms_roughness": -1e-9, "correl_length": 2e-8}, A.PT_ERR_INVALID, "negative roughness"),
])
def test_pt_create_rejects_invalid_materials(built, change, status, match):
    """pt_create checks the materials on the host before it looks for a
    device, so these rejections hold with or without a GPU."""
    from pentrack_gb300 import Engine, Scene, scenes
    from pentrack_gb300.engine import EngineError
    cols = {"fermi_real": 250.0, "fermi_imag": 0.0, "diff_prob": 0.0, "spinflip_prob": 0.0, "rms_roughness": 0.0,
            "correl_length": 0.0, "internal_bfield": 0.0, "modified_lambert_prob": 0.0, "loss_per_bounce": 0.0}
    cols.update(change)
    sc = Scene()
    sc.add_material("wall", *cols.values())
    sc.add_material("vacuum", 0.0)
    sc.add_solid(1, "wall")
    sc.add_solid(2, "vacuum", scenes.box_mesh((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5)))
    with pytest.raises(EngineError, match=match) as ex:
        Engine(sc)
    assert ex.value.status == status


def test_3dtable_units(built, tmp_path):
    """3Dtable: centimetres and gauss (src/field_3d.cpp:193-198)."""
    from pentrack_gb300 import ConfigScene
    _write_case(tmp_path)
    cfg = tmp_path / "t.in"
    cfg.write_text(CONFIG.replace("1 OPERA3D table.tab  bramp  1  0  1", "1 3Dtable table.tab  1  1  0"))
    cs = ConfigScene(cfg)
    d, _ = cs.desc()
    f = d.fields[0]
    assert abs(f.b_scale - 1e-4) < 1e-18 and f.e_scale == 100
    from pentrack_gb300 import workloads
    ax, _ = workloads.quadrupole_table(12)
    np.testing.assert_allclose(_arr(f.x, f.nx), ax[0] * 0.01, rtol=1e-15)


def test_comsol_table(built, tmp_path, oracle_mod):
    """COMSOL (ReadComsolField, src/field_3d.cpp:124-183): a text export of
    x y z Bx By Bz with '%' headers and space, tab or comma separators, in
    any point order, read by the config front end and by scenes.read_comsol
    into the same TabField3 (B scale, boundary width, coordinate scale; box =
    the data's extent) -- the same field at random points."""
    from pentrack_gb300 import ConfigScene, Scene, scenes, workloads
    ax, comps = workloads.quadrupole_table(8)
    X, Y, Z = np.meshgrid(*ax, indexing="ij")
    rows = np.column_stack([X.ravel() * 100, Y.ravel() * 100, Z.ravel() * 100] + [c.ravel() for c in comps[:3]])
    rows = rows[np.random.default_rng(3).permutation(len(rows))]
    seps = [" ", "\t", ", "]
    lines = ["% Model: synthetic", "% x y z VectorX VectorY VectorZ"]
    lines += [seps[i % 3].join(f"{v:.17g}" for v in r) for i, r in enumerate(rows)]
    (tmp_path / "comsol.txt").write_text("\n".join(lines) + "\n")
    (tmp_path / "config.in").write_text("[GLOBAL]\nsimtime 1\n\n[MATERIALS]\ndefault 0 0 0 0 0 0 0 0 0\n\n"
                                        "[GEOMETRY]\n1 ignored default\n\n[FIELDS]\n1 COMSOL comsol.txt 2 0.01 0.01\n")
    cs = ConfigScene(tmp_path / "config.in")
    axes, c = scenes.read_comsol(tmp_path / "comsol.txt", 0.01)
    for a, b in zip(axes, ax):
        np.testing.assert_allclose(a, b, rtol=1e-15, atol=1e-17)
    sc = Scene()
    sc.add_material("default", 0.0)
    sc.add_solid(1, "default")
    sc.add_table3d(*axes, c["BX"], c["BY"], c["BZ"], b_scale=2.0, e_scale=0.0, boundary_width=0.01)
    rng = np.random.default_rng(4)
    lo, hi = [a[0] for a in axes], [a[-1] for a in axes]
    q = np.column_stack([rng.uniform(lo[k] - 0.01, hi[k] + 0.01, 400) for k in range(3)] + [np.zeros(400)])
    a = oracle_mod.Oracle(cs).field(q)
    b = oracle_mod.Oracle(sc).field(q)
    for u, v in zip(a, b):
        np.testing.assert_array_equal(u, v)
    assert np.abs(a[0]).max() > 0


@pytest.mark.gpu
def test_config_scene_tracks_like_direct_scene(built, tmp_path):
    from pentrack_gb300 import ConfigScene, Engine, Scene, config_run_params, scenes
    cyl, blk, ax, comps = _write_case(tmp_path)
    cs = ConfigScene(tmp_path / "config.in")
    p = config_run_params(tmp_path / "config.in", "neutron")
    # no spin tracking here: with Bmax 0.1 T the Bloch integration would
    # resolve Larmor periods of ~1 ns near the axis for the whole run
    p.bmax = 0.0
    sc = Scene()
    sc.add_material("default", 250.0, 0.0, 0.05, 0.0, 0.0, 0.0, 0.0, 0.0, 1e-4)
    sc.add_material("wall", 183.0, 0.0852, 0.1, 1e-5, 0.0, 0.0, 0.0, 0.0, 0.0)
    sc.add_material("vacuum", 0.0)
    sc.add_solid(1, "default")
    sc.add_solid(10, "wall", scenes.read_stl(tmp_path / "block.STL"), ignore=[(0.5, 1.0), (2e-3, 3e-3)])
    sc.add_solid(2, "vacuum", scenes.read_stl(tmp_path / "cylinder.STL"))
    sc.add_table3d(*ax, *comps, b_scale=0.75, box=(ax[0][-1], ax[0][0], ax[1][-1], ax[1][0], ax[2][-1], ax[2][0]))
    sc.add_uniform_e(0, 0, 1e5, e_scale=2.0)
    ids = np.arange(500, dtype=np.int64)
    pos, (E, ph, th, pol) = scenes.source_cylinder(7, ids, 0.06, 0.19, -0.04, 0.04, 0.0, 200e-9, polarization=0.0)
    parts = scenes.make_particles(7, ids, pos, E, ph, th, pol)
    o1, s1 = Engine(cs).integrate(p, parts)
    o2, s2 = Engine(sc).integrate(p, parts)
    for k in ("t", "y", "stop_id", "n_hit"):
        assert np.array_equal(getattr(o1, k), getattr(o2, k)), k
