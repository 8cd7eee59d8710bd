"""2D (OPERA2D / 2Dtable) field tables on the CPU: TabField (src/field_2d.cpp)
in the oracle pinned against the reference's own ALGLIB, the table readers,
and the reference's field tests as known answers.

* spline2dbuildbicubicv + spline2ddiff / spline2dcalc: golden vectors from
  the reference's vendored ALGLIB 3.15.0 (tests/golden/alglib_spline2d.npz,
  made by tests/golden/gen_golden.py) on uniform and random grids, at random
  points and at the nodes, compared with the oracle's TabField bit for bit.
* The readers: the Python reader and the library's config front end read
  the same tables; the reference's two 2D test tables
  (tests/golden/opera2d_tables.npz) round-trip through the writer.
* test/2DFieldTest: the cosine table (B_z = cos(pi r) + cos(pi z) in units
  of 1e-4 T, V = 1e4 (cos(pi r) + cos(pi z)) V) against the analytic field
  inside the grid, the linear table (B_z = 0.5 T/m z) to rounding.
"""
import os

import numpy as np
import pytest

from pentrack_gb300 import _abi as A

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def table_scene(r, z, **cols):
    from pentrack_gb300.engine import Scene
    sc = Scene()
    sc.add_material("default", 0.0)
    sc.add_solid(1, "default")
    sc.add_table2d(r, z, **cols)
    return sc


def test_oracle_tabfield_matches_alglib_bitwise(oracle_mod):
    g = np.load(os.path.join(GOLD, "alglib_spline2d.npz"))
    for k in range(int(g["n_cases"])):
        x, y, F, px, py, out = (g[f"{a}{k}"] for a in ("x", "y", "f", "px", "py", "out"))
        o = oracle_mod.Oracle(table_scene(x, y, bz=F))
        q = np.column_stack([px, np.zeros_like(px), py, np.zeros_like(px)])
        # TabField's range: x0 <= r < x0 + (x1 - x0)(m - 1), likewise in z
        # (src/field_2d.cpp:291); the random grids' node points can lie beyond it
        inside = (px >= x[0]) & (px < x[0] + (x[1] - x[0]) * (len(x) - 1)) & (py >= y[0]) & \
                 (py < y[0] + (y[1] - y[0]) * (len(y) - 1))
        B, dB, _, _ = o.field(q)
        assert np.array_equal(B[inside, 2], out[inside, 0]), f"case {k}: spline2ddiff value"
        assert np.array_equal(dB[inside, 2, 0], out[inside, 1]), f"case {k}: d/dr"
        assert np.array_equal(dB[inside, 2, 2], out[inside, 2]), f"case {k}: d/dz"
        assert np.all(B[~inside] == 0) and np.all(dB[~inside] == 0)
        Bv, _, _, _ = o.field(q, grad=False)
        assert np.array_equal(Bv[inside, 2], out[inside, 4]), f"case {k}: spline2dcalc value"
        assert inside.sum() >= 64


def test_opera2d_reader_round_trip(tmp_path):
    from pentrack_gb300 import scenes as S
    g = np.load(os.path.join(GOLD, "opera2d_tables.npz"))
    for key in ("linear", "cosine"):
        r, z = g[f"{key}_r"], g[f"{key}_z"]
        cols = {c: g[f"{key}_{c}"] for c in ("BR", "BZ", "V")}
        p = tmp_path / f"{key}.tab"
        S.write_opera2d(str(p), r, z, cols, lengthunit=0.01)
        (r2, z2), c2 = S.read_opera2d(str(p), 0.01)
        np.testing.assert_allclose(r2, r, rtol=1e-15, atol=1e-17)
        np.testing.assert_allclose(z2, z, rtol=1e-15, atol=1e-17)
        assert sorted(c2) == sorted(cols)
        for c in cols:
            np.testing.assert_array_equal(c2[c], cols[c])


CONFIG = """[GLOBAL]
simtype 1
simtime 1

[MATERIALS]
default 0 0 0 0 0 0 0 0 0

[GEOMETRY]
1 ignored default

[FIELDS]
1 OPERA2D cosine.tab 0.0001 1 0.01
2 2Dtable linear.tab 1 1
"""


def test_config_front_end_reads_opera2d_like_python(tmp_path, oracle_mod):
    """[FIELDS] OPERA2D (lengthconv given) and the deprecated 2Dtable
    (centimetres, gauss, V/cm: B x 1e-4, E x 100; ReadOperaField2,
    src/field_2d.cpp:37-66) through pt_config_load equal the Python scene."""
    from pentrack_gb300 import scenes as S
    from pentrack_gb300.engine import ConfigScene
    g = np.load(os.path.join(GOLD, "opera2d_tables.npz"))
    for key in ("linear", "cosine"):
        S.write_opera2d(str(tmp_path / f"{key}.tab"), g[f"{key}_r"], g[f"{key}_z"],
                        {c: g[f"{key}_{c}"] for c in ("BR", "BZ", "V")}, lengthunit=0.01)
    cfg = tmp_path / "config.in"
    cfg.write_text(CONFIG)
    cs = ConfigScene(cfg)
    d, _ = cs.desc()
    assert d.n_fields == 2 and d.fields[0].type == A.FIELD_TAB2D and d.fields[1].type == A.FIELD_TAB2D
    assert d.fields[1].b_scale == 1e-4 and d.fields[1].e_scale == 100.0
    sc = table_scene(g["cosine_r"], g["cosine_z"], br=g["cosine_BR"], bz=g["cosine_BZ"], v=g["cosine_V"],
                     b_scale=1e-4, e_scale=1.0)
    sc.add_table2d(g["linear_r"], g["linear_z"], br=g["linear_BR"], bz=g["linear_BZ"], v=g["linear_V"],
                   b_scale=1e-4, e_scale=100.0)
    rng = np.random.default_rng(5)
    q = np.column_stack([rng.uniform(-0.7, 0.7, (500, 2)), rng.uniform(-0.1, 1.1, 500), np.zeros(500)])
    a = oracle_mod.Oracle(cs).field(q)
    b = oracle_mod.Oracle(sc).field(q)
    for u, v in zip(a, b):
        np.testing.assert_array_equal(u, v)


def test_2d_field_test_known_answers(oracle_mod):
    """test/2DFieldTest: the bicubic cosine field against cos(pi r) + cos(pi z)
    away from the grid's edges (the reference's README expects the spline's
    over/undershoot at the edges); the linear table to rounding."""
    g = np.load(os.path.join(GOLD, "opera2d_tables.npz"))
    sc = table_scene(g["cosine_r"], g["cosine_z"], br=g["cosine_BR"], bz=g["cosine_BZ"], v=g["cosine_V"],
                     b_scale=1e-4, e_scale=1.0)
    o = oracle_mod.Oracle(sc)
    rng = np.random.default_rng(11)
    n = 2000
    r, phi, z = rng.uniform(0.2, 0.8, n), rng.uniform(0, 2 * np.pi, n), rng.uniform(0.2, 0.8, n)
    q = np.column_stack([r * np.cos(phi), r * np.sin(phi), z, np.zeros(n)])
    B, dB, V, E = o.field(q)
    ana = np.cos(np.pi * r) + np.cos(np.pi * z)
    np.testing.assert_allclose(B[:, 2], ana, atol=2e-4)
    np.testing.assert_allclose(np.hypot(B[:, 0], B[:, 1]), 0.0, atol=1e-12)
    np.testing.assert_allclose(V / 1e4, ana, atol=2e-4)
    Eana = np.pi * 1e4 * np.sqrt(np.sin(np.pi * r) ** 2 + np.sin(np.pi * z) ** 2)
    np.testing.assert_allclose(np.linalg.norm(E, axis=1), Eana, rtol=5e-3)
    # the gradient the tracker uses: dBz/dz = -pi sin(pi z), dBz/dx = -pi sin(pi r) x / r
    np.testing.assert_allclose(dB[:, 2, 2], -np.pi * np.sin(np.pi * z), atol=5e-3)
    np.testing.assert_allclose(dB[:, 2, 0], -np.pi * np.sin(np.pi * r) * np.cos(phi), atol=5e-3)
    # outside the grid's range nothing is added
    Bo, _, Vo, _ = o.field(np.array([[0.0, 0.0, 1.0, 0.0], [0.8, 0.8, 0.5, 0.0], [0.3, 0.0, -0.01, 0.0]]))
    assert np.all(Bo == 0) and np.all(Vo == 0)

    lin = table_scene(g["linear_r"], g["linear_z"], br=g["linear_BR"], bz=g["linear_BZ"], b_scale=5e-5, e_scale=0.0)
    B, dB, V, E = oracle_mod.Oracle(lin).field(q)
    np.testing.assert_allclose(B[:, 2], 0.5 * z, rtol=1e-13)
    np.testing.assert_allclose(dB[:, 2, 2], 0.5, rtol=1e-13)
    assert np.all(V == 0) and np.all(E == 0)


def test_cylindrical_conversion_of_a_rotating_field(oracle_mod):
    """B_r and B_phi tables: B = B_r e_r + B_phi e_phi and its Cartesian
    Jacobian (src/field_2d.cpp:300-333) against central differences of B."""
    r = np.linspace(0.0, 1.0, 21)
    z = np.linspace(-0.5, 0.5, 11)
    R, Z = np.meshgrid(r, z, indexing="ij")
    o = oracle_mod.Oracle(table_scene(r, z, br=R * (1 + Z), bphi=R ** 2 - Z, bz=R * R + Z))
    rng = np.random.default_rng(3)
    p = np.column_stack([rng.uniform(-0.6, 0.6, (300, 2)), rng.uniform(-0.4, 0.4, 300)])
    p = p[np.hypot(p[:, 0], p[:, 1]) > 0.05]
    q = np.column_stack([p, np.zeros(len(p))])
    B, dB, _, _ = o.field(q)
    rr = np.hypot(p[:, 0], p[:, 1])
    cp, sp = p[:, 0] / rr, p[:, 1] / rr
    Br, Bphi = rr * (1 + p[:, 2]), rr ** 2 - p[:, 2]
    np.testing.assert_allclose(B[:, 0], Br * cp - Bphi * sp, atol=1e-3)
    np.testing.assert_allclose(B[:, 1], Br * sp + Bphi * cp, atol=1e-3)
    h = 1e-6
    for j in range(3):
        d = np.zeros(4)
        d[j] = h
        fd = (o.field(q + d)[0] - o.field(q - d)[0]) / (2 * h)
        np.testing.assert_allclose(dB[:, :, j], fd, atol=1e-6)


def test_opera2d_all_columns_and_y_column(tmp_path, oracle_mod):
    """A table with the optional " 2 Y [LENGU]" coordinate and every field
    column (RBX, RBY, RBZ, EX, EY, EZ, RV), read by the Python reader and by
    the config front end into the same field; the E map takes precedence
    over the potential (src/field_2d.cpp:262-283), so V is zero"""
    from pentrack_gb300 import scenes as S
    from pentrack_gb300.engine import ConfigScene
    r = np.linspace(0.0, 30.0, 7)
    z = np.linspace(-20.0, 40.0, 9)
    R, Z = np.meshgrid(r, z, indexing="ij")
    cols = {"BR": R * Z * 1e-2, "BPHI": R * R * 1e-3, "BZ": np.cos(R / 10) + Z * 1e-2, "ER": R * 3.0, "EPHI": -R,
            "EZ": Z * 2.0, "V": R + Z}
    tags = [("RBX", "BR"), ("RBY", "BPHI"), ("RBZ", "BZ"), ("EX", "ER"), ("EY", "EPHI"), ("EZ", "EZ"), ("RV", "V")]
    lines = [f"{len(r)} 1 {len(z)} 2", " 1 X [LENGU]", " 2 Y [LENGU]", " 3 Z [LENGU]"]
    lines += [f" {4 + i} {t} [UNIT]" for i, (t, _) in enumerate(tags)]
    lines.append(" 0")
    for i in range(len(r)):
        for j in range(len(z)):
            lines.append(" ".join(f"{v:.17g}" for v in [r[i], 0.0, z[j]] + [cols[c][i, j] for _, c in tags]))
    (tmp_path / "t.tab").write_text("\n".join(lines) + "\n")
    (r2, z2), c2 = S.read_opera2d(str(tmp_path / "t.tab"), 0.01)
    np.testing.assert_allclose(r2, r * 0.01, rtol=1e-15)
    np.testing.assert_allclose(z2, z * 0.01, rtol=1e-15, atol=1e-18)
    for _, c in tags:
        np.testing.assert_array_equal(c2[c], cols[c])
    (tmp_path / "config.in").write_text("[GLOBAL]\nsimtime 1\n\n[MATERIALS]\ndefault 0 0 0 0 0 0 0 0 0\n\n"
                                        "[GEOMETRY]\n1 ignored default\n\n[FIELDS]\n1 OPERA2D t.tab 0.5 2 0.01\n")
    cs = ConfigScene(tmp_path / "config.in")
    sc = table_scene(r2, z2, br=c2["BR"], bphi=c2["BPHI"], bz=c2["BZ"], v=c2["V"], er=c2["ER"], ephi=c2["EPHI"],
                     ez=c2["EZ"], b_scale=0.5, e_scale=2.0)
    rng = np.random.default_rng(8)
    q = np.column_stack([rng.uniform(-0.35, 0.35, (300, 2)), rng.uniform(-0.25, 0.45, 300), np.zeros(300)])
    a, b = oracle_mod.Oracle(cs).field(q), oracle_mod.Oracle(sc).field(q)
    for u, v in zip(a, b):
        np.testing.assert_array_equal(u, v)
    assert np.all(a[2] == 0) and np.abs(a[3]).max() > 0
