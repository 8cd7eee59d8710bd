"""Pins of the CPU oracle against the reference's own code and published vectors.

* ALGLIB spline1dgriddiffcubic and libtricubic tricubic_get_coeff: golden
  vectors produced by the reference's vendored sources (tests/golden/gen_golden.py),
  compared bit for bit.
* Philox4x32-10: the published Random123 known-answer vectors.
* Dormand-Prince 5(4) dense stepper: accuracy on a forced oscillator.
"""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_spline_derivs_match_alglib_bitwise(oracle_mod):
    g = np.load(os.path.join(GOLD, "alglib_spline.npz"))
    for k, n in enumerate(g["n"]):
        a, b = g["offset"][k], g["offset"][k + 1]
        d = oracle_mod.spline_derivs(g["x"][a:b], g["y"][a:b])
        assert np.array_equal(d, g["d"][a:b]), f"case {k} (n={n})"


def test_tricubic_coefficients_match_libtricubic_bitwise(oracle_mod):
    g = np.load(os.path.join(GOLD, "tricubic.npz"))
    for i in range(len(g["x"])):
        a = oracle_mod.tricubic_coeff(g["x"][i])
        assert np.array_equal(a, g["a"][i])


def test_tricubic_horner_matches_libtricubic_eval(oracle_mod):
    """tricubic_eval_fast (src/field_3d.cpp:36-121) vs libtricubic's own evaluator."""
    g = np.load(os.path.join(GOLD, "tricubic.npz"))
    for i in range(len(g["a"])):
        x, y, z = g["pts"][i]
        for j, der in enumerate(((0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1))):
            v = oracle_mod.tricubic_eval(g["a"][i], x, y, z, *der)
            ref = g["eval"][i, j]
            assert abs(v - ref) <= 1e-12 * max(1.0, abs(ref))


@pytest.mark.parametrize("ctr,key,expect", [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
])
def test_philox_known_answers(oracle_mod, ctr, key, expect):
    from pentrack_gb300 import scenes
    assert tuple(oracle_mod.philox(ctr, key)) == expect
    out = scenes.philox4x32_10(*[np.array([c], dtype=np.uint32) for c in ctr], np.uint32(key[0]), np.uint32(key[1]))
    assert tuple(int(o[0]) for o in out) == expect


def test_uniform_stream_host_equals_oracle(oracle_mod):
    from pentrack_gb300 import scenes
    ids = np.array([0, 1, 17, 2**40 + 3], dtype=np.int64)
    for draw in (0, 1, 5, 2**33 + 1):
        u = scenes.uniform(12345, ids, draw)
        for i, pid in enumerate(ids):
            assert u[i] == oracle_mod.lib().pto_uniform(12345, int(pid), draw)
    assert ((u >= 0) & (u < 1)).all()


def test_dopri5_dense_stepper_accuracy(oracle_mod):
    """Forced damped oscillator y'' = -y - 0.1 y' + 0.5 cos 3t against scipy's
    DOP853 at rtol 1e-13: accepted points within the 1e-9 tolerance regime and
    the continuous extension at mid-step of comparable accuracy."""
    from scipy.integrate import solve_ivp
    L = oracle_mod.lib()
    n = 40
    t = np.zeros(2 * n)
    y = np.zeros(4 * n)
    y0 = np.array([1.0, 0.0])
    dp = oracle_mod._dp
    L.pto_dopri5_selftest(0.0, dp(y0), 0.01, n, dp(t), dp(y))
    t, y = t.reshape(n, 2), y.reshape(n, 4)
    f = lambda tt, yy: [yy[1], -yy[0] - 0.1 * yy[1] + 0.5 * np.cos(3 * tt)]  # noqa: E731
    ts = np.concatenate([t[:, 1], 0.5 * (t[:, 0] + t[:, 1])])
    order = np.argsort(ts)
    sol = solve_ivp(f, (0, ts.max()), y0, method="DOP853", rtol=1e-13, atol=1e-14, t_eval=ts[order], dense_output=False)
    ref = np.empty((2 * n, 2))
    ref[order] = sol.y.T
    assert np.max(np.abs(y[:, 0:2] - ref[:n])) < 2e-8
    assert np.max(np.abs(y[:, 2:4] - ref[n:])) < 2e-8
    assert t[-1, 1] > 1.0  # the controller grew the step from 0.01


def test_synthetic_fixtures_replicate_reference_files(oracle_mod):
    """The generated hollow cube, centred cube and 3D gradient table equal the
    reference's test/ fixtures (read as data when the golden file was made):
    same surfaces (identical collisions of random segments, whatever the
    quad diagonals) and the same table."""
    from pentrack_gb300 import Scene, scenes, workloads
    g = np.load(os.path.join(GOLD, "reference_fixtures.npz"))
    rng = np.random.default_rng(5)

    def hits(tris, segs):
        sc = Scene()
        sc.add_material("m", 0.0)
        sc.add_solid(1, 0)
        sc.add_solid(2, 0, tris)
        cnt, s, n, sid, dn = oracle_mod.Oracle(sc).collisions(segs)
        return cnt, np.where(np.arange(8)[None, :] < cnt[:, None], s, 0), np.where(np.arange(8)[None, :] < cnt[:, None], dn, 0)

    for mine, ref, lo, hi in ((workloads.hollow_cube_mesh(), g["hollow"], -0.2, 1.2),
                              (scenes.box_mesh((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5)), g["cube"], -0.8, 0.8)):
        assert len(mine) == len(ref)
        segs = rng.uniform(lo, hi, size=(2000, 6))
        a, b = hits(mine, segs), hits(ref, segs)
        assert np.array_equal(a[0], b[0])
        assert np.allclose(a[1], b[1], rtol=0, atol=1e-12) and np.allclose(a[2], b[2], rtol=0, atol=1e-12)
    sc, _, _ = workloads.integration_test(n=1)
    f = sc.fields[0]
    assert np.allclose(f["x"], g["tab_x"]) and np.allclose(f["z"], g["tab_z"])
    assert np.allclose(f["bz"].reshape(6, 6, 6), g["tab_bz"])
    g2 = np.load(os.path.join(GOLD, "opera2d_tables.npz"))
    sc, _, _ = workloads.integration_test(n=1, full=True)
    f = sc.fields[0]
    assert f["type"] == 5 and np.allclose(f["x"], g2["linear_r"]) and np.allclose(f["z"], g2["linear_z"])
    for k, c in (("bx", "BR"), ("bz", "BZ"), ("v", "V")):
        assert np.allclose(f[k].reshape(11, 11), g2[f"linear_{c}"])


def test_oracle_harmonic_terms_match_reference_closed_forms(oracle_mod):
    """The oracle's harmonic terms (derived symbolically from the expansion's
    definition) against the reference's closed forms for l <= 2
    (src/harmonicfields.cpp:76-288), with offset and scale."""
    from pentrack_gb300 import Scene, scenes
    rng = np.random.default_rng(5)
    coeffs = [(0, -1, 0.3), (0, 0, 1e-6), (0, 1, -0.2), (1, -2, 7.5), (1, -1, 0.4), (1, 0, -1.1), (1, 1, 0.9),
              (1, 2, 0.5), (2, -3, 1.7), (2, -2, -0.6), (2, -1, 0.8), (2, 0, 1.2), (2, 1, -0.3), (2, 2, 0.25), (2, 3, 2.0)]
    sc = Scene()
    sc.add_material("m", 0.0)
    sc.add_solid(1, 0)
    sc.add_solid(2, 0, scenes.box_mesh((-1, -1, -1), (1, 1, 1)))
    off = (0.01, -0.02, 0.03)
    sc.add_harmonic(coeffs, offset=off, b_scale=2.0)
    p = rng.uniform(-0.3, 0.3, (400, 3))
    B, dB, _, _ = oracle_mod.Oracle(sc).field(np.column_stack([p, np.zeros(len(p))]))
    x, y, z = (p[:, k] + off[k] for k in range(3))
    o = 0 * x
    forms = {
        (0, -1): (o, 1 + o, o), (0, 0): (o, o, 1 + o), (0, 1): (1 + o, o, o),
        (1, -2): (y, x, o), (1, -1): (o, z, y), (1, 0): (-x / 2, -y / 2, z), (1, 1): (z, o, x), (1, 2): (x, -y, o),
        (2, -3): (2 * x * y, (x - y) * (x + y), o), (2, -2): (2 * y * z, 2 * x * z, 2 * x * y),
        (2, -1): (-x * y / 2, -x * x / 4 - 3 * y * y / 4 + z * z, 2 * y * z), (2, 0): (-x * z, -y * z, -x * x / 2 - y * y / 2 + z * z),
        (2, 1): (-3 * x * x / 4 - y * y / 4 + z * z, -x * y / 2, 2 * x * z), (2, 2): (2 * x * z, -2 * y * z, (x - y) * (x + y)),
        (2, 3): ((x - y) * (x + y), -2 * x * y, o),
    }
    ref = np.zeros((len(p), 3))
    for l, m, g in coeffs:
        ref += 2.0 * g * np.column_stack(forms[(l, m)])
    assert np.max(np.abs(B - ref)) < 1e-13 * np.abs(ref).max()
    assert np.max(np.abs(np.trace(dB, axis1=1, axis2=2))) < 1e-12
    assert np.max(np.abs(dB - np.transpose(dB, (0, 2, 1)))) < 1e-12


def test_axis_spline_matches_alglib_bitwise(oracle_mod):
    """IntegrateSpin's precession-axis spline (interpolatefields 1):
    spline1dbuildcubic + spline1dcalc of the reference's ALGLIB
    (tests/golden/alglib_spline1d.npz) at random points, the nodes and beyond
    both ends, equal to the oracle's Spline1 bit for bit"""
    g = np.load(os.path.join(GOLD, "alglib_spline1d.npz"))
    for k in range(int(g["n_cases"])):
        v = oracle_mod.spline1d_calc(g[f"x{k}"], g[f"y{k}"], g[f"p{k}"])
        assert np.array_equal(v, g[f"v{k}"]), k
