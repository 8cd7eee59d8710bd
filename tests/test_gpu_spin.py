"""Spin tracking (needs a GB300): IntegrateSpin's Bloch integration (LOOP D,
src/tracking.cpp:373-483; SpinDerivs/SpinPrecessionAxis, src/particle.cpp:
141-193) on the GPU against the oracle, in the adjoint-spin configuration's
setting: B0 = 1 uT along z, E = 1e6 V/m along z, specular walls, spins
starting along x, spin integration on (spintimes 0 100, Bmax 1 T).

Tolerances: trajectories are bit-identical (FP64 field mode, same arithmetic
as the oracle, and a uniform table has no gradient force); spin end states
agree to 1e-9 (the table's B differs by rounding between the device's
Hermite form and the oracle's Lekien-Marsden form, so the 1e-12-tolerance
spin steps do not agree bit for bit); the accumulated phase equals
|gamma_n| B0 t to 1e-6
relative (the v x E and Thomas terms are below 1e-4 of it here) and S_z stays
below 1e-3 (the axis tilt by v x E / c^2)."""
import numpy as np
import pytest

from pentrack_gb300 import _abi as A

pytestmark = pytest.mark.gpu


def spin_setup(n=64, simtime=0.2):
    from pentrack_gb300 import Scene, scenes, workloads
    sc = Scene()
    sc.add_material("wall", 335.0)
    sc.add_material("vacuum", 0.0)
    sc.add_solid(1, "wall")
    sc.add_solid(2, "vacuum", scenes.cylinder_mesh(0.2, -0.06, 0.06, 128))
    ax = (np.linspace(-0.25, 0.25, 6), np.linspace(-0.25, 0.25, 6), np.linspace(-0.1, 0.1, 5))
    shape = (6, 6, 5)
    sc.add_table3d(*ax, np.zeros(shape), np.zeros(shape), np.full(shape, 1e-6))
    sc.add_uniform_e(0.0, 0.0, 1e6)
    ids = np.arange(n, dtype=np.int64)
    pos, (E, ph, th, pol) = scenes.source_cylinder(1004, ids, 0.0, 0.19, -0.05, 0.05, 0.0, 200e-9, polarization=1.0)
    parts = scenes.make_particles(1004, ids, pos, E, ph, th, pol)
    parts.spin[:] = 0.0
    parts.spin[0] = 1.0  # spins along x (the configuration's override of the random azimuth)
    params = workloads.run_params(A.NEUTRON, simtime=simtime, tau=0.0, tmax=9e99, lmax=9e99, bmax=1.0,
                                  spintimes=(0.0, 100.0), seed=1004)
    return sc, params, parts


@pytest.mark.parametrize("mode", [A.MODE_PLAIN, A.MODE_BATCHED])
def test_spin_precession_matches_oracle(built, oracle_mod, mode):
    from pentrack_gb300 import Engine, scenes
    sc, params, parts = spin_setup()
    oout, ost = oracle_mod.Oracle(sc).integrate(params, parts)
    params.mode = mode
    gout, gst = Engine(sc).integrate(params, parts)
    assert ost["spin_steps"] > 1000 and abs(gst["spin_steps"] - ost["spin_steps"]) <= 1e-3 * ost["spin_steps"]
    assert np.array_equal(gout.y, oout.y) and np.array_equal(gout.t, oout.t)
    assert np.all(gout.stop_id == A.ID_NOT_FINISH)
    assert np.max(np.abs(gout.spin - oout.spin)) < 1e-9
    # precession about z at |gamma_n| B0: phase and the rotated transverse spin
    t = gout.t - parts.t
    w = abs(scenes.GAMMA_N) * 1e-6
    np.testing.assert_allclose(gout.spin[4], w * t, rtol=1e-6)
    np.testing.assert_allclose(gout.spin[3], t, rtol=1e-12)
    np.testing.assert_allclose(np.sqrt((gout.spin[:3] ** 2).sum(0)), 1.0, atol=1e-8)
    np.testing.assert_allclose(gout.spin[2], 0.0, atol=1e-3)  # tilt of the axis by v x E / c^2 ~ 1e-4


def test_interpolated_axis_matches_oracle(built, oracle_mod):
    """interpolatefields 1 (src/tracking.cpp:404-421): the precession axis
    from cubic splines through 11 values per trajectory step; GPU against the
    oracle with the same criteria, and against the exact axis within the
    interpolation error"""
    from pentrack_gb300 import Engine
    sc, params, parts = spin_setup(n=32)
    exact, _ = Engine(sc).integrate(params, parts)
    params.interpolatefields = 1
    oout, ost = oracle_mod.Oracle(sc).integrate(params, parts)
    gout, gst = Engine(sc).integrate(params, parts)
    assert ost["spin_steps"] > 500 and abs(gst["spin_steps"] - ost["spin_steps"]) <= 1e-3 * ost["spin_steps"]
    assert np.array_equal(gout.y, oout.y) and np.array_equal(gout.t, oout.t)
    assert np.max(np.abs(gout.spin - oout.spin)) < 1e-9
    assert np.max(np.abs(gout.spin[:3] - exact.spin[:3])) < 1e-6
    assert np.max(np.abs(gout.spin[4] - exact.spin[4])) < 1e-6 * np.max(exact.spin[4])
