"""Oracle-level physics checks on the reference's own known answers (CPU).

The reference's test/IntegrationTest is its only analytic known-answer test of
integrator + field + collision path: UCN fly on parabolas with
a = -g - |mu_n| dBz/dz / m_n and the landing x must equal
x0 + vx0 * t(z_end) (test/IntegrationTest/showintegrationresult.cxx:1-7).
It runs with the OPERA3D half only (dBz/dz = 0.5 T/m) and in full, the
OPERA2D and OPERA3D tables together (1 T/m, a = -15.5754762729 m/s^2 as
showintegrationresult.cxx states).
"""
import pytest
import numpy as np

from pentrack_gb300 import _abi as A


def landing_residual(parts, out, a):
    x0, z0, vx0, vz0 = parts.y[0], parts.y[2], parts.y[3], parts.y[5]
    ze = out.y[2]
    t_hit = (-vz0 - np.sqrt(vz0 * vz0 - 2 * a * (z0 - ze))) / a
    return out.y[0] - x0 - vx0 * t_hit


@pytest.mark.parametrize("full", [False, True])
def test_integration_test_known_answer_oracle(oracle_mod, full):
    from pentrack_gb300 import workloads
    sc, params, parts = workloads.integration_test(n=200, full=full)
    orc = oracle_mod.Oracle(sc)
    out, st = orc.integrate(params, parts, nthreads=4)
    a = workloads.integration_test_acceleration(1.0 if full else 0.5)
    assert abs(a - (-15.5754762729 if full else -12.691)) < 1e-3
    # absorbed in the floor on the first wall contact (fast ones reach the ceiling instead)
    first = (out.n_hit == 1) & (out.stop_id == A.ID_ABSORBED_IN_MATERIAL) & (out.y[2] < 0.5)
    assert first.sum() > 100
    res = landing_residual(parts, out, a)[first]
    assert np.max(np.abs(res)) < 1e-6, np.max(np.abs(res))
    # absorbed inside the 1 mm UCNdet floor
    assert np.all(out.y[2][first] < 0) and np.all(out.y[2][first] > -0.001)


def test_cube_storage_energy_conservation_oracle(oracle_mod):
    """Specular total reflection and gravity only: total energy is conserved to
    the integrator tolerance over 5 s of storage."""
    from pentrack_gb300 import workloads
    sc, params, parts = workloads.cube_storage(n=64, simtime=5.0)
    orc = oracle_mod.Oracle(sc)
    out, st = orc.integrate(params, parts, nthreads=4)
    assert np.all(out.stop_id == A.ID_NOT_FINISH)
    assert np.allclose(out.t, 5.0)
    # H = Ekin + m g z + Fermi potential of the current solid (vacuum inside the cube)
    m = 1.0454074345680994e-08
    g = 9.80665
    c2 = 299792458.0 ** 2

    def H(y):
        v2 = (y[3:6] ** 2).sum(0)
        return 0.5 * m * v2 * (1 + 0.75 * v2 / c2) + m * g * y[2]

    dh = np.abs(H(out.y) - H(parts.y))
    assert np.max(dh) < 1e-13, np.max(dh)  # eV, i.e. < 1e-4 neV
    assert np.all(out.n_hit > 0)
    assert np.all(out.solid == 2)


def test_absorption_per_bounce_matches_the_complex_potential_step(oracle_mod):
    """TNeutron::OnHit for total reflection (src/neutron.cpp:219-256): a UCN
    bouncing vertically on a floor with Fermi potential 250 - 20i neV and
    1e-3 loss per bounce is absorbed with probability
    1 - |(k1 - k2)/(k1 + k2)|^2 + loss per hit, k = sqrt(E_normal - U).  The
    number of hits to absorption is geometric: n / sum(hits) estimates it."""
    from pentrack_gb300 import Scene, scenes, workloads
    sc = Scene()
    sc.add_material("floor", 250.0, fermi_imag=20.0, loss_per_bounce=1e-3)
    sc.add_material("vacuum", 0.0)
    sc.add_solid(1, "floor")
    sc.add_solid(2, "vacuum", scenes.box_mesh((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5)))
    n = 3000
    ids = np.arange(n, dtype=np.int64)
    e0 = 30e-9
    pos = np.zeros((3, n))
    pos[0], pos[1] = 0.1, 0.13  # off the box's face diagonals, which a ray from the centre would graze
    parts = scenes.make_particles(1, ids, pos, np.full(n, e0), np.zeros(n), np.full(n, np.pi), np.ones(n))
    params = workloads.run_params(A.NEUTRON, simtime=300.0, tau=0.0, tmax=9e99, lmax=9e99, bmax=0.0,
                                  spintimes=(0, 0), seed=1)
    out, _ = oracle_mod.Oracle(sc).integrate(params, parts)
    assert np.all(out.stop_id == A.ID_ABSORBED_ON_SURFACE)
    v0 = np.sqrt((parts.y[3:6, 0] ** 2).sum())
    en = 0.5 * scenes.M_N * (v0 * v0 + 2 * scenes.GRAV * 0.5)  # normal energy at the floor
    k1 = np.sqrt(complex(en, 0.0))
    k2 = np.sqrt(complex(en - 250e-9, -20e-9))
    p = 1 - abs((k1 - k2) / (k1 + k2)) ** 2 + 1e-3
    p_hat = n / out.n_hit.sum()
    sigma = p * np.sqrt((1 - p) / n)
    assert abs(p_hat - p) < 4 * sigma, (p_hat, p, sigma)


def _floor_drop(oracle_mod, fermi, diff_prob=0.0, n=3000, simtime=0.6, e0=30e-9):
    """UCN falling vertically from (0.1, 0.13, 0) onto the floor of a 1 m box
    whose outside (the default solid) has the given Fermi potential.  A UCN
    leaving the box moves along its outward normal, so the surface properties
    that apply are the box's own (OnHit takes the leaving solid's material
    then, src/neutron.cpp:191): the diffuse probability is set there."""
    from pentrack_gb300 import Scene, scenes, workloads
    sc = Scene()
    sc.add_material("floor", fermi)
    sc.add_material("vacuum", 0.0, diff_prob=diff_prob)
    sc.add_solid(1, "floor")
    sc.add_solid(2, "vacuum", scenes.box_mesh((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5)))
    ids = np.arange(n, dtype=np.int64)
    pos = np.zeros((3, n))
    pos[0], pos[1] = 0.1, 0.13
    parts = scenes.make_particles(2, ids, pos, np.full(n, e0), np.zeros(n), np.full(n, np.pi), np.ones(n))
    params = workloads.run_params(A.NEUTRON, simtime=simtime, tau=0.0, tmax=9e99, lmax=9e99, bmax=0.0,
                                  spintimes=(0, 0), seed=2)
    out, _ = oracle_mod.Oracle(sc).integrate(params, parts)
    v0 = np.sqrt((parts.y[3:6, 0] ** 2).sum())
    return parts, out, v0 * v0 + 2 * scenes.GRAV * 0.5  # squared speed at the floor


def test_transmission_probability_above_the_potential_step(oracle_mod):
    """Enormal > Estep (src/neutron.cpp:221-240): reflection with probability
    |(k1 - k2)/(k1 + k2)|^2 for real k, otherwise transmission into the floor."""
    from pentrack_gb300 import scenes
    parts, out, vf2 = _floor_drop(oracle_mod, 50.0)
    en = 0.5 * scenes.M_N * vf2
    k1, k2 = np.sqrt(en), np.sqrt(en - 50e-9)
    R = ((k1 - k2) / (k1 + k2)) ** 2
    # transmitted UCN fall through the floor and leave the geometry's bounding
    # box (ID_HIT_BOUNDARIES, CheckSegment); reflected ones are still flying
    refl = (out.stop_id == A.ID_NOT_FINISH).mean()
    assert np.all(out.n_hit == 1) and np.all(np.isin(out.stop_id, (A.ID_NOT_FINISH, A.ID_HIT_BOUNDARIES)))
    assert np.all(out.y[2][out.stop_id == A.ID_NOT_FINISH] > -0.5)
    assert abs(refl - R) < 4 * np.sqrt(R * (1 - R) / parts.n), (refl, R)


def test_lambert_reflection_directions(oracle_mod):
    """DiffProb 1 (ReflectLambert, src/neutron.cpp:150-183): the outgoing
    direction about the normal has density cos(theta) sin(theta), so
    cos^2(theta) is uniform; horizontal velocity is conserved in flight, so
    sin^2(theta) = v_horizontal^2 / v_floor^2 at the end."""
    from scipy import stats
    from pentrack_gb300 import scenes
    v0 = scenes.speed_from_energy(np.array([30e-9]), scenes.M_N)[0]
    t1 = (-v0 + np.sqrt(v0 * v0 + scenes.GRAV)) / scenes.GRAV  # the fall of 0.5 m to the floor
    # stop 1 ms after the bounce: a second floor hit within 1 ms needs cos(theta) < 0.002
    parts, out, vf2 = _floor_drop(oracle_mod, 250.0, diff_prob=1.0, simtime=t1 + 1e-3)
    assert (out.n_hit == 1).mean() > 0.998
    c2 = 1 - (out.y[3] ** 2 + out.y[4] ** 2) / vf2
    assert stats.kstest(c2, "uniform").pvalue > 1e-3


def test_spinflip_per_hit_and_decay_fraction(oracle_mod):
    """SpinflipProb flips the polarisation at a hit with that probability
    (src/neutron.cpp:193-196, counted in Nspinflip); with tau the particle
    decays at an exponentially distributed proper time
    (src/tracking.cpp:19-26, 144-155)."""
    from pentrack_gb300 import Scene, scenes, workloads
    sc = Scene()
    sc.add_material("wall", 335.0)
    sc.add_material("vacuum", 0.0, spinflip_prob=0.3)
    sc.add_solid(1, "wall")
    sc.add_solid(2, "vacuum", scenes.box_mesh((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5)))
    n = 3000
    ids = np.arange(n, dtype=np.int64)
    pos, (E, ph, th, pol) = scenes.source_box(3, ids, (-0.45, -0.45, -0.45), (0.45, 0.45, 0.45), 0.0, 100e-9)
    parts = scenes.make_particles(3, ids, pos, E, ph, th, pol)
    params = workloads.run_params(A.NEUTRON, simtime=5.0, tau=10.0, tmax=9e99, lmax=9e99, bmax=0.0,
                                  spintimes=(0, 0), seed=3)
    out, _ = oracle_mod.Oracle(sc).integrate(params, parts)
    hits = out.n_hit.sum()
    p = out.n_spinflip.sum() / hits
    assert hits > 20000 and abs(p - 0.3) < 4 * np.sqrt(0.3 * 0.7 / hits), p
    dec = (out.stop_id == A.ID_DECAYED).mean()
    q = 1 - np.exp(-5.0 / 10.0)  # proper time = lab time to 1e-16 for UCN
    assert np.all(np.isin(out.stop_id, (A.ID_DECAYED, A.ID_NOT_FINISH)))
    assert abs(dec - q) < 4 * np.sqrt(q * (1 - q) / n), (dec, q)


def test_cyclotron_orbits_close_after_whole_periods(oracle_mod):
    """TParticle::EquationOfMotion's Lorentz force with the relativistic factors
    (src/particle.cpp:105-135): in a uniform 1 T field a 500 eV proton and a
    500 keV electron started perpendicular to B return to their start point
    after whole periods 2 pi gamma m / (q B)."""
    from pentrack_gb300 import Scene, scenes, workloads
    sc = Scene()
    sc.add_material("vacuum", 0.0)
    sc.add_material("detector", 0.0)
    # charged particles fly in the default solid (any other solid absorbs
    # them); two small cubes at opposite corners span the geometry's box
    sc.add_solid(1, "vacuum")
    corners = np.vstack([scenes.box_mesh((-1, -1, -1), (-0.9, -0.9, -0.9)), scenes.box_mesh((0.9, 0.9, 0.9), (1, 1, 1))])
    sc.add_solid(2, "detector", corners)
    sc.add_harmonic([(0, 0, 1.0)])
    for species, E, m in ((A.PROTON, 500.0, scenes.M_P), (A.ELECTRON, 500e3, scenes.M_E)):
        ids = np.arange(4, dtype=np.int64)
        pos = np.tile(np.array([[0.1], [0.13], [0.05]]), (1, 4))
        parts = scenes.make_particles(4, ids, pos, np.full(4, E), np.linspace(0, 1.5, 4), np.full(4, np.pi / 2),
                                      np.ones(4), species=species)
        gamma = 1 + E / (m * scenes.C0 ** 2)
        period = 2 * np.pi * gamma * m / 1.0  # m in eV s^2/m^2, so q B / m in units of e: omega = B / (gamma m)
        params = workloads.run_params(species, simtime=5 * period, tau=0.0, tmax=9e99, lmax=9e99, bmax=0.0,
                                      spintimes=(0, 0), seed=4)
        out, _ = oracle_mod.Oracle(sc).integrate(params, parts)
        assert np.all(out.stop_id == A.ID_NOT_FINISH)
        v = np.sqrt((parts.y[3:6] ** 2).sum(0))
        r = gamma * m * v / 1.0
        assert 1e-3 < r[0] < 1e-2
        dpos = np.sqrt(((out.y[0:3] - parts.y[0:3]) ** 2).sum(0))
        assert np.all(dpos < 1e-5 * r), (species, dpos / r)
        np.testing.assert_allclose(np.sqrt((out.y[3:6] ** 2).sum(0)), v, rtol=1e-7)


def test_exb_drift_is_a_straight_line(oracle_mod):
    """The Lorentz force with a uniform E (EDMStaticEField) and B: a proton
    moving at the drift velocity E x B / B^2 feels no net force and keeps its
    velocity (src/particle.cpp:105-135)."""
    from pentrack_gb300 import Scene, scenes, workloads
    sc = Scene()
    sc.add_material("vacuum", 0.0)
    sc.add_material("detector", 0.0)
    sc.add_solid(1, "vacuum")
    corners = np.vstack([scenes.box_mesh((-1, -1, -1), (-0.9, -0.9, -0.9)), scenes.box_mesh((0.9, 0.9, 0.9), (1, 1, 1))])
    sc.add_solid(2, "detector", corners)
    sc.add_harmonic([(0, 0, 1.0)])
    sc.add_uniform_e(1e4, 0.0, 0.0)
    n = 3
    pos = np.tile(np.array([[0.1], [0.13], [0.05]]), (1, n))
    parts = scenes.make_particles(5, np.arange(n, dtype=np.int64), pos, np.full(n, 1.0), np.zeros(n),
                                  np.full(n, np.pi / 2), np.ones(n), species=A.PROTON)
    parts.y[3:6] = np.array([[0.0], [-1e4], [0.0]])
    params = workloads.run_params(A.PROTON, simtime=1e-6, tau=0.0, tmax=9e99, lmax=9e99, bmax=0.0,
                                  spintimes=(0, 0), seed=5)
    out, _ = oracle_mod.Oracle(sc).integrate(params, parts)
    assert np.all(out.stop_id == A.ID_NOT_FINISH)
    dt = out.t - parts.t
    np.testing.assert_allclose(out.y[1], parts.y[1] - 1e4 * dt, rtol=0, atol=1e-9)
    np.testing.assert_allclose(out.y[0], parts.y[0], rtol=0, atol=1e-9)
    np.testing.assert_allclose(out.y[3:6], parts.y[3:6], rtol=0, atol=1e-3)


def test_interpolated_precession_axis_oracle(oracle_mod):
    """interpolatefields 1 in the oracle: the spin end states of the spline
    axis agree with the exact axis within the interpolation error, and the
    accumulated phase with |gamma_n| B0 t"""
    import sys
    import os
    sys.path.insert(0, os.path.dirname(__file__))
    from test_gpu_spin import spin_setup
    from pentrack_gb300 import scenes
    sc, params, parts = spin_setup(n=6, simtime=0.05)
    o = oracle_mod.Oracle(sc)
    exact, _ = o.integrate(params, parts)
    params.interpolatefields = 1
    interp, st = o.integrate(params, parts)
    assert st["spin_steps"] > 100
    assert np.array_equal(interp.y, exact.y)
    assert np.max(np.abs(interp.spin[:3] - exact.spin[:3])) < 1e-6
    w = abs(scenes.GAMMA_N) * 1e-6
    np.testing.assert_allclose(interp.spin[4], w * (interp.t - parts.t), rtol=1e-6)


def test_geometry_test_ignored_solids_oracle(oracle_mod):
    """test/GeometryTest/config.in: UCN stored in the steel hollow unit cube,
    which two unit cubes (centred on (0,0,0) and (1,0,0)) overlap, each listed
    twice -- as the default material ignored from 5 s to 10 s and as detector
    material ignored from 0 s to 5 s -- so the same surfaces change role at
    5 s, while UCN are inside them.  The reference's criterion: no geometry
    or integration errors; here also: absorption inside the box happens only
    in the cubes and only after 5 s."""
    from pentrack_gb300 import Scene, scenes as S, workloads
    from pentrack_gb300.engine import run_params
    sc = Scene()
    sc.add_material("default", 0.0)
    sc.add_material("Steel", 183.0, 0.1, 0.03)
    sc.add_material("UCNdet", 0.0, 0.1)
    c0 = S.box_mesh((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5))
    c1 = S.box_mesh((0.5, -0.5, -0.5), (1.5, 0.5, 0.5))
    sc.add_solid(1, "default")
    sc.add_solid(2, "default", c0, ignore=[(5.0, 10.0)])
    sc.add_solid(3, "default", c1, ignore=[(5.0, 10.0)])
    sc.add_solid(4, "Steel", workloads.hollow_cube_mesh())
    sc.add_solid(5, "UCNdet", c0, ignore=[(0.0, 5.0)])
    sc.add_solid(6, "UCNdet", c1, ignore=[(0.0, 5.0)])
    n = 2000
    ids = np.arange(n, dtype=np.int64)
    pos, (E, ph, th, pol) = S.source_box(5, ids, (0, 0, 0), (1, 1, 1), 0.0, 300e-9, polarization=0.0)
    parts = S.make_particles(5, ids, pos, E, ph, th, pol)
    params = run_params(A.NEUTRON, simtime=10.0, tau=0.0, tmax=9e99, lmax=9e99, bmax=0.1, spintimes=(0, 0), seed=5)
    out, st = oracle_mod.Oracle(sc).integrate(params, parts, nthreads=8)
    bad = (A.ID_GEOMETRY_ERROR, A.ID_CGAL_ERROR, A.ID_ODEINT_ERROR, A.ID_INITIAL_NOT_FOUND)
    assert not np.isin(out.stop_id, bad).any(), np.unique(out.stop_id, return_counts=True)
    # absorption in material inside the box: in the detector cubes, which are
    # ignored until 5 s (the default-material copies of the same cubes, which
    # do not absorb, are the active ones until then), so only after 5 s
    absorbed = out.stop_id == A.ID_ABSORBED_IN_MATERIAL
    p = out.y[0:3]
    interior = np.all((p > 0) & (p < 1), axis=0)
    in_cubes = ((np.abs(p[0]) < 0.5) | (np.abs(p[0] - 1) < 0.5)) & (np.abs(p[1]) < 0.5) & (np.abs(p[2]) < 0.5)
    det = absorbed & interior
    assert det.sum() > 100 and np.all(in_cubes[det]) and np.all(out.t[det] >= 5.0)
