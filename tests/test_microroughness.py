"""MicroRoughness (src/microroughness.cpp, TNeutron::OnHit's MR branches) in
the oracle, on the CPU.

* Steyerl's copper data, the reference's own MicroRoughness known answers
  (test/microroughnessTests.cpp, with its tolerances).
* MRDist against the reference's formula written out here with numpy complex
  numbers and scipy's I0, for reflection and transmission, with and
  without the phi integration.
* MRProb: the restated odeint integration (tolerance 1e-6) written out
  again here, and its convergence to adaptive quadrature.
* MRDistMax at least the maximum over a dense grid of the distribution.
* A rough floor under a box of UCN below its Fermi potential: the fraction
  of floor contacts that scatter diffusely equals the mean MRProb of those
  contacts (4 sigma), and the scattered directions are sin-distributed
  about the normal (cos theta uniform, KS), since the reference's envelope
  is the transmission maximum, which is zero below the potential step.
"""
import numpy as np
import pytest

from pentrack_gb300 import _abi as A

M_N = 1.0454074345680994e-08
ELE_E = 1.602176487e-19
HBAR = 1.05457266e-34


def mr_dist_literal(transmit, integral, v, n, Estep, b, w, theta, phi):
    from scipy.special import i0
    if theta < 0 or theta > np.pi / 2:
        return 0.0
    v = np.asarray(v, float)
    v2 = v @ v
    vn = v @ np.asarray(n, float)
    E = 0.5 * M_N * v2
    if transmit and E <= Estep:
        return 0.0
    ki = np.sqrt(2 * M_N * E) * ELE_E / HBAR
    kc = np.sqrt(2 * M_N * complex(Estep, 0)) * ELE_E / HBAR
    ci = abs(vn / np.sqrt(v2))
    Si = 2 * ci / (ci + np.sqrt(complex(ci * ci - kc * kc / ki / ki)))
    ct, st = np.cos(theta), np.sin(theta)
    kt = 0.0
    if transmit:
        kt = np.sqrt(2 * M_N * (E - Estep)) * ELE_E / HBAR
        if -(kc * kc).real / kt / kt > ct * ct:
            return 0.0
        So = 2 * ct / (ct + np.sqrt(ct * ct + kc * kc / kt / kt))
    else:
        So = 2 * ct / (ct + np.sqrt(ct * ct - kc * kc / ki / ki))
    si = np.sin(np.arccos(ci))
    kk = kt if transmit else ki
    if not integral:
        Fmu = np.exp(-w * w / 2 * (ki * ki * si * si + kk * kk * st * st - 2 * ki * kk * si * st * np.cos(phi)))
    else:
        Fmu = np.exp(-w * w / 2 * (ki * ki * si * si + kk * kk * st * st)) * 2 * np.pi * i0(w * w * ki * kk * si * st)
    factor = (kc ** 4).real * b * b * w * w / 8 / np.pi / ci
    if transmit:
        factor *= kt / ki
    if integral:
        factor *= st
    return factor * abs(Si) ** 2 * abs(So) ** 2 * Fmu


def contacts(seed=3, n=40):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        E = rng.uniform(20e-9, 300e-9)
        th = rng.uniform(0.02, 1.5)
        ph = rng.uniform(0, 2 * np.pi)
        v = np.sqrt(2 * E / M_N) * np.array([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), -np.cos(th)])
        out.append((v, np.array([0.0, 0.0, 1.0]), rng.choice([250e-9, 90e-9, -40e-9]), rng.uniform(0.5e-9, 3e-9),
                    rng.uniform(5e-9, 40e-9)))
    return out


def steyerl_cases():
    """the reference's MicroRoughness known answers (test/microroughnessTests.cpp,
    Steyerl's copper data; tests/golden/steyerl_mr.npz by gen_mr_fixture.py)"""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "steyerl_mr.npz"))
    kCu, b, w = float(g["kCu"]), float(g["bCu"]), float(g["wCu"])
    fermi = HBAR * HBAR * kCu * kCu / 2.0 / M_N / ELE_E / ELE_E
    vabs = 2.0 * np.pi * HBAR / M_N / ELE_E / float(g["wavelength"])
    th = float(g["theta_i"])
    v = np.array([vabs * np.sin(th), 0.0, vabs * np.cos(th)])
    normal = np.array([0.0, 0.0, -1.0])
    totals = []
    for lam, p in g["total"]:
        k = 2.0 * np.pi / lam / 1e-10
        ti = np.arccos(2.0 / 3.0 * kCu / k) if k > kCu else 48.0 / 180.0 * np.pi
        va = HBAR * k / M_N / ELE_E
        totals.append((np.array([va * np.sin(ti), 0.0, va * np.cos(ti)]), p))
    return dict(v=v, normal=normal, fermi=fermi, b=b, w=w, reflection=g["reflection"], transmission=g["transmission"],
                totals=totals)


def check_steyerl(dist, prob):
    """the reference's tolerances: a distribution value above 0.01 within 20 %
    of the iso-line's level, below it within 0.005; the total diffuse
    probability (reflection + transmission) within 2 %"""
    c = steyerl_cases()
    for transmit, table in ((False, c["reflection"]), (True, c["transmission"])):
        for level, th, ph in table:
            d = dist(transmit, c["v"], c["normal"], c["fermi"], c["b"], c["w"], th / 180 * np.pi, ph / 180 * np.pi)
            if d > 0.01:
                assert abs(d - level) <= 0.2 * level, (transmit, level, th, ph, d)
            else:
                assert abs(d - level) <= 0.005, (transmit, level, th, ph, d)
    for v, p in c["totals"]:
        r = prob(False, v, c["normal"], c["fermi"], c["b"], c["w"]) + prob(True, v, c["normal"], c["fermi"], c["b"], c["w"])
        assert abs(r - p) <= 0.02 * p, (p, r)


def test_oracle_reproduces_steyerl_copper_data(oracle_mod):
    check_steyerl(lambda tr, v, n, E, b, w, th, ph: oracle_mod.mr("dist", v, n, E, b, w, tr, False, th, ph),
                  lambda tr, v, n, E, b, w: oracle_mod.mr("prob", v, n, E, b, w, tr))


def test_mr_dist_matches_the_reference_formula(oracle_mod):
    rng = np.random.default_rng(1)
    for v, n, Estep, b, w in contacts():
        for transmit in (False, True):
            for integral in (False, True):
                for theta in rng.uniform(0, np.pi / 2, 5):
                    phi = rng.uniform(0, 2 * np.pi)
                    a = oracle_mod.mr("dist", v, n, Estep, b, w, transmit, integral, theta, phi)
                    r = mr_dist_literal(transmit, integral, v, n, Estep, b, w, theta, phi)
                    assert abs(a - r) <= 1e-12 * abs(r) + 1e-300, (transmit, integral, a, r)
    assert oracle_mod.mr("dist", *contacts()[0], theta=-0.1) == 0.0


def odeint_integrate(f, tol=1e-6):
    """odeint's integrate() of dx/dt = f(t) from 0 to pi/2 as the oracle
    restates it (Dormand-Prince 5(4) dense output, first step 0.01)"""
    T, t, x, dt, d0 = np.pi / 2, 0.0, 0.0, 0.01, f(0.0)
    eps = np.finfo(float).eps
    b = (35 / 384, 500 / 1113, 125 / 192, -2187 / 6784, 11 / 84)
    e = (35 / 384 - 5179 / 57600, 500 / 1113 - 7571 / 16695, 125 / 192 - 393 / 640, -2187 / 6784 + 92097 / 339200,
         11 / 84 - 187 / 2100, -1 / 40)
    while T - t > eps:
        while t + dt - T <= eps:
            while True:
                k3, k4, k5, k6 = f(t + dt * (3 / 10)), f(t + dt * (4 / 5)), f(t + dt * (8 / 9)), f(t + dt)
                xn = x + dt * (b[0] * d0 + b[1] * k3 + b[2] * k4 + b[3] * k5 + b[4] * k6)
                xe = dt * (e[0] * d0 + e[1] * k3 + e[2] * k4 + e[3] * k5 + e[4] * k6 + e[5] * k6)
                err = abs(xe) / (tol + tol * (abs(x) + abs(dt) * abs(d0)))
                if not err <= 1:
                    dt *= max(0.9 * err ** (-1 / 3), 0.2)
                    continue
                t, x, d0 = t + dt, xn, k6
                if err < 0.5:
                    dt *= 0.9 * max(3.2e-4, err) ** (-1 / 5)
                break
        if T - t > eps:
            dt, d0 = T - t, f(t)
    return x


def test_mr_prob_and_max(oracle_mod):
    """MRProb is the integration scheme above at the reference's tolerance
    (1e-6): the same scheme at 1e-10 converges to the quadrature, and at
    1e-6 it is within the tolerance where the integrand is smooth; where
    it has a cusp (reflection above the potential step, where the outgoing
    amplitude turns complex) or a jump (transmission below a negative step)
    the few steps of the coarse tolerance miss by up to a few per cent and
    a few tens of per cent, as the reference's integration does."""
    from scipy.integrate import quad
    for v, n, Estep, b, w in contacts(seed=4, n=24):
        E = 0.5 * M_N * (v @ v)
        for transmit in (False, True):
            f = lambda th: oracle_mod.mr("dist", v, n, Estep, b, w, transmit, True, th)  # noqa: E731
            p = oracle_mod.mr("prob", v, n, Estep, b, w, transmit)
            assert abs(p - odeint_integrate(f)) <= 1e-12 * abs(p) + 1e-300
            q = quad(f, 0, np.pi / 2, epsabs=1e-13, epsrel=1e-11, limit=500)[0]
            assert abs(odeint_integrate(f, 1e-10) - q) <= 5e-8 + 1e-5 * q
            if transmit and Estep < 0:
                assert abs(p - q) <= 0.35 * q, (transmit, p, q)
            elif not transmit and 0 < Estep < E:
                assert abs(p - q) <= 0.05 * q, (transmit, p, q)
            else:
                assert abs(p - q) <= 1e-5 + 1e-4 * q, (transmit, p, q)
            m = oracle_mod.mr("max", v, n, Estep, b, w, transmit)
            grid = max(oracle_mod.mr("dist", v, n, Estep, b, w, transmit, False, th)
                       for th in np.linspace(0, np.pi / 2, 2001))
            # m is a value of the distribution, so it cannot exceed its maximum;
            # it must not fall below any grid value (the peak next to the
            # transmission cut-off is narrower than the grid spacing)
            assert m >= grid * (1 - 1e-6), (transmit, m, grid)


def rough_box(b=3e-9, w=25e-9):
    """UCN stored in a 1.2 x 1.2 x 0.7 m box of a smooth 250 neV material
    (the default medium around the vacuum solid) whose floor at z = -0.1 m
    is the top face of a rough slab (MicroRoughness, 250 neV, higher ID), so
    that the floor contact is vacuum -> rough with no coplanar faces"""
    from pentrack_gb300 import Scene, scenes as S
    from pentrack_gb300.engine import run_params
    sc = Scene()
    sc.add_material("smooth", 250.0)
    sc.add_material("vacuum", 0.0)
    sc.add_material("rough", 250.0, rms_roughness=b, correl_length=w)
    sc.add_solid(1, "smooth")
    sc.add_solid(2, "vacuum", S.box_mesh((-0.6, -0.6, -0.2), (0.6, 0.6, 0.6)))
    sc.add_solid(3, "rough", S.box_mesh((-0.7, -0.7, -0.3), (0.7, 0.7, -0.1)))
    return sc, run_params


def rough_box_run(n, simtime, seed=77):
    from pentrack_gb300 import scenes as S
    sc, run_params = rough_box()
    ids = np.arange(n, dtype=np.int64)
    pos, (E, ph, th, pol) = S.source_box(seed, ids, (-0.5, -0.5, 0.2), (0.5, 0.5, 0.3), 20e-9, 150e-9)
    parts = S.make_particles(seed, ids, pos, E, ph, th, pol)
    params = run_params(A.NEUTRON, simtime=simtime, tau=0.0, tmax=9e99, lmax=9e99, bmax=0.1, spintimes=(0, 0),
                        seed=seed)
    params.hitlog = 1
    params.log_capacity = 2_000_000
    return sc, params, parts


def floor_contacts(rec):
    """floor hits of a hit log: incident and outgoing velocities, and
    whether the reflection was specular (v_out = mirror of v_in up to the
    gravity acting across the hit's 1e-8 m bracket; a diffuse one turns the
    velocity by O(1))"""
    n = rec[:, 13:16]
    fl = (np.abs(rec[:, 4] + 0.1) < 1e-6) & (np.abs(n[:, 2]) > 0.5)  # not the side walls' lowest points
    v1, v2 = rec[fl, 5:8], rec[fl, 9:12]
    mirror = v1.copy()
    mirror[:, 2] *= -1
    spec = np.all(np.abs(v2 - mirror) <= 1e-4 * np.abs(v1).max(axis=1, keepdims=True), axis=1)
    return v1, v2, spec, n[fl]


def test_rough_floor_scatters_as_the_model_says(oracle_mod):
    from scipy import stats
    sc, params, parts = rough_box_run(1500, 3.0)
    o = oracle_mod.Oracle(sc)
    out, st = o.integrate(params, parts, nthreads=8)
    rec = o.read_log(A.LOG_HIT)
    v1, v2, spec, nrm = floor_contacts(rec)
    assert len(v1) > 5000
    # the floor's normal points out of the box's wall solid, into the box: (0, 0, 1) or its opposite
    p = np.array([oracle_mod.mr("prob", v1[i], nrm[i], 250e-9, 3e-9, 25e-9) for i in range(len(v1))])
    diffuse = ~spec
    expect = p.sum()
    sigma = np.sqrt((p * (1 - p)).sum())
    assert abs(diffuse.sum() - expect) < 4 * sigma + 3, (diffuse.sum(), expect, sigma)
    # diffusely scattered directions: cos theta to the normal uniform on [0, 1]
    cth = np.abs(v2[diffuse, 2]) / np.linalg.norm(v2[diffuse], axis=1)
    assert stats.kstest(cth, "uniform").pvalue > 1e-3
    assert np.all(v2[diffuse, 2] > 0)  # back into the box
    # no particle lost: walls are total reflectors without loss
    assert np.all(out.stop_id == A.ID_NOT_FINISH)
