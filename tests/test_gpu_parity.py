"""GPU engine vs the CPU oracle through the C ABI (needs a GB300).

Tolerances (FP64 state update):
* field values and gradients: the device evaluates the tensor-product cubic
  Hermite form of the same tricubic the oracle evaluates in the reference's
  Lekien-Marsden/Horner form: relative 1e-12 of the table scale (FP64 mode),
  1e-5 (FP32 field mode).
* segment-mesh collisions: identical hit sets, bit-identical parameters s.
* per-particle end states of the deterministic cube storage: within 1e-6
  relative (positions to the 1 m cube, velocities to the particle speed).
"""
import numpy as np
import pytest

from pentrack_gb300 import _abi as A

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng(built):
    from pentrack_gb300 import Engine
    return Engine


def nonlinear_table(n=(9, 11, 7)):
    rng = np.random.default_rng(3)
    ax = []
    for k, m in enumerate(n):
        a = np.sort(rng.uniform(-0.3, 0.3, m))
        a[0], a[-1] = -0.3, 0.3
        ax.append(a)
    X, Y, Z = np.meshgrid(*ax, indexing="ij")
    bx = 0.7 * np.sin(3 * X) * np.cos(2 * Y) + 0.1 * Z
    by = 0.5 * np.cos(4 * Y + Z) - 0.2 * X * Y
    bz = 1e-5 + 0.3 * X * Z * Z + np.sin(5 * Z)
    return ax, (bx, by, bz)


def table_scene(ax, comps, **kw):
    from pentrack_gb300 import Scene, scenes
    sc = Scene()
    sc.add_material("m", 0.0)
    sc.add_solid(1, 0)
    sc.add_solid(2, 0, scenes.box_mesh((-0.25, -0.25, -0.25), (0.25, 0.25, 0.25)))
    sc.add_table3d(*ax, *comps, **kw)
    return sc


@pytest.mark.parametrize("kind", ["quadrupole", "nonlinear", "boundary"])
def test_tab3_field_matches_oracle(eng, oracle_mod, kind):
    from pentrack_gb300 import workloads
    if kind == "quadrupole":
        ax, comps = workloads.quadrupole_table(16)
        sc = table_scene(ax, comps)
    elif kind == "nonlinear":
        ax, comps = nonlinear_table()
        sc = table_scene(ax, comps, b_scale=1.3)
    else:
        ax, comps = nonlinear_table()
        sc = table_scene(ax, comps, boundary_width=0.05, box=(0.25, -0.28, 0.3, -0.3, 0.2, -0.3))
    rng = np.random.default_rng(11)
    lo = np.array([a[0] for a in ax]) - 0.05
    hi = np.array([a[-1] for a in ax]) + 0.05
    q = np.column_stack([rng.uniform(lo, hi, (4000, 3)), np.zeros(4000)])
    q[:50, 0] = ax[0][rng.integers(0, len(ax[0]), 50)]  # exactly on grid planes
    e = eng(sc)
    B, dB, _, _ = e.field(q)
    Bo, dBo, _, _ = oracle_mod.Oracle(sc).field(q)
    scale = max(np.abs(Bo).max(), 1e-30)
    gscale = max(np.abs(dBo).max(), 1e-30)
    assert np.max(np.abs(B - Bo)) <= 1e-12 * scale
    assert np.max(np.abs(dB - dBo)) <= 1e-11 * gscale
    # FP32 field mode: FP32 node table, corner-linear base split off
    B32, dB32, _, _ = e.field(q, precision=A.PREC_FP32)
    assert np.max(np.abs(B32 - Bo)) <= 1e-6 * scale
    assert np.max(np.abs(dB32 - dBo)) <= 1e-6 * gscale
    inside = (np.abs(B).sum(1) > 0)
    assert inside.sum() > 1000 and (~inside).sum() > 100  # both regimes exercised


def test_harmonic_field_closed_forms(eng):
    """HarmonicExpansionBField l <= 2 against the closed forms of the reference's
    expansion (src/harmonicfields.cpp:76-288 for these (l, m))."""
    from pentrack_gb300 import Scene, scenes
    rng = np.random.default_rng(4)
    coeffs = [(0, -1, 0.3), (0, 0, 1e-6), (0, 1, -0.2), (1, -2, 7.5), (1, -1, 0.4), (1, 0, -1.1), (1, 1, 0.9),
              (1, 2, 0.5), (2, -3, 1.7), (2, -2, -0.6), (2, -1, 0.8), (2, 0, 1.2), (2, 1, -0.3), (2, 2, 0.25), (2, 3, 2.0)]
    sc = Scene()
    sc.add_material("m", 0.0)
    sc.add_solid(1, 0)
    sc.add_solid(2, 0, scenes.box_mesh((-1, -1, -1), (1, 1, 1)))
    off = (0.01, -0.02, 0.03)
    sc.add_harmonic(coeffs, offset=off)
    p = rng.uniform(-0.3, 0.3, (500, 3))
    B, dB, _, _ = eng(sc).field(np.column_stack([p, np.zeros(len(p))]))
    x, y, z = (p[:, k] + off[k] for k in range(3))
    ref = np.zeros((len(p), 3))
    forms = {
        (0, -1): (0 * x, 1 + 0 * x, 0 * x), (0, 0): (0 * x, 0 * x, 1 + 0 * x), (0, 1): (1 + 0 * x, 0 * x, 0 * x),
        (1, -2): (y, x, 0 * x), (1, -1): (0 * x, z, y), (1, 0): (-x / 2, -y / 2, z), (1, 1): (z, 0 * x, x),
        (1, 2): (x, -y, 0 * x),
        (2, -3): (2 * x * y, (x - y) * (x + y), 0 * x), (2, -2): (2 * y * z, 2 * x * z, 2 * x * y),
        (2, -1): (-x * y / 2, -x * x / 4 - 3 * y * y / 4 + z * z, 2 * y * z), (2, 0): (-x * z, -y * z, -x * x / 2 - y * y / 2 + z * z),
        (2, 1): (-3 * x * x / 4 - y * y / 4 + z * z, -x * y / 2, 2 * x * z), (2, 2): (2 * x * z, -2 * y * z, (x - y) * (x + y)),
        (2, 3): ((x - y) * (x + y), -2 * x * y, 0 * x),
    }
    for l, m, g in coeffs:
        fx, fy, fz = forms[(l, m)]
        ref += g * np.column_stack([fx, fy, fz])
    assert np.max(np.abs(B - ref)) < 1e-13 * np.abs(ref).max()
    # gradient: curl-free and divergence-free, and consistent with finite differences
    assert np.max(np.abs(np.trace(dB, axis1=1, axis2=2))) < 1e-12
    assert np.max(np.abs(dB - np.transpose(dB, (0, 2, 1)))) < 1e-12
    h = 1e-6
    q = np.column_stack([p, np.zeros(len(p))])
    for k in range(3):
        qp, qm = q.copy(), q.copy()
        qp[:, k] += h
        qm[:, k] -= h
        fd = (eng(sc).field(qp)[0] - eng(sc).field(qm)[0]) / (2 * h)
        assert np.max(np.abs(fd - dB[:, :, k])) < 1e-6


def test_harmonic_field_matches_oracle(eng, oracle_mod):
    """Every HarmonicExpansionBField term up to l = 5 (random G), with offset,
    box, smoothing band and scale: device polynomial vs the oracle's terms
    derived symbolically (oracle/gen_harmonic.py)."""
    from pentrack_gb300 import Scene, scenes
    rng = np.random.default_rng(12)
    coeffs = [(l, m, float(rng.normal()) * 10.0 ** -l) for l in range(6) for m in range(-l - 1, l + 2)]
    sc = Scene()
    sc.add_material("m", 0.0)
    sc.add_solid(1, 0)
    sc.add_solid(2, 0, scenes.box_mesh((-1, -1, -1), (1, 1, 1)))
    sc.add_harmonic(coeffs, offset=(0.02, -0.01, 0.03), b_scale=0.8, boundary_width=0.05,
                    box=(0.3, -0.3, 0.3, -0.3, 0.25, -0.25))
    p = rng.uniform(-0.35, 0.35, (3000, 3))
    q = np.column_stack([p, np.zeros(len(p))])
    B, dB, _, _ = eng(sc).field(q)
    Bo, dBo, _, _ = oracle_mod.Oracle(sc).field(q)
    scale, gscale = np.abs(Bo).max(), np.abs(dBo).max()
    assert np.max(np.abs(B - Bo)) <= 1e-12 * scale
    assert np.max(np.abs(dB - dBo)) <= 1e-11 * gscale
    B32, dB32, _, _ = eng(sc).field(q, precision=A.PREC_FP32)
    assert np.max(np.abs(B32 - Bo)) <= 1e-6 * scale
    inside = np.abs(Bo).sum(1) > 0
    assert inside.sum() > 1000 and (~inside).sum() > 100


@pytest.mark.parametrize("mesh", ["cylinder", "hollow"])
def test_collisions_match_oracle(eng, oracle_mod, mesh):
    from pentrack_gb300 import Scene, scenes, workloads
    sc = Scene()
    sc.add_material("m", 0.0)
    sc.add_solid(1, 0)
    if mesh == "cylinder":
        sc.add_solid(2, 0, scenes.cylinder_mesh(0.2, -0.05, 0.05, 256))
        sc.add_solid(3, 0, scenes.box_mesh((-0.1, -0.1, -0.02), (0.1, 0.1, 0.02)), ignore=[(1.0, 2.0)])
        lo, hi = -0.3, 0.3
    else:
        sc.add_solid(2, 0, workloads.hollow_cube_mesh())
        lo, hi = -0.2, 1.2
    rng = np.random.default_rng(21)
    p = rng.uniform(lo, hi, (3000, 3))
    d = rng.normal(size=(3000, 3)) * rng.choice([1e-9, 1e-6, 1e-3, 0.1, 1.0], size=(3000, 1))
    segs = np.hstack([p, p + d])
    # segments ending exactly on a plane of the mesh
    segs[:100, 5] = segs[:100, 2] * 0 + (0.05 if mesh == "cylinder" else 0.0)
    e = eng(sc)
    c1, s1, n1, i1, d1 = e.collisions(segs)
    c2, s2, n2, i2, d2 = oracle_mod.Oracle(sc).collisions(segs)
    assert np.array_equal(c1, c2)
    assert (c1 > 0).sum() > 150
    for i in np.nonzero(c1 > 0)[0]:
        k = min(c1[i], 8)
        assert np.array_equal(s1[i, :k], s2[i, :k])
        assert np.array_equal(i1[i, :k], i2[i, :k])
        assert np.allclose(n1[i, :k], n2[i, :k], rtol=0, atol=1e-15)
        assert np.allclose(d1[i, :k], d2[i, :k], rtol=1e-15, atol=1e-300)
    pts = rng.uniform(lo, hi, (3000, 3))
    assert np.array_equal(e.point_solids(pts), oracle_mod.Oracle(sc).point_solids(pts))


def compare_states(gpu, orc, pos_tol=1e-6, vel_tol=1e-6):
    assert np.array_equal(gpu.stop_id, orc.stop_id)
    assert np.allclose(gpu.t, orc.t, rtol=1e-9, atol=1e-9)
    dpos = np.abs(gpu.y[0:3] - orc.y[0:3]).max(0)
    v = np.sqrt((orc.y[3:6] ** 2).sum(0)) + 1e-3
    dvel = np.abs(gpu.y[3:6] - orc.y[3:6]).max(0) / v
    return dpos, dvel


def test_cube_storage_parity(eng, oracle_mod):
    """The plain-method configuration at its stated size: 10,000 UCN in the
    closed unit cube (gravity, specular 335 neV walls, 0-200 neV) for 100 s,
    per-particle end states within 1e-6 of the oracle."""
    from pentrack_gb300 import workloads
    sc, params, parts = workloads.cube_storage(n=10_000, simtime=100.0)
    gout, gst = eng(sc).integrate(params, parts)
    oout, ost = oracle_mod.Oracle(sc).integrate(params, parts)
    dpos, dvel = compare_states(gout, oout)
    assert np.max(dpos) < 1e-6, np.max(dpos)
    assert np.max(dvel) < 1e-6, np.max(dvel)
    assert np.array_equal(gout.n_hit, oout.n_hit)
    assert np.all(gout.stop_id == A.ID_NOT_FINISH)
    assert gst["rk_accepted"] == ost["rk_accepted"]
    # the FP64 arithmetic of the integrator is identical on both sides
    # (explicit FMA chains, deterministic step-size power): bitwise end states
    bitwise = np.all(gout.y == oout.y, axis=0) & (gout.t == oout.t)
    assert bitwise.mean() >= 0.99, bitwise.mean()


@pytest.mark.parametrize("mode", [A.MODE_PLAIN, A.MODE_BATCHED])
def test_fenced_cube_bisection_dead_ends(eng, oracle_mod, mode):
    """Non-convex geometry: chords that cut a corner of the inner block while
    neither half does make the bisection back up (iterate_collision returning
    false at a level).  The GPU's stack-based search must visit the same
    intervals as the recursive reference: identical dead-end counts, hit
    counts and (almost always) bitwise end states."""
    from pentrack_gb300 import workloads
    sc, params, parts = workloads.fenced_cube(n=2000, simtime=100.0)
    oout, ost = oracle_mod.Oracle(sc).integrate(params, parts)
    params.mode = mode
    gout, gst = eng(sc).integrate(params, parts)
    assert ost["bisect_dead"] > 20
    assert gst["bisect_dead"] == ost["bisect_dead"]
    assert gst["bisection_levels"] == ost["bisection_levels"]
    assert np.array_equal(gout.n_hit, oout.n_hit)
    assert np.array_equal(gout.stop_id, oout.stop_id)
    dpos, dvel = compare_states(gout, oout)
    assert np.max(dpos) < 1e-6, np.max(dpos)
    bitwise = np.all(gout.y == oout.y, axis=0) & (gout.t == oout.t)
    assert bitwise.mean() >= 0.99, bitwise.mean()


def test_integration_test_known_answer_gpu(eng):
    from pentrack_gb300 import workloads
    sc, params, parts = workloads.integration_test(n=500)
    out, st = eng(sc).integrate(params, parts)
    a = workloads.integration_test_acceleration(0.5)
    first = (out.n_hit == 1) & (out.stop_id == A.ID_ABSORBED_IN_MATERIAL) & (out.y[2] < 0.5)
    assert first.sum() > 250
    x0, z0, vx0, vz0 = parts.y[0], parts.y[2], parts.y[3], parts.y[5]
    ze = out.y[2]
    t_hit = (-vz0 - np.sqrt(vz0 * vz0 - 2 * a * (z0 - ze))) / a
    res = (out.y[0] - x0 - vx0 * t_hit)[first]
    assert np.max(np.abs(res)) < 1e-6


def test_field_storage_short_parity(eng, oracle_mod):
    """Field-storage physics (tricubic quadrupole, +-mu grad|B|,
    Fermi walls with Lambert diffuse and loss, decay) over 0.5 s: the same
    Philox stream drives both, so end states agree particle by particle."""
    from pentrack_gb300 import workloads
    sc, params, parts = workloads.field_storage(n=512, simtime=0.5)
    e = eng(sc)
    sc, params, parts = workloads.field_storage(n=512, simtime=0.5, engine=e)
    gout, gst = e.integrate(params, parts)
    oout, ost = oracle_mod.Oracle(sc).integrate(params, parts)
    # The two sides evaluate the same tricubic in different exact forms
    # (Hermite vs Lekien-Marsden/Horner); 1e-16 differences in the force are
    # amplified by the step-size controller and the 1e-8 m bisection brackets
    # to ~1e-8 m over 0.5 s, and rarely flip a random branch.
    same = gout.stop_id == oout.stop_id
    assert same.mean() > 0.97
    dpos, dvel = compare_states_loose(gout, oout, same)
    assert np.median(dpos) < 1e-7
    assert np.mean(dpos < 1e-6) > 0.9
    assert abs(gst["hits"] - ost["hits"]) <= 0.02 * ost["hits"]


def compare_states_loose(g, o, mask):
    dpos = np.abs(g.y[0:3, mask] - o.y[0:3, mask]).max(0)
    v = np.sqrt((o.y[3:6, mask] ** 2).sum(0)) + 1e-3
    dvel = np.abs(g.y[3:6, mask] - o.y[3:6, mask]).max(0) / v
    return dpos, dvel


def test_pause_and_resume_is_bit_identical(eng):
    """Advancing in lab-time windows (paused at step boundaries) gives exactly
    the uninterrupted result."""
    from pentrack_gb300 import workloads
    sc, params, parts = workloads.field_storage(n=256, simtime=0.3)
    e = eng(sc)
    one, _ = e.integrate(params, parts)
    b = e.batch(params, parts)
    for tp in (0.05, 0.1, 0.17, 0.3, float("inf")):
        st = b.advance(tp)
    win = b.read()
    assert st["active"] == 0
    for k in ("t", "y", "spin", "stop_id", "n_hit", "n_step", "h_max", "n_accepted"):
        assert np.array_equal(getattr(one, k), getattr(win, k)), k


@pytest.mark.parametrize("mode", [A.MODE_BATCHED, A.MODE_PHASED])
@pytest.mark.parametrize("precision", [A.PREC_FP64, A.PREC_FP32])
def test_plain_and_batched_forms_are_bit_identical(eng, precision, mode):
    """The batched forms (persistent lanes refilled from a device queue inside
    a device-scheduled CUDA graph; host-driven phase split) schedule the same
    per-particle arithmetic as the plain form, so every output is
    bit-identical."""
    from pentrack_gb300 import workloads
    sc, params, parts = workloads.field_storage(n=4096, simtime=0.4)
    e = eng(sc)
    params.field_precision = precision
    params.mode = A.MODE_PLAIN
    plain, sp = e.integrate(params, parts)
    params.mode = mode
    batched, sb = e.integrate(params, parts)
    for k in ("t", "y", "spin", "stop_id", "n_hit", "n_step", "n_spinflip", "h_max", "noflip_prob", "n_accepted",
              "n_rejected", "solid"):
        assert np.array_equal(getattr(plain, k), getattr(batched, k)), k
    assert sp["rk_accepted"] == sb["rk_accepted"]
    assert sb["try_ms"] > 0
    if mode == A.MODE_BATCHED:
        assert sb["graph_launches"] >= 1 and sb["sched_outer_iters"] >= 1


@pytest.mark.parametrize("scheduler,max_run,period", [(A.SCHED_PHASED, 0, 0), (A.SCHED_PHASED, 0, 1), (A.SCHED_PERSISTENT, 0, 0),
                                                      (A.SCHED_PERSISTENT, 3, 2), (A.SCHED_PERSISTENT_WIDE, 1, 1),
                                                      (A.SCHED_PHASED_WIDE, 0, 0),
                                                      (A.SCHED_AUTO, 0, 2)])
def test_batched_schedulers_are_bit_identical(eng, scheduler, max_run, period):
    """Every scheduler of the batched form (phase split or persistent lanes in
    the device-scheduled graph, the autotuner switching between them), a
    hand-back after max_run consecutive steps and short graph periods only
    change which lane runs a particle when: the results stay the plain
    form's, in step budgets as the bench uses them."""
    from pentrack_gb300 import workloads
    sc, params, parts = workloads.field_storage(n=6000, simtime=0.3)
    e = eng(sc)
    params.field_precision = A.PREC_FP32
    params.mode = A.MODE_PLAIN
    pb = e.batch(params, parts)
    for _ in range(3):
        pb.advance(max_steps=16)
    plain = pb.read()
    params.mode = A.MODE_BATCHED
    params.max_run, params.period_iters, params.scheduler = max_run, period, scheduler
    bb = e.batch(params, parts)
    for _ in range(3):
        st = bb.advance(max_steps=16)
    batched = bb.read()
    for k in ("t", "y", "stop_id", "n_hit", "n_step", "h_max", "n_accepted", "n_rejected"):
        assert np.array_equal(getattr(plain, k), getattr(batched, k)), k
    assert st["graph_launches"] >= 1
    if scheduler == A.SCHED_AUTO:  # the trials ran, one scheduler was chosen
        assert st["scheduler"] in (A.SCHED_PHASED, A.SCHED_PERSISTENT, A.SCHED_PERSISTENT_WIDE, A.SCHED_PHASED_WIDE)
        assert all(x > 0 for x in st["tune_ns_per_try"])
    else:
        assert st["scheduler"] == scheduler
