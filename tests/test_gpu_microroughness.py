"""MicroRoughness walls on the device (needs a GB300) against the oracle.

* The kernels' MRDist, MRProb and MRDistMax (pt_mr_eval) equal the oracle's
  (1e-12; integrals and maxima 1e-7) and reproduce the reference's Steyerl
  copper known answers with its tolerances.

* A rough floor below the UCN's energies (tests/test_microroughness.py's
  box, 1,500 UCN x 3 s): the plain and batched forms are identical; the
  diffuse fraction of the GPU's floor contacts equals their mean MRProb
  (4 sigma) and the diffuse directions are sin-distributed about the normal
  (KS); stop IDs equal the oracle's and the end states agree (the MR
  directions use cos/sin/acos, whose last bit may differ between CUDA and
  the host library).
* A rough floor of 60 neV under UCN of up to 150 neV, so that MicroRoughness
  transmission and reflection above the step both occur: the counts of
  floor contacts, diffuse reflections and transmissions agree with the
  oracle's within binomial errors, and the end heights by KS.
"""
import numpy as np
import pytest

from pentrack_gb300 import _abi as A

pytestmark = pytest.mark.gpu

from test_microroughness import check_steyerl, contacts, floor_contacts, rough_box_run  # noqa: E402


def test_device_mr_functions_equal_oracle_and_steyerl(built, oracle_mod):
    """pt_mr_eval (the kernels' own MRDist / MRProb / MRDistMax) against the
    oracle's restatement (std::complex, the library I0) at random contacts,
    and against the reference's Steyerl copper known answers"""
    from pentrack_gb300 import Engine
    from test_opera2d import table_scene
    e = Engine(table_scene(np.linspace(0, 1, 3), np.linspace(0, 1, 3), bz=np.zeros((3, 3))))
    rng = np.random.default_rng(2)
    cs = contacts(seed=6, n=64)
    for transmit in (False, True):
        for integral in (False, True):
            th, ph = rng.uniform(0, np.pi / 2, len(cs)), rng.uniform(0, 2 * np.pi, len(cs))
            g = e.mr("dist", [c[0] for c in cs], [c[1] for c in cs], [c[2] for c in cs], [c[3] for c in cs],
                     [c[4] for c in cs], transmit, integral, th, ph)
            o = np.array([oracle_mod.mr("dist", *c, transmit, integral, th[i], ph[i]) for i, c in enumerate(cs)])
            np.testing.assert_allclose(g, o, rtol=1e-12, atol=1e-300)
        for what in ("prob", "max"):
            g = e.mr(what, [c[0] for c in cs], [c[1] for c in cs], [c[2] for c in cs], [c[3] for c in cs],
                     [c[4] for c in cs], transmit)
            o = np.array([oracle_mod.mr(what, *c, transmit) for c in cs])
            # the integration's steps and the maximum's search points carry
            # the two sides' last-bit differences of cos/sin/exp (measured
            # up to 5e-9 relative)
            np.testing.assert_allclose(g, o, rtol=1e-7, atol=1e-300)
    check_steyerl(lambda tr, v, n, E, b, w, th, ph: e.mr("dist", v, n, E, b, w, tr, False, th, ph)[0],
                  lambda tr, v, n, E, b, w: e.mr("prob", v, n, E, b, w, tr)[0])


def run_both(sc, params, parts, oracle_mod):
    from pentrack_gb300 import Engine
    e = Engine(sc)
    params.mode = A.MODE_PLAIN
    gp, _ = e.integrate(params, parts)
    rp, _ = e.read_log(A.LOG_HIT)
    params.mode = A.MODE_BATCHED
    gb, _ = e.integrate(params, parts)
    rb, _ = e.read_log(A.LOG_HIT)
    o = oracle_mod.Oracle(sc)
    oo, _ = o.integrate(params, parts, nthreads=8)
    return gp, rp, gb, rb, oo, o.read_log(A.LOG_HIT)


def test_rough_floor_below_the_step_gpu(built, oracle_mod):
    from scipy import stats
    sc, params, parts = rough_box_run(1500, 3.0)
    gp, rp, gb, rb, oo, ro = run_both(sc, params, parts, oracle_mod)
    for k in ("t", "y", "stop_id", "n_hit"):
        assert np.array_equal(getattr(gp, k), getattr(gb, k)), k
    assert np.array_equal(rp, rb)
    v1, v2, spec, nrm = floor_contacts(rp)
    assert len(v1) > 5000
    p = np.array([oracle_mod.mr("prob", v1[i], nrm[i], 250e-9, 3e-9, 25e-9) for i in range(len(v1))])
    diffuse = ~spec
    assert abs(diffuse.sum() - p.sum()) < 4 * np.sqrt((p * (1 - p)).sum()) + 3, (diffuse.sum(), p.sum())
    cth = np.abs(v2[diffuse, 2]) / np.linalg.norm(v2[diffuse], axis=1)
    assert stats.kstest(cth, "uniform").pvalue > 1e-3
    assert np.all(v2[diffuse, 2] > 0)
    assert np.array_equal(gp.stop_id, oo.stop_id)
    od = ~floor_contacts(ro)[2]
    assert abs(int(diffuse.sum()) - int(od.sum())) <= 0.02 * od.sum() + 5
    dpos = np.abs(gp.y[0:3] - oo.y[0:3]).max(0)
    assert np.median(dpos) < 1e-9 and np.mean(dpos < 1e-6) > 0.95, (np.median(dpos), np.mean(dpos < 1e-6))


def test_rough_floor_above_the_step_gpu(built, oracle_mod):
    from scipy import stats
    from test_microroughness import rough_box
    from pentrack_gb300 import scenes as S
    sc, run_params = rough_box()
    sc.materials[2] = (60.0,) + sc.materials[2][1:]  # the rough slab at 60 neV
    n = 3000
    ids = np.arange(n, dtype=np.int64)
    pos, (E, ph, th, pol) = S.source_box(91, ids, (-0.5, -0.5, 0.2), (0.5, 0.5, 0.3), 20e-9, 150e-9)
    parts = S.make_particles(91, ids, pos, E, ph, th, pol)
    params = run_params(A.NEUTRON, simtime=2.0, tau=0.0, tmax=9e99, lmax=9e99, bmax=0.1, spintimes=(0, 0), seed=91)
    params.hitlog = 1
    params.log_capacity = 2_000_000
    gp, rp, gb, rb, oo, ro = run_both(sc, params, parts, oracle_mod)
    assert np.array_equal(gp.y, gb.y) and np.array_equal(rp, rb)

    def counts(rec):
        n = rec[:, 13:16]
        top = (np.abs(rec[:, 4] + 0.1) < 1e-6) & (np.abs(n[:, 2]) > 0.5) & (rec[:, 5 + 2] < 0)  # downward at the top face
        v1, v2 = rec[top, 5:8], rec[top, 9:12]
        refl = v2[:, 2] > 0
        mirror = np.all(np.abs(v2 - v1 * [1, 1, -1]) <= 1e-4 * np.abs(v1).max(1, keepdims=True), axis=1)
        # specular transmission keeps the tangential velocity
        trans_spec = ~refl & np.all(np.abs(v2[:, :2] - v1[:, :2]) <= 1e-4 * np.abs(v1).max(1, keepdims=True), axis=1)
        return top.sum(), (refl & ~mirror).sum(), (~refl & ~trans_spec).sum(), (~refl).sum()

    g, o = counts(rp), counts(ro)
    assert g[1] > 50 and g[2] > 10, g  # diffuse reflections and MicroRoughness transmissions happen
    for a, b in zip(g, o):
        assert abs(int(a) - int(b)) <= 4 * np.sqrt(max(a, b)) + 5, (g, o)
    assert stats.ks_2samp(gp.y[2], oo.y[2]).pvalue > 1e-3
