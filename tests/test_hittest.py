"""The reference's wall-hit test (test/HitTest): UCN of 110 neV fired at 45
degrees from 1 mm in front of the inner wall of the hollow unit cube, an
aluminium shell (Fermi potential 54.1 neV, imaginary part 0.00756 neV, 10 %
Lambert reflection), tracked for 1 ms so that each meets the wall once.  The
reflected, transmitted, specularly reflected and specularly transmitted
fractions of the hit log must equal the values its macro
(test/HitTest/showscatterdist.cxx) expects, within 4 binomial standard
errors; the fixture tests/golden/hittest.npz holds the configuration and
those values (tests/golden/gen_hittest_fixture.py)."""
import os

import numpy as np
import pytest

from pentrack_gb300 import _abi as A

GOLD = os.path.join(os.path.dirname(__file__), "golden", "hittest.npz")


def hittest_setup(n, seed=31):
    from pentrack_gb300 import Scene, scenes as S, workloads
    from pentrack_gb300.engine import run_params
    g = np.load(GOLD)
    sc = Scene()
    sc.add_material("default", 0.0)
    sc.add_material("Al", *[float(v) for v in g["al"]])
    sc.add_solid(1, "default")
    sc.add_solid(2, "Al", workloads.hollow_cube_mesh())
    src = g["source"]
    lo, hi = (src[0], src[2], src[4]), (src[1], src[3], src[5])
    th, ph = float(g["theta_v"]) * np.pi / 180, float(g["phi_v"]) * np.pi / 180
    E = float(g["energy"])
    ids = np.arange(n, dtype=np.int64)
    pos, (E, phv, thv, pol) = S.source_box(seed, ids, lo, hi, E, E, theta=(th, th), phi=(ph, ph), polarization=0.0)
    parts = S.make_particles(seed, ids, pos, E, phv, thv, pol)
    params = run_params(A.NEUTRON, simtime=float(g["simtime"]), tau=880.0, tmax=9e99, lmax=9e99, bmax=0.1,
                        spintimes=(0, 0), seed=seed)
    params.hitlog = 1
    params.log_capacity = 4 * n
    return sc, params, parts, g


def scatter_fractions(rec):
    """showscatterdist.cxx's classification of the hit records"""
    v1, v2, n = rec[:, 5:8], rec[:, 9:12], rec[:, 13:16]
    th1 = np.arccos((v1 * n).sum(1) / np.linalg.norm(v1, axis=1))
    th2 = np.arccos((v2 * n).sum(1) / np.linalg.norm(v2, axis=1))
    ph1, ph2 = np.arctan2(v1[:, 0], v1[:, 2]), np.arctan2(v2[:, 0], v2[:, 2])
    refl = th2 < np.pi / 2
    spec_r = (th1 - np.pi / 2 - th2) ** 2 + (ph1 - ph2) ** 2 < 1e-6
    spec_t = ~refl & ((ph1 - ph2) ** 2 < 1e-16)
    return len(rec), refl.sum(), (~refl).sum(), spec_r.sum(), spec_t.sum()


def check_fractions(rec, g):
    total, refl, trans, spec_r, spec_t = scatter_fractions(rec)
    for k, m, p in ((refl, total, float(g["reflected"])), (trans, total, float(g["transmitted"])),
                    (spec_r, refl, float(g["specular_reflected"])), (spec_t, trans, float(g["specular_transmitted"]))):
        assert abs(k / m - p) <= 4 * np.sqrt(p * (1 - p) / m), (k, m, p)
    return total, refl, trans, spec_r, spec_t


def test_hittest_oracle(oracle_mod):
    n = 20000
    sc, params, parts, g = hittest_setup(n)
    o = oracle_mod.Oracle(sc)
    out, st = o.integrate(params, parts, nthreads=8)
    rec = o.read_log(A.LOG_HIT)
    assert len(rec) == n and np.array_equal(np.sort(rec[:, 0]), np.arange(n))  # one wall contact each
    check_fractions(rec, g)


@pytest.mark.gpu
def test_hittest_gpu(built, oracle_mod):
    """the same on the GPU (plain and batched forms identical), and equal to
    the oracle's hit records"""
    from pentrack_gb300 import Engine
    n = 20000
    sc, params, parts, g = hittest_setup(n)
    e = Engine(sc)
    out, _ = e.integrate(params, parts)
    rec, total = e.read_log(A.LOG_HIT)
    assert total == n and len(rec) == n
    gf = check_fractions(rec, g)
    params.mode = A.MODE_BATCHED
    outb, _ = e.integrate(params, parts)
    recb, _ = e.read_log(A.LOG_HIT)
    assert np.array_equal(out.y, outb.y) and np.array_equal(rec, recb)
    o = oracle_mod.Oracle(sc)
    o.integrate(params, parts, nthreads=8)
    assert scatter_fractions(o.read_log(A.LOG_HIT)) == gf
