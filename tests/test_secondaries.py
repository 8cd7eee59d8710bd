"""Neutron-decay secondaries (TNeutron::Decay, src/neutron.cpp:285-375):
four-momentum conservation, the proton recoil spectrum (KS against
ProtonBetaSpectrum, src/globals.cpp:84-92), the electron endpoint, and the
secondaries starting at the decay time and point of their parent."""
import numpy as np

from pentrack_gb300 import _abi as A
from pentrack_gb300 import scenes as S
from pentrack_gb300 import secondaries


def test_decay_kinematics_at_rest_and_moving():
    from scipy import stats
    n = 20000
    ids = np.arange(n)
    pp, pe, pnu = secondaries.decay_momenta(11, ids, np.zeros((3, n)))
    tot = pp + pe + pnu
    mn = S.M_N * S.C0
    np.testing.assert_allclose(tot[0], mn, rtol=1e-13)
    assert np.max(np.abs(tot[1:4])) < 1e-13 * mn
    ep = (pp[0] - S.M_P * S.C0) * S.C0
    ee = (pe[0] - S.M_E * S.C0) * S.C0
    assert np.all((ep > 0) & (ep < 751.0)) and np.all((ee > 0) & (ee < 782.5e3))
    grid = np.linspace(0, 750, 30001)
    cdf = np.cumsum(secondaries.proton_beta_spectrum(grid))
    cdf /= cdf[-1]
    assert stats.kstest(np.clip(ep, 0, 750), lambda e: np.interp(e, grid, cdf)).pvalue > 1e-3
    # a moving neutron: momenta add up to its four-momentum
    v = np.vstack([np.full(n, 3.0), np.full(n, -4.0), np.full(n, 1.0)])
    pp, pe, pnu = secondaries.decay_momenta(11, ids, v)
    tot = pp + pe + pnu
    g = 1 / np.sqrt(1 - (v ** 2).sum(0) / S.C0 ** 2)
    np.testing.assert_allclose(tot[0], g * mn, rtol=1e-13)
    np.testing.assert_allclose(tot[1:4], g * S.M_N * v, rtol=1e-6, atol=1e-13 * mn)


def test_secondaries_start_at_the_decay():
    from pentrack_gb300.engine import ParticleSet
    n = 50
    rng = np.random.default_rng(2)
    nset = ParticleSet(n, id=np.arange(100, 100 + n), t=rng.uniform(0, 1000, n), y=rng.normal(size=(9, n)))
    nset.stop_id[:] = np.where(np.arange(n) % 3 == 0, A.ID_DECAYED, A.ID_NOT_FINISH)
    p, e = secondaries.neutron_decay(4, nset)
    dec = nset.stop_id == A.ID_DECAYED
    assert p.n == e.n == dec.sum()
    assert np.array_equal(p.t, nset.t[dec]) and np.array_equal(e.y[0:3], nset.y[0:3, dec])
    assert np.array_equal(p.id & ((1 << 40) - 1), nset.id[dec]) and np.array_equal(e.id >> 41, np.ones(e.n, np.int64))
    assert np.all(np.abs(p.y[7]) == 1) and np.all(np.abs(e.y[7]) == 1)
    vp = np.sqrt((p.y[3:6] ** 2).sum(0))
    assert np.all((vp > 0) & (vp < 4e5))  # 750 eV protons: < 3.8e5 m/s
