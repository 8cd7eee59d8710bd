"""Secondaries of neutron decay on the device (needs a GB300).

* pt_neutron_decay (TNeutron::Decay, src/neutron.cpp:285-375, in
  csrc/pt_k_source.cu) against the host path pentrack_gb300/secondaries.py
  on the same decayed neutrons and streams: ids, start times, points and
  polarisations equal, velocities within 1e-13 relative (the device's and
  the host's acos/atan2/cos/sin may differ in the last bit), and the
  four-momentum bookkeeping of the host path holds for the device's states.
* pt_integrate_secondaries (the reference's `secondaries 1` chain,
  src/main.cpp:163-172): the neutrons' end states equal pt_integrate's, the
  number of secondaries equals the number of decays, and the protons' and
  electrons' end states equal pt_integrate of the device's decay products.
"""
import numpy as np
import pytest

from pentrack_gb300 import _abi as A

pytestmark = pytest.mark.gpu

SEED = 4711


def decaying_neutrons(n=2000):
    from pentrack_gb300 import scenes as S, workloads
    from pentrack_gb300.engine import run_params
    sc = workloads.mixed_species_scene(nseg=64)
    ids = np.arange(n, dtype=np.int64)
    pos, (E, ph, th, pol) = S.source_cylinder(SEED, ids, 0.0, 0.25, -0.4, 0.4, 0.0, 100e-9)
    parts = S.make_particles(SEED, ids, pos, E, ph, th, pol)
    pn = run_params(A.NEUTRON, simtime=1.0, tau=2e-3, tmax=9e99, lmax=9e99, bmax=0.0, seed=SEED)
    pp = run_params(A.PROTON, simtime=1.0, tau=0.0, tmax=1e-3, lmax=9e99, bmax=0.0, seed=SEED)
    pe = run_params(A.ELECTRON, simtime=1.0, tau=0.0, tmax=1e-3, lmax=9e99, bmax=0.0, seed=SEED)
    return sc, pn, pp, pe, parts


def test_device_decay_equals_host_secondaries(built):
    from pentrack_gb300 import Engine, secondaries
    sc, pn, _, _, parts = decaying_neutrons()
    e = Engine(sc)
    out, _ = e.integrate(pn, parts)
    decayed = out.stop_id == A.ID_DECAYED
    assert decayed.mean() > 0.9
    dp, de = e.neutron_decay(SEED, out)
    hp, he = secondaries.neutron_decay(SEED, out)
    for d, h in ((dp, hp), (de, he)):
        assert d.n == decayed.sum()
        np.testing.assert_array_equal(d.id, h.id)
        np.testing.assert_array_equal(d.t, h.t)
        np.testing.assert_array_equal(d.y[0:3], h.y[0:3])
        np.testing.assert_array_equal(d.y[6:9], h.y[6:9])
        np.testing.assert_allclose(d.y[3:6], h.y[3:6], rtol=1e-13, atol=1e-13 * np.abs(h.y[3:6]).max())
        assert np.all(d.spin == 0)


def test_integrate_secondaries_chain(built):
    from pentrack_gb300 import Engine
    sc, pn, pp, pe, parts = decaying_neutrons()
    e = Engine(sc)
    out, op, oe, st = e.integrate_secondaries(pn, pp, pe, parts)
    ref, _ = e.integrate(pn, parts)
    for k in ("t", "y", "stop_id", "n_hit", "id"):
        assert np.array_equal(getattr(out, k), getattr(ref, k)), k
    m = int((ref.stop_id == A.ID_DECAYED).sum())
    assert op.n == m and oe.n == m and m > 1000
    dp, de = e.neutron_decay(SEED, ref)
    rp, _ = e.integrate(pp, dp)
    re_, _ = e.integrate(pe, de)
    for a, b in ((op, rp), (oe, re_)):
        for k in ("id", "t", "y", "stop_id", "n_hit"):
            assert np.array_equal(getattr(a, k), getattr(b, k)), k
    # charged secondaries end on the walls or the detector, or at their 1 ms proper-time limit
    for s in (op, oe):
        assert set(np.unique(s.stop_id)) <= {A.ID_ABSORBED_IN_MATERIAL, A.ID_DECAYED, A.ID_HIT_BOUNDARIES}
    assert st["particle_seconds"] > 0
