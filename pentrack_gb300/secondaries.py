"""Secondaries of neutron decay: the proton and electron TNeutron::Decay
creates at the decay point (src/neutron.cpp:285-375), for tracking as
separate proton and electron runs (the reference's `secondaries 1`,
src/main.cpp:163-172).

Per decayed neutron: the proton's kinetic energy from the recoil spectrum
ProtonBetaSpectrum (src/globals.cpp:84-92, on [0, 750] eV; sampled here by
rejection against the formula, the reference interpolates it piecewise
linearly) and its direction (azimuth uniform, polar angle from the sine
distribution on [0, pi/2], as the reference draws it) in the neutron rest
frame; the electron from the two-body decay of the remaining virtual state
(neutrino mass 1 eV/c^2), isotropic in that state's rest frame and boosted
(BOOST, src/globals.cpp:67-78); all momenta boosted with the neutron's
velocity.  Energies as the reference forms them: the proton's by the
beta^2 series, the electron's relativistically.  Polarisations are +-1 with
equal probability.  Draws come from a per-parent Philox stream apart from
the source's, so the secondaries do not depend on the batch.
"""
import numpy as np

from . import _abi as A
from . import scenes as S

_STREAM = 5000  # counter offset of the decay draws in a parent's stream


def proton_beta_spectrum(E):
    """ProtonBetaSpectrum (src/globals.cpp:84-92): relative intensity (< 1) of
    decay protons at kinetic energy E [eV]; the reference's 4/3 is integer
    division (= 1) and is kept."""
    E = np.asarray(E, dtype=np.float64)
    dm = S.M_N - S.M_P
    xi = S.M_E / dm
    sigma = 1 - 2 * E * S.M_N / dm ** 2 / S.C0 ** 2
    a = ((sigma - xi ** 2) / sigma) ** 2 * np.sqrt(1 - sigma)
    g1 = a * (4 * (1 + xi ** 2 / sigma) - 1 * ((sigma - xi ** 2) / sigma * (1 - sigma)))
    g2 = a * (4 * (1 + xi ** 2 / sigma - 2 * sigma) - 1 * ((sigma - xi ** 2) / sigma * (1 - sigma)))
    return 0.5 * (g1 + -0.1017 * g2)


def _boost(beta, p):
    """BOOST (src/globals.cpp:67-78) of four-vectors p (4, n) by velocities beta (3, n)"""
    b2 = beta[0] * beta[0] + beta[1] * beta[1] + beta[2] * beta[2]
    gamma = 1.0 / np.sqrt(1.0 - b2)
    bp = beta[0] * p[1] + beta[1] * p[2] + beta[2] * p[3]
    with np.errstate(invalid="ignore", divide="ignore"):
        gamma2 = np.where(b2 > 0, (gamma - 1.0) / np.where(b2 > 0, b2, 1.0), 0.0)
    return np.vstack([gamma * (p[0] + bp),
                      p[1] + gamma2 * bp * beta[0] + gamma * beta[0] * p[0],
                      p[2] + gamma2 * bp * beta[1] + gamma * beta[1] * p[0],
                      p[3] + gamma2 * bp * beta[2] + gamma * beta[2] * p[0]])


def decay_momenta(seed, ids, v):
    """Four-momenta [eV/c] of proton, electron and neutrino (each (4, n)) for
    neutrons with velocities v (3, n), the draws keyed by the parents' ids."""
    ids = np.asarray(ids, dtype=np.int64)
    c0 = S.C0
    m_nue = 1 / c0 ** 2

    def draw(k):
        return S.uniform(seed, ids, S.SOURCE_STREAM + np.uint64(_STREAM + k))

    ekin = S.spectrum_sampler(proton_beta_spectrum, 0.0, 750.0, first_draw=_STREAM + 100)(seed, ids)
    pp0 = ekin / c0 + S.M_P * c0
    pabs = np.sqrt(pp0 * pp0 - S.M_P * S.M_P * c0 * c0)
    b1, d1 = 2 * S.PI * draw(0), np.arccos(1.0 - draw(1))  # sin_distribution on [0, pi/2]
    pp = np.vstack([pp0, pabs * np.sin(d1) * np.cos(b1), pabs * np.sin(d1) * np.sin(b1), pabs * np.cos(d1)])
    virt = np.vstack([S.M_N * c0 - pp[0], -pp[1], -pp[2], -pp[3]])
    m2v = virt[0] * virt[0] - virt[1] * virt[1] - virt[2] * virt[2] - virt[3] * virt[3]
    pe0 = (m2v + S.M_E * S.M_E * c0 * c0 - m_nue * m_nue * c0 * c0) / 2 / np.sqrt(m2v)
    pabs = np.sqrt(pe0 * pe0 - S.M_E * S.M_E * c0 * c0)
    b2, d2 = 2 * S.PI * draw(2), np.arccos(1.0 - draw(3))
    pe = np.vstack([pe0, pabs * np.sin(d2) * np.cos(b2), pabs * np.sin(d2) * np.sin(b2), pabs * np.cos(d2)])
    pe = _boost(virt[1:4] / virt[0], pe)
    pnu = virt - pe
    beta = np.asarray(v, dtype=np.float64) / c0
    return _boost(beta, pp), _boost(beta, pe), _boost(beta, pnu)


def neutron_decay(seed, neutrons, which=None):
    """Protons and electrons (two ParticleSets) from the decayed neutrons of a
    tracked set (stop ID ID_DECAYED, or the indices `which`), starting at the
    decay time and point.  Their ids are the parent's id + 2^40 (protons) and
    + 2^41 (electrons), so that their streams differ; the parent's id is
    id & (2^40 - 1)."""
    idx = np.nonzero(neutrons.stop_id == A.ID_DECAYED)[0] if which is None else np.asarray(which)
    ids = neutrons.id[idx]
    pp, pe, _ = decay_momenta(seed, ids, neutrons.y[3:6, idx])
    c0 = S.C0
    bp2 = (pp[1] * pp[1] + pp[2] * pp[2] + pp[3] * pp[3]) / pp[0] / pp[0]
    e_p = S.M_P * c0 * c0 * bp2 * (0.5 + bp2 * (3. / 8. + bp2 * (5. / 16.)))
    e_e = pe[0] * c0 - S.M_E * c0 * c0
    out = []
    for p, e, m, species, off, k in ((pp, e_p, S.M_P, A.PROTON, 40, 4), (pe, e_e, S.M_E, A.ELECTRON, 41, 5)):
        ph = np.arctan2(p[2], p[1])
        th = np.arccos(p[3] / np.sqrt(p[1] * p[1] + p[2] * p[2] + p[3] * p[3]))
        pol = np.where(S.uniform(seed, ids, S.SOURCE_STREAM + np.uint64(_STREAM + k)) < 0.5, 1.0, -1.0)
        sid = ids + (np.int64(1) << np.int64(off))
        parts = S.make_particles(seed, sid, neutrons.y[0:3, idx], e, ph, th, pol, species=species)
        parts.t[:] = neutrons.t[idx]
        out.append(parts)
    return out[0], out[1]
