"""Stochastic-configuration parity (needs a GB300): the field-storage physics
(diffuse walls, losses, decay, +-mu grad|B|) in the bench's FP32 field mode
and batched form against the FP64 oracle, compared as distributions.

Criterion (the reference's stochastic-config contract): two-sample
Kolmogorov-Smirnov p > 0.01 on end time, end position (x, y, z) and end
polarisation; stop-ID fractions within 3 standard errors."""
import numpy as np
import pytest

from pentrack_gb300 import _abi as A

pytestmark = pytest.mark.gpu


def test_field_storage_distributions_match_oracle(built, oracle_mod):
    stats = pytest.importorskip("scipy.stats")
    from pentrack_gb300 import Engine, workloads
    n, T = 4000, 4.0
    sc = workloads.field_storage_scene()
    e = Engine(sc)
    _, params, parts = workloads.field_storage(n=n, simtime=T, engine=e, first_id=500_000)
    oout, _ = oracle_mod.Oracle(sc).integrate(params, parts)
    params.mode = A.MODE_BATCHED
    params.field_precision = A.PREC_FP32
    gout, _ = e.integrate(params, parts)
    for name, g, o in (("t_end", gout.t, oout.t), ("x", gout.y[0], oout.y[0]), ("y", gout.y[1], oout.y[1]),
                       ("z", gout.y[2], oout.y[2]), ("pol", gout.y[7], oout.y[7])):
        p = stats.ks_2samp(g, o).pvalue
        assert p > 0.01, (name, p)
    for sid in np.union1d(np.unique(gout.stop_id), np.unique(oout.stop_id)):
        fg, fo = np.mean(gout.stop_id == sid), np.mean(oout.stop_id == sid)
        se = np.sqrt(max(fo * (1 - fo), 1.0 / n) / n)
        assert abs(fg - fo) <= 3 * np.sqrt(2) * se + 1.0 / n, (sid, fg, fo)


@pytest.mark.parametrize("species", [A.PROTON, A.ELECTRON])
def test_mixed_species_distributions_match_oracle(built, oracle_mod, species):
    """The mixed-species workload (decay protons / beta electrons in a 1 T solenoid plus a
    30 kV/m field, absorbing wall and detector): end time, end z and the
    fractions of particles absorbed in the wall and on the detector."""
    stats = pytest.importorskip("scipy.stats")
    from pentrack_gb300 import Engine, workloads
    sc, runs = workloads.mixed_species(n_protons=2000, n_electrons=2000)
    params, parts = runs[species]
    oout, _ = oracle_mod.Oracle(sc).integrate(params, parts)
    params.mode = A.MODE_BATCHED
    gout, gst = Engine(sc).integrate(params, parts)
    assert np.all(gout.stop_id == A.ID_ABSORBED_IN_MATERIAL) and np.all(oout.stop_id == A.ID_ABSORBED_IN_MATERIAL)
    for name, g, o in (("t_end", gout.t, oout.t), ("z", gout.y[2], oout.y[2])):
        p = stats.ks_2samp(g, o).pvalue
        assert p > 0.01, (name, p)
    n = len(parts.t)
    for sid in (2, 3):
        fg, fo = np.mean(gout.solid == sid), np.mean(oout.solid == sid)
        assert abs(fg - fo) <= 3 * np.sqrt(2 * max(fo * (1 - fo), 1.0 / n) / n) + 1.0 / n, (sid, fg, fo)
