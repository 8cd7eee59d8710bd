"""Field storage over the full 200 s (needs a GB300): the bench's mode (batched
form, FP32 field table) against the FP64 oracle's end states of the same
10,000 UCN (seed 1002, ids 700,000 .. 709,999), stored in
tests/golden/field_storage_200s.npz by tests/golden/gen_storage_fixture.py.

Criteria (the stochastic-configuration contract): two-sample KS p > 0.01 on
end time, end position (x, y, z) and end polarisation; stop-ID fractions
within 3 standard errors of the difference; mean wall hits within 2 %; energy
drift (H_end - H_start)/(t_end - t_start) of the stored particles: median and
99th percentile of |drift| within 3x the oracle's (plus 1e-14 eV/s)."""
import os

import numpy as np
import pytest

from pentrack_gb300 import _abi as A

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "field_storage_200s.npz")


def total_energy(engine, t, y):
    from pentrack_gb300 import scenes
    m, c2 = scenes.M_N, scenes.C0 ** 2
    v2 = (y[3:6] ** 2).sum(0)
    B = engine.field(np.column_stack([y[0], y[1], y[2], t]))[0]
    return 0.5 * m * v2 * (1 + 0.75 * v2 / c2) + m * scenes.GRAV * y[2] - y[7] * (scenes.MU_N / scenes.ELE_E) * np.sqrt((B ** 2).sum(1))


def test_field_storage_200s_distributions_match_oracle(built):
    stats = pytest.importorskip("scipy.stats")
    from pentrack_gb300 import Engine, workloads
    ref = np.load(FIXTURE)
    n, first = int(ref["n"]), int(ref["first_id"])
    sc, params, parts = workloads.field_storage(n=n, simtime=float(ref["simtime"]), first_id=first)
    e = Engine(sc)
    params.mode = A.MODE_BATCHED
    params.field_precision = A.PREC_FP32
    out, st = e.integrate(params, parts)
    assert st["active"] == 0
    for name, g, o in (("t_end", out.t, ref["t"]), ("x", out.y[0], ref["x"]), ("y", out.y[1], ref["y"]),
                       ("z", out.y[2], ref["z"]), ("pol", out.y[7], ref["pol"])):
        p = stats.ks_2samp(g, o).pvalue
        assert p > 0.01, (name, p)
    sids = ref["stop_id"].astype(np.int32)
    for sid in np.union1d(np.unique(out.stop_id), np.unique(sids)):
        fg, fo = np.mean(out.stop_id == sid), np.mean(sids == sid)
        se = np.sqrt(2 * max(fo * (1 - fo), 1.0 / n) / n)
        assert abs(fg - fo) <= 3 * se + 1.0 / n, (sid, fg, fo)
    assert np.mean(sids == A.ID_ABSORBED_ON_SURFACE) > 0.05  # the walls' loss per bounce acts
    assert abs(out.n_hit.mean() - ref["n_hit"].mean()) <= 0.02 * ref["n_hit"].mean()
    live = (out.stop_id == A.ID_NOT_FINISH)
    drift = np.abs(total_energy(e, out.t, out.y) - total_energy(e, parts.t, parts.y)) / np.maximum(out.t - parts.t, 1e-30)
    od = np.abs(ref["drift"][sids == A.ID_NOT_FINISH])
    gd = drift[live]
    for q in (50, 99):
        g, o = np.percentile(gd, q), np.percentile(od, q)
        assert g <= 3 * o + 1e-14, (q, g, o)
