"""The adjoint-spin configuration over its full 100 s (needs a GB300): 128 UCN
of the workload (seed 1004, ids 0 .. 127; B0 = 1 uT along z plus the eight
l <= 2 harmonic terms, E = 1e6 V/m, specular walls, spins along x, Bloch
integration along every trajectory step) on the GPU against the FP64
oracle's end states of the same UCN, stored in
tests/golden/adjoint_spin_100s.npz by tests/golden/gen_spin_fixture.py.

The GPU evaluates the harmonic field from precomputed polynomials and the
oracle term by term, so the two differ by rounding from the first step, and
2,000 wall reflections per UCN carry that apart.  Criteria:
* every UCN is still stored at t = 100 s on both sides (specular walls, no
  decay), end time and spin-integration time 100 s to 1e-9 relative (the
  last step ends at T up to rounding), |S| = 1 to 1e-6;
* Bloch step totals within 0.5 % of the oracle's;
* the phase offsets phi - |gamma_n| B0 t (the harmonic terms' and the v x E
  term's share, about 1e-4 rad) and the end S_x, S_y: two-sample KS
  p > 0.01 and means within 3 standard errors; end positions and wall-hit
  counts: KS p > 0.01."""
import os

import numpy as np
import pytest

from pentrack_gb300 import _abi as A

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "adjoint_spin_100s.npz")


def test_adjoint_spin_100s_matches_oracle(built):
    stats = pytest.importorskip("scipy.stats")
    from pentrack_gb300 import Engine, scenes, workloads
    ref = np.load(FIXTURE)
    n, T = int(ref["n"]), float(ref["simtime"])
    sc, params, parts = workloads.adjoint_spin(n=n, simtime=T)
    params.mode = A.MODE_PLAIN
    params.field_precision = A.PREC_FP64
    out, st = Engine(sc).integrate(params, parts)
    bad = []  # every criterion is evaluated and reported together
    if not (np.all(out.stop_id == A.ID_NOT_FINISH) and np.all(ref["stop_id"] == A.ID_NOT_FINISH)):
        bad.append(("stop IDs", np.unique(out.stop_id)))
    for name, g, o in (("t_end", out.t, ref["t"]), ("spin time", out.spin[3], ref["spin"][3])):
        if np.max(np.abs(g - T)) > 1e-9 * T or np.max(np.abs(o - T)) > 1e-9 * T:
            bad.append((name, float(np.max(np.abs(g - T))), float(np.max(np.abs(o - T)))))
    norm = np.max(np.abs(np.sqrt((out.spin[:3] ** 2).sum(0)) - 1.0))
    if norm > 1e-6:
        bad.append(("|S| - 1", float(norm)))
    steps_ref = int(ref["spin_steps"])
    if abs(st["spin_steps"] - steps_ref) > 5e-3 * steps_ref:
        bad.append(("Bloch steps", st["spin_steps"], steps_ref))
    w0 = abs(scenes.GAMMA_N) * 1e-6
    dphi_g, dphi_o = out.spin[4] - w0 * out.t, ref["spin"][4] - w0 * ref["t"]
    for name, g, o in (("phase offset", dphi_g, dphi_o), ("S_x", out.spin[0], ref["spin"][0]),
                       ("S_y", out.spin[1], ref["spin"][1])):
        p = stats.ks_2samp(g, o).pvalue
        se = np.sqrt((g.var() + o.var()) / n)
        if p <= 0.01 or abs(g.mean() - o.mean()) > 3 * se + 1e-12:
            bad.append((name, "KS p", p, "means", g.mean(), o.mean(), "se", se))
    for name, g, o in (("x", out.y[0], ref["y"][0]), ("y", out.y[1], ref["y"][1]), ("z", out.y[2], ref["y"][2]),
                       ("hits", out.n_hit, ref["n_hit"])):
        p = stats.ks_2samp(g, o).pvalue
        if p <= 0.01:
            bad.append((name, "KS p", p))
    assert not bad, bad
