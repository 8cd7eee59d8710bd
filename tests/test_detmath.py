"""The step adjuster's deterministic power function (include/pt_detmath.h),
shared by the kernels and the oracle, against the library pow on the host.

odeint's default_step_adjuster scales a rejected step by
max(0.9 err^(-1/3), 0.2) and a step with err < 0.5 by 0.9 max(err, 5^-5)^(-1/5),
so the result matters for err in [5^-5, (0.9/0.2)^3 = 91.125]: there the
relative error must stay below 1e-15; over [1e-300, 1e300] below 1e-13."""
import math

import numpy as np
import pytest


@pytest.mark.parametrize("p", [-1.0 / 3.0, -1.0 / 5.0])
@pytest.mark.parametrize("lo,hi,tol", [(5.0 ** -5, 91.125, 1e-15), (1e-300, 1e300, 1e-13)])
def test_detpow_matches_library_pow(built, oracle_mod, p, lo, hi, tol):
    L = oracle_mod.lib()
    rng = np.random.default_rng(17)
    xs = np.exp(rng.uniform(math.log(lo), math.log(hi), 20000))
    xs[:4] = (lo, hi, 0.5, 1.0)
    worst = max(abs(L.pto_detpow(float(x), p) - math.pow(x, p)) / math.pow(x, p) for x in xs)
    assert worst < tol, worst


def test_detpow_exact_cases(built, oracle_mod):
    L = oracle_mod.lib()
    assert L.pto_detpow(1.0, -0.2) == 1.0
    assert abs(L.pto_detpow(5.0 ** -5, -0.2) - 5.0) <= 4.5e-16 * 5.0
    assert abs(L.pto_detpow(8.0, -1.0 / 3.0) - 0.5) <= 2.3e-16
