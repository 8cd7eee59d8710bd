"""Gradients of spin observables with respect to harmonic-expansion
coefficients, for the adjoint-spin setting (a weak holding field plus
HarmonicExpansionBField terms, spins starting transverse).

The observables are the mean accumulated precession phase (spin[4], the
integral of the Larmor frequency that IntegrateSpin records,
src/tracking.cpp:373-483), the mean transverse spin component S.x and the
polarisation |<S>|.  Their gradients come from central finite differences
over complete tracking runs, one fresh scene per perturbed coefficient, with
the same particles and random streams; the error is O(h^2) plus the
tracking's own tolerance.  An adjoint of the integration (one backward pass
for all coefficients) is not built.
"""
import numpy as np


def observables(out):
    """mean phase, mean S.x and |<S>| of a tracked set"""
    s = out.spin
    return {"phase": float(np.mean(s[4])), "sx": float(np.mean(s[0])),
            "polarisation": float(np.sqrt((np.mean(s[0:3], axis=1) ** 2).sum()))}


def fd_gradients(make_scene, coeffs, params, particles, integrate=None, rel_step=1e-3, abs_step=None):
    """(observables at coeffs, {name: gradient array over the coefficients}).
    `make_scene(coeffs)` builds the scene for a list of (l, m, G);
    `integrate(scene, params, particles)` tracks (default: a new Engine on the
    scene, on the GPU).  Step h = rel_step |G| (abs_step, or rel_step, for
    G = 0)."""
    if integrate is None:
        from .engine import Engine

        def integrate(scene, p, ps):
            return Engine(scene).integrate(p, ps)[0]

    coeffs = [tuple(c) for c in coeffs]
    base = observables(integrate(make_scene(coeffs), params, particles))
    grads = {k: np.zeros(len(coeffs)) for k in base}
    for k, (l, m, g) in enumerate(coeffs):
        h = rel_step * abs(g) if g != 0 else (abs_step if abs_step is not None else rel_step)
        plus = list(coeffs)
        minus = list(coeffs)
        plus[k] = (l, m, g + h)
        minus[k] = (l, m, g - h)
        op = observables(integrate(make_scene(plus), params, particles))
        om = observables(integrate(make_scene(minus), params, particles))
        for name in base:
            grads[name][k] = (op[name] - om[name]) / (2 * h)
    return base, grads
