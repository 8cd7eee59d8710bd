"""Gradients of spin observables with respect to harmonic-expansion
coefficients, for the adjoint-spin setting (a weak holding field plus
HarmonicExpansionBField terms, spins starting transverse).

The observables are the mean accumulated precession phase (spin[4], the
integral of the Larmor frequency that IntegrateSpin records,
src/tracking.cpp:373-483), the mean transverse spin component S.x and the
polarisation |<S>|.  Their gradients come from central finite differences
over complete tracking runs, one fresh scene per perturbed coefficient, with
the same particles and random streams; the error is O(h^2) plus the
tracking's own tolerance.  The adjoint (pt_adjoint, one backward pass for
all coefficients) gives the same gradients pathwise: `adjoint_gradients`
contracts it with the observables' derivatives, and `SpinTracking` wraps the
forward pass and the adjoint as a torch.autograd.Function whose input is
the coefficient vector and whose output is the end spins.
"""
import numpy as np


def observables(out):
    """mean phase, mean S.x, mean S.y and |<S>| of a tracked set"""
    s = out.spin
    return {"phase": float(np.mean(s[4])), "sx": float(np.mean(s[0])), "sy": float(np.mean(s[1])),
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


def observable_cotangents(out, name):
    """dL/d(end spin) (5, n) for L = the observable `name` of the tracked set"""
    n = out.n
    d = np.zeros((5, n))
    s = out.spin
    if name == "phase":
        d[4] = 1.0 / n
    elif name == "sx":
        d[0] = 1.0 / n
    elif name == "sy":
        d[1] = 1.0 / n
    elif name == "polarisation":
        m = np.mean(s[0:3], axis=1)
        p = np.sqrt((m ** 2).sum())
        if p > 0:
            d[0:3] = (m / p)[:, None] / n
    else:
        raise ValueError(name)
    return d


def adjoint_gradients(engine, params, particles, field=1, names=("phase", "sx", "sy", "polarisation"), checkpoint_interval=1024):
    """(observables, {name: dL/dG over the coefficients of harmonic field
    `field`}) from one forward pass and one pt_adjoint call per observable on
    the GPU (FP64 field mode)."""
    from . import _abi as A
    params.field_precision = A.PREC_FP64
    out, _ = engine.integrate(params, particles)
    base = observables(out)
    grads, stats = {}, []
    for name in names:
        g, _, st = engine.adjoint(params, particles, field, observable_cotangents(out, name),
                                  checkpoint_interval=checkpoint_interval)
        grads[name] = g
        stats.append(st)
    return base, grads, stats


def make_spin_tracking(make_scene, terms, params, particles, field=1, checkpoint_interval=1024, device=0):
    """A torch.autograd.Function over the coefficients G of harmonic field
    `field` (the (l, m) of `terms` fixed): forward tracks `particles` with
    the scene make_scene([(l, m, G_k)]) and returns the end spins (5, n);
    backward calls pt_adjoint with the incoming gradient of the end spins.
    The harness builds one Engine per distinct G vector."""
    import torch
    from . import _abi as A
    from .engine import Engine
    params.field_precision = A.PREC_FP64
    cache = {}

    def engine_for(g):
        key = tuple(float(x) for x in g)
        if key not in cache:
            cache.clear()
            cache[key] = Engine(make_scene([(l, m, gk) for (l, m, _), gk in zip(terms, key)]), device=device)
        return cache[key]

    class SpinTracking(torch.autograd.Function):
        @staticmethod
        def forward(ctx, g):
            e = engine_for(g.detach().cpu().numpy())
            out, _ = e.integrate(params, particles)
            ctx.save_for_backward(g)
            return torch.from_numpy(out.spin.copy())

        @staticmethod
        def backward(ctx, grad_spin):
            (g,) = ctx.saved_tensors
            e = engine_for(g.detach().cpu().numpy())
            dg, _, _ = e.adjoint(params, particles, field, grad_spin.detach().cpu().numpy().astype(np.float64),
                                 checkpoint_interval=checkpoint_interval)
            return torch.from_numpy(dg).to(g.dtype)

    return SpinTracking
