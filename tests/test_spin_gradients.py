"""Finite-difference gradients of the spin observables (adjoint-spin
setting) with the oracle as the tracker: the phase derivative with respect
to the uniform (l, m) = (0, 0) coefficient (B_z) equals |gamma_n| times the
tracked time, since the phase integrates |gamma_n| |B| and B is along z."""
import time

import numpy as np

from pentrack_gb300 import _abi as A
from pentrack_gb300 import spin_gradients


def test_phase_gradient_of_the_holding_field(oracle_mod):
    from pentrack_gb300 import Scene, scenes, workloads

    def make_scene(coeffs):
        sc = Scene()
        sc.add_material("wall", 335.0)
        sc.add_material("vacuum", 0.0)
        sc.add_solid(1, "wall")
        sc.add_solid(2, "vacuum", scenes.cylinder_mesh(0.2, -0.06, 0.06, 64))
        sc.add_harmonic(coeffs)
        sc.add_uniform_e(0.0, 0.0, 1e6)
        return sc

    ids = np.arange(6, dtype=np.int64)
    pos, (E, ph, th, pol) = scenes.source_cylinder(1004, ids, 0.0, 0.19, -0.05, 0.05, 0.0, 200e-9, polarization=1.0)
    parts = scenes.make_particles(1004, ids, pos, E, ph, th, pol)
    parts.spin[:] = 0.0
    parts.spin[0] = 1.0
    params = workloads.run_params(A.NEUTRON, simtime=0.01, tau=0.0, tmax=9e99, lmax=9e99, bmax=1.0,
                                  spintimes=(0.0, 100.0), seed=1004)
    coeffs = [(0, 0, 1e-6), (1, 0, 2e-10), (2, 1, -1e-10)]

    def integrate(sc, p, ps):
        return oracle_mod.Oracle(sc).integrate(p, ps)[0]

    t0 = time.perf_counter()
    base, grads = spin_gradients.fd_gradients(make_scene, coeffs, params, parts, integrate=integrate, rel_step=1e-4)
    assert time.perf_counter() - t0 < 120
    out = integrate(make_scene(coeffs), params, parts)
    tmean = float(np.mean(out.t - parts.t))
    np.testing.assert_allclose(base["phase"], abs(scenes.GAMMA_N) * 1e-6 * tmean, rtol=1e-4)
    np.testing.assert_allclose(grads["phase"][0], abs(scenes.GAMMA_N) * tmean, rtol=1e-3)
    assert np.all(np.isfinite(grads["sx"])) and np.all(np.isfinite(grads["polarisation"]))
