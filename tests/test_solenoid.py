"""The finite-solenoid closed form (include/pt_solenoid.h, through the
oracle): Bulirsch's cel against scipy's complete elliptic integrals, and the
field against a direct Biot-Savart integration of the sheet current.

Tolerances: cel to 1e-14 relative; B to 1e-9 of the central field (the
quadrature's accuracy); the Jacobian against finite differences of B to 1e-6
of the field scale per metre, and divergence- and curl-free to the same."""
import numpy as np
import pytest

from pentrack_gb300 import _abi as A


def _scene(a=0.5, b=1.0, bc=1.0, center=(0.01, -0.02, 0.03)):
    from pentrack_gb300 import Scene, scenes
    sc = Scene()
    sc.add_material("m", 0.0)
    sc.add_solid(1, 0)
    sc.add_solid(2, 0, scenes.box_mesh((-2, -2, -2), (2, 2, 2)))
    sc.add_solenoid(a, b, bc, center=center)
    return sc


def test_solenoid_centre_and_biot_savart(oracle_mod):
    a, b, bc = 0.5, 1.0, 1.0
    center = np.array([0.01, -0.02, 0.03])
    orc = oracle_mod.Oracle(_scene(a, b, bc, tuple(center)))
    pts = np.array([[0, 0, 0], [0.1, 0.05, 0.2], [0.3, -0.1, -0.7], [0.2, 0.2, 1.3], [0.4, 0.0, 0.9], [0.7, 0.1, 0.4]])
    B, dB, _, _ = orc.field(np.column_stack([pts + center, np.zeros(len(pts))]))
    np.testing.assert_allclose(B[0], [0, 0, bc], atol=1e-12)
    mu0nI = bc * np.sqrt(a * a + b * b) / b

    # sheet current K = n I phi_hat on rho = a, |z'| <= b: trapezoid rule in phi
    # (periodic, spectrally accurate) times Gauss-Legendre panels in z'
    nphi = 1024
    phi = 2 * np.pi * np.arange(nphi) / nphi
    gx, gw = np.polynomial.legendre.leggauss(24)
    edges = np.linspace(-b, b, 81)
    zq = np.concatenate([0.5 * (e1 - e0) * gx + 0.5 * (e1 + e0) for e0, e1 in zip(edges[:-1], edges[1:])])
    wq = np.concatenate([0.5 * (e1 - e0) * gw for e0, e1 in zip(edges[:-1], edges[1:])])
    P_, Z_ = np.meshgrid(phi, zq, indexing="ij")
    W_ = np.broadcast_to(wq, P_.shape) * (2 * np.pi / nphi) * a
    src = np.stack([a * np.cos(P_), a * np.sin(P_), Z_], -1)
    K = np.stack([-np.sin(P_), np.cos(P_), 0 * P_], -1)

    def biot_savart(p):
        r = p - src
        d3 = np.linalg.norm(r, axis=-1) ** 3
        return (np.cross(K, r) / d3[..., None] * W_[..., None]).sum((0, 1)) * mu0nI / (4 * np.pi)

    for p, Bp in zip(pts, B):
        np.testing.assert_allclose(Bp, biot_savart(p), atol=1e-9 * bc)
    # Jacobian: finite differences, divergence and curl
    h = 1e-5
    q = np.column_stack([pts + center, np.zeros(len(pts))])
    for k in range(3):
        qp, qm = q.copy(), q.copy()
        qp[:, k] += h
        qm[:, k] -= h
        fd = (orc.field(qp)[0] - orc.field(qm)[0]) / (2 * h)
        np.testing.assert_allclose(dB[:, :, k], fd, atol=1e-6 * bc)
    assert np.max(np.abs(np.trace(dB, axis1=1, axis2=2))) < 1e-6
    assert np.max(np.abs(dB - np.transpose(dB, (0, 2, 1)))) < 1e-6


@pytest.mark.gpu
def test_solenoid_field_gpu_matches_oracle(built, oracle_mod):
    from pentrack_gb300 import Engine
    sc = _scene()
    rng = np.random.default_rng(3)
    q = np.column_stack([rng.uniform(-0.45, 0.45, (2000, 2)), rng.uniform(-1.5, 1.5, 2000), np.zeros(2000)])
    q[:20, :2] = 0.0  # on the axis
    B, dB, _, _ = Engine(sc).field(q)
    Bo, dBo, _, _ = oracle_mod.Oracle(sc).field(q)
    np.testing.assert_allclose(B, Bo, rtol=0, atol=1e-13)
    np.testing.assert_allclose(dB, dBo, rtol=0, atol=1e-8)
