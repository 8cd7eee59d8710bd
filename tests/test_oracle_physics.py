"""Oracle-level physics checks on the reference's own known answers (CPU).

The reference's test/IntegrationTest is its only analytic known-answer test of
integrator + field + collision path: UCN fly on parabolas with
a = -g - |mu_n| dBz/dz / m_n and the landing x must equal
x0 + vx0 * t(z_end) (test/IntegrationTest/showintegrationresult.cxx:1-7).
Here it runs with the OPERA3D half only (dBz/dz = 0.5 T/m).
"""
import numpy as np

from pentrack_gb300 import _abi as A


def landing_residual(parts, out, a):
    x0, z0, vx0, vz0 = parts.y[0], parts.y[2], parts.y[3], parts.y[5]
    ze = out.y[2]
    t_hit = (-vz0 - np.sqrt(vz0 * vz0 - 2 * a * (z0 - ze))) / a
    return out.y[0] - x0 - vx0 * t_hit


def test_integration_test_known_answer_oracle(oracle_mod):
    from pentrack_gb300 import workloads
    sc, params, parts = workloads.integration_test(n=200)
    orc = oracle_mod.Oracle(sc)
    out, st = orc.integrate(params, parts, nthreads=4)
    a = workloads.integration_test_acceleration(0.5)
    assert abs(a - (-12.691)) < 1e-3
    # absorbed in the floor on the first wall contact (fast ones reach the ceiling instead)
    first = (out.n_hit == 1) & (out.stop_id == A.ID_ABSORBED_IN_MATERIAL) & (out.y[2] < 0.5)
    assert first.sum() > 100
    res = landing_residual(parts, out, a)[first]
    assert np.max(np.abs(res)) < 1e-6, np.max(np.abs(res))
    # absorbed inside the 1 mm UCNdet floor
    assert np.all(out.y[2][first] < 0) and np.all(out.y[2][first] > -0.001)


def test_cube_storage_energy_conservation_oracle(oracle_mod):
    """Specular total reflection and gravity only: total energy is conserved to
    the integrator tolerance over 5 s of storage."""
    from pentrack_gb300 import workloads
    sc, params, parts = workloads.cube_storage(n=64, simtime=5.0)
    orc = oracle_mod.Oracle(sc)
    out, st = orc.integrate(params, parts, nthreads=4)
    assert np.all(out.stop_id == A.ID_NOT_FINISH)
    assert np.allclose(out.t, 5.0)
    # H = Ekin + m g z + Fermi potential of the current solid (vacuum inside the cube)
    m = 1.0454074345680994e-08
    g = 9.80665
    c2 = 299792458.0 ** 2

    def H(y):
        v2 = (y[3:6] ** 2).sum(0)
        return 0.5 * m * v2 * (1 + 0.75 * v2 / c2) + m * g * y[2]

    dh = np.abs(H(out.y) - H(parts.y))
    assert np.max(dh) < 1e-13, np.max(dh)  # eV, i.e. < 1e-4 neV
    assert np.all(out.n_hit > 0)
    assert np.all(out.solid == 2)
