"""[SOURCE] section of a config.in (CreateParticleSource, src/source.cpp:
204-229; TParticleSource, src/source.cpp:18-84): config parsing, formula
distributions, pulsed start times, and particles from a cylindrical volume
and a cylindrical surface source."""
import numpy as np
import pytest

from pentrack_gb300 import _abi as A
from pentrack_gb300 import config_source as cs


def test_read_config_and_formulas(tmp_path):
    p = tmp_path / "c.in"
    p.write_text("[GLOBAL]\nsimtime 100 # s\n\n[SOURCE]\n  sourcemode\tcylvolume\n# comment\nEmax 3e-7\n")
    cfg = cs.read_config(str(p))
    assert cfg["GLOBAL"]["simtime"].strip() == "100" and cfg["SOURCE"]["sourcemode"].strip() == "cylvolume"
    p.write_text("[SOURCE]\nEmax 1\nEmax 2\n")
    with pytest.raises(ValueError):
        cs.read_config(str(p))
    f = cs.formula("2*x^2 - sqrt(x) + sin(pi*x)")
    x = np.linspace(0, 1, 7)
    np.testing.assert_allclose(f(x), 2 * x ** 2 - np.sqrt(x) + np.sin(np.pi * x))
    for bad in ("__import__('os')", "x.real", "x[0]", "open"):
        with pytest.raises(ValueError):
            cs.formula(bad)
    inv = cs.distribution("x^0.5", 0.0, 1.0)
    u = np.linspace(0, 1, 101)
    np.testing.assert_allclose(inv(u), u ** (2 / 3), atol=2e-3)
    np.testing.assert_allclose(cs.distribution("", 2.0, 5.0)(u), 2.0 + 3.0 * u, rtol=1e-12)
    t = cs.time_distribution(10.0, 2.0, 0.5)(np.random.default_rng(1).uniform(size=4000))
    assert np.all((t % 2.0) <= 0.5) and t.max() < 10.0 and len(np.unique(np.floor(t / 2))) == 5


def test_cylindrical_volume_and_surface_sources(tmp_path):
    from scipy import stats
    from pentrack_gb300 import workloads, logger
    p = tmp_path / "config.in"
    p.write_text("[SOURCE]\nsourcemode cylvolume\nparameters 0 0.2 0 360 -0.05 0.05\nparticle neutron\n"
                 "ActiveTime 5\npolarization 1\nEmin 0\nEmax 250e-9\nspectrum x^0.5\n"
                 "phi_v_min 0\nphi_v_max 360\nphi_v 1\ntheta_v_min 0\ntheta_v_max 180\ntheta_v sin(x)\n")
    kind, parts = cs.source_from_config(str(p), 4000, 9)
    assert kind == A.NEUTRON and parts.n == 4000
    r = np.sqrt(parts.y[0] ** 2 + parts.y[1] ** 2)
    assert np.all(r <= 0.2) and np.all(np.abs(parts.y[2]) <= 0.05) and np.all(parts.y[7] == 1)
    assert stats.kstest((r / 0.2) ** 2, "uniform").pvalue > 1e-3
    e = logger.kinetic_energy(A.NEUTRON, parts.y[3:6])
    assert np.all(e <= 250e-9 * (1 + 1e-9)) and stats.kstest((e / 250e-9) ** 1.5, "uniform").pvalue > 1e-3
    cz = parts.y[5] / np.sqrt((parts.y[3:6] ** 2).sum(0))
    assert stats.kstest(0.5 * (cz + 1), "uniform").pvalue > 1e-3
    assert np.all((parts.t >= 0) & (parts.t <= 5)) and parts.t.std() > 1
    # the same section as a surface source on the storage cube's top face
    sc, _, _ = workloads.cube_storage(n=1)
    p.write_text("[SOURCE]\nsourcemode cylsurface\nparameters 0 0.3 -180 180 0.49 0.51\nparticle neutron\n"
                 "Emin 0\nEmax 100e-9\nEnormal 10e-9\n")
    kind, parts = cs.source_from_config(str(p), 2000, 9, scene=sc)
    assert np.allclose(parts.y[2], 0.5 + 1e-8, atol=1e-15) and np.all(parts.y[5] > 0) and np.all(parts.t == 0)
    e = logger.kinetic_energy(A.NEUTRON, parts.y[3:6])
    assert np.all((e >= 10e-9 * (1 - 1e-9)) & (e <= 110e-9 * (1 + 1e-9)))
    p.write_text("[SOURCE]\nsourcemode sphere\n")
    with pytest.raises(ValueError):
        cs.source_from_config(str(p), 10, 9)


INTEGRATION_TEST_CONFIG = """[GLOBAL]
simtype 1
simcount 1000
simtime 10

[SOURCE]
sourcemode boxvolume
parameters 0.1	0.1	0.5	0.5		0.01	0.01
particle neutron
ActiveTime 0
PhaseSpaceWeighting 0
Emin 10e-9
Emax 150e-9
spectrum 1
phi_v_min 0
phi_v_max 0
phi_v 1
theta_v_min 5
theta_v_max 5
theta_v 1
polarization 1

[PARTICLES]
tau 0
endlog 1
endlogvars xstart ystart zstart xend yend zend vxstart vystart vzstart vxend vyend vzend
hitlog 0
"""


def test_reference_integration_test_source(tmp_path):
    """The source and end-log settings of the reference's integration test
    (test/IntegrationTest/config.in): every neutron starts at (0.1, 0.5, 0.01)
    with azimuth 0 and polar angle 5 degrees, 10-150 neV, polarisation +1; the
    end log is on with its twelve columns."""
    from pentrack_gb300 import logger
    p = tmp_path / "config.in"
    p.write_text(INTEGRATION_TEST_CONFIG)
    kind, parts = cs.source_from_config(str(p), 1000, 3)
    assert kind == A.NEUTRON
    assert np.all(parts.y[0] == 0.1) and np.all(parts.y[1] == 0.5) and np.all(parts.y[2] == 0.01)
    v = np.sqrt((parts.y[3:6] ** 2).sum(0))
    np.testing.assert_allclose(parts.y[5] / v, np.cos(5 * np.pi / 180), rtol=1e-12)
    assert np.all(parts.y[4] == 0) and np.all(parts.y[3] > 0) and np.all(parts.y[7] == 1) and np.all(parts.t == 0)
    e = logger.kinetic_energy(A.NEUTRON, parts.y[3:6])
    assert np.all((e > 10e-9 * (1 - 1e-9)) & (e < 150e-9 * (1 + 1e-9))) and e.std() > 30e-9
    on, names = logger.log_settings(str(p), "neutron")
    assert on and names[:3] == ["xstart", "ystart", "zstart"] and len(names) == 12
    assert logger.log_settings(str(p), "neutron", "hit") == (False, None)
