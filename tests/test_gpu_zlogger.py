"""End log from a GPU run (needs a GB300): the logger's start energy, with
fields and solids from the engine's query entry points, against the start
energy the kernels computed (TParticle::GetInitialTotalEnergy,
src/particle.cpp:17-19).  Both evaluate the same formulas on the same FP64
field, so they agree to rounding (1e-12 relative)."""
import numpy as np
import pytest

from pentrack_gb300 import _abi as A
from pentrack_gb300 import logger

pytestmark = pytest.mark.gpu


def test_endlog_from_gpu_run(built, tmp_path):
    from pentrack_gb300 import Engine, workloads
    sc, params, parts = workloads.field_storage(n=2000, simtime=0.05, table_n=16)
    eng = Engine(sc)
    params.mode = A.MODE_BATCHED
    out, _ = eng.integrate(params, parts)
    v = logger.end_variables(sc, A.NEUTRON, parts, out, eng.field, eng.point_solids)
    np.testing.assert_allclose(v["Hstart"], out.h_start, rtol=1e-12, atol=0)
    # every source point is in the vacuum cylinder; a particle that entered the
    # wall material ends in the default solid (ID 1)
    assert np.all(v["solidstart"] == 2) and np.all(np.isin(v["solidend"], (1, 2)))
    path = logger.write_endlog(str(tmp_path), sc, A.NEUTRON, parts, out, eng.field, eng.point_solids, jobnumber=3)
    lines = open(path).read().splitlines()
    assert len(lines) == 2001 and lines[0].split() == list(logger.END_TITLES)
