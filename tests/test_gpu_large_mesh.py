"""The large-mesh configuration (needs a GB300): the 200,000-triangle
noise-perturbed torus and sphere with the tricubic multipole at the
configuration's 128^3 (and at 32^3), 2,000 UCN, GPU vs oracle over 0.5 s.

Tolerances as for the field-storage physics test: the device and the oracle
evaluate the same tricubic in different exact forms, so force differences of
1e-16 grow through the step controller; >= 97 % equal stop IDs and wall-hit
totals within 2 %, median end-position difference below 1e-7 m."""
import numpy as np
import pytest

from pentrack_gb300 import _abi as A

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("table_n", [32, 128])
def test_large_mesh_short_parity(built, oracle_mod, table_n):
    from pentrack_gb300 import Engine, workloads
    sc = workloads.large_mesh_scene(table_n=table_n)
    e = Engine(sc)
    _, params, parts = workloads.large_mesh(n=2000, simtime=0.5, table_n=table_n, scene=sc, engine=e)
    oout, ost = oracle_mod.Oracle(sc).integrate(params, parts)
    params.mode = A.MODE_BATCHED
    gout, gst = e.integrate(params, parts)
    same = gout.stop_id == oout.stop_id
    assert same.mean() > 0.97
    assert ost["hits"] > 10000 and abs(gst["hits"] - ost["hits"]) <= 0.02 * ost["hits"]
    dpos = np.abs(gout.y[0:3, same] - oout.y[0:3, same]).max(0)
    assert np.median(dpos) < 1e-7
    # every particle started inside one of the two volumes
    assert np.all(gout.stop_id != A.ID_INITIAL_NOT_FOUND)
