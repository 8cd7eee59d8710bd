"""End log in the reference's text layout (TLogger::Print "end" +
TTextLogger::DoLog, src/logger.cpp:42-126, 314-334): file name, header,
column order and number format, and the start energy against the oracle's
(which follows TParticle::GetInitialTotalEnergy, src/particle.cpp:17-19)."""
import numpy as np
import pytest

from pentrack_gb300 import _abi as A
from pentrack_gb300 import logger


def two_solid_scene():
    from pentrack_gb300 import Scene, scenes
    sc = Scene()
    sc.add_material("wall", 250.0, internal_bfield=0.5)
    sc.add_material("vacuum", 0.0)
    sc.add_solid(1, "wall")
    sc.add_solid(2, "vacuum", scenes.box_mesh((-1, -1, -1), (1, 1, 1)), ignore=[(5.0, 6.0)])
    return sc


def test_endlog_layout(tmp_path):
    from pentrack_gb300.engine import ParticleSet
    sc = two_solid_scene()
    rng = np.random.default_rng(3)
    n = 4
    start = ParticleSet(n, id=np.arange(10, 10 + n), t=np.array([0.0, 1.0, 5.5, 2.0]), y=rng.normal(size=(9, n)),
                        spin=rng.normal(size=(5, n)))
    start.y[7] = [1, -1, 1, -1]
    end = start.copy()
    end.t = start.t + 3.25
    end.y = rng.normal(size=(9, n))
    end.spin[3] = [0.0, 2.0, 1.0, 0.0]
    end.stop_id[:] = [-1, -2, 1, -4]
    end.n_hit[:] = [3, 0, 7, 1]
    end.noflip_prob[:] = [1.0, 0.25, 0.5, 1.0]

    def field(q):
        B = np.column_stack([np.full(len(q), 1e-6), q[:, 0] * 1e-3, np.zeros(len(q))])
        return B, np.zeros((len(q), 3, 3)), q[:, 2] * 10.0, np.zeros((len(q), 3))

    def point_solids(p):
        return np.where(np.abs(p).max(1) < 1, np.uint64(2), np.uint64(0)).astype(np.uint64)

    path = logger.write_endlog(str(tmp_path), sc, A.NEUTRON, start, end, field, point_solids, jobnumber=7)
    assert path.endswith("000000000007neutronend.out")
    lines = open(path).read().split("\n")
    assert lines[0] == " ".join(logger.END_TITLES) + " "
    assert lines[-1] == "" and len(lines) == n + 2
    v = logger.end_variables(sc, A.NEUTRON, start, end, field, point_solids, jobnumber=7)
    for i in range(n):
        assert lines[1 + i] == "".join("%.15g " % v[t][i] for t in logger.END_TITLES)
        vals = [float(x) for x in lines[1 + i].split()]
        assert len(vals) == len(logger.END_TITLES)
    col = {t: k for k, t in enumerate(logger.END_TITLES)}
    row = [float(x) for x in lines[1].split()]
    assert row[col["particle"]] == 11 and row[col["jobnumber"]] == 7 and row[col["stopID"]] == -1
    # solids: inside the box -> ID 2 unless t in its ignore window [5, 6)
    inside = np.abs(start.y[0:3]).max(0) < 1
    expect = np.where(inside & ~((start.t >= 5) & (start.t < 6)), 2, 1)
    assert np.array_equal(v["solidstart"], expect)
    assert np.allclose(v["spinflipprob"], [0.0, 0.75, 0.5, 0.0])
    assert np.array_equal(v["wL"], np.where(end.spin[3] > 0, end.spin[4] / np.where(end.spin[3] > 0, end.spin[3], 1), 0))
    # a subset by name; formulas are refused
    p2 = logger.write_endlog(str(tmp_path), sc, A.NEUTRON, start, end, field, point_solids, jobnumber=8,
                             logvars=["particle", "Hend", "stopID"])
    assert open(p2).readline() == "particle Hend stopID \n"
    with pytest.raises(ValueError):
        logger.write_endlog(str(tmp_path), sc, A.NEUTRON, start, end, field, point_solids, logvars=["Hend-Hstart"])


def test_endlog_start_energy_matches_oracle(oracle_mod):
    from pentrack_gb300 import workloads
    sc, params, parts = workloads.field_storage(n=200, simtime=0.02, table_n=16)
    orc = oracle_mod.Oracle(sc)
    out, _ = orc.integrate(params, parts)
    v = logger.end_variables(sc, A.NEUTRON, parts, out, orc.field, orc.point_solids)
    np.testing.assert_allclose(v["Hstart"], out.h_start, rtol=1e-15, atol=0)
    assert np.all(out.h_max >= v["Hstart"] - 1e-18)
    # energy is conserved along the stored trajectories to the integrator's accuracy
    live = out.stop_id == A.ID_NOT_FINISH
    assert live.sum() > 100
    assert np.max(np.abs(v["Hend"][live] - v["Hstart"][live])) < 1e-13
