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


def test_cpp_endlog_writer_matches_python_byte_for_byte(built, oracle_mod, tmp_path):
    """pt_endlog_write (the C ABI's end-log writer, C++ streams at precision
    15) and logger.write_endlog write the same file, given the same fields and
    solids: the C++ writer's formatting and energies are the Python ones."""
    import ctypes as C
    from pentrack_gb300 import workloads, engine
    sc, params, parts = workloads.field_storage(n=300, simtime=0.02, table_n=16)
    orc = oracle_mod.Oracle(sc)
    out, _ = orc.integrate(params, parts)

    def fields_solids(s):
        B, _, V, _ = orc.field(np.column_stack([s.y[0], s.y[1], s.y[2], s.t]))
        idx = logger.current_solid(sc, orc.point_solids(np.ascontiguousarray(s.y[0:3].T)), s.t)
        return np.ascontiguousarray(B), np.ascontiguousarray(V), np.ascontiguousarray(idx.astype(np.int32))

    B0, V0, S0 = fields_solids(parts)
    B1, V1, S1 = fields_solids(out)
    d_py, d_cpp = tmp_path / "py", tmp_path / "cpp"
    d_py.mkdir()
    d_cpp.mkdir()
    py = logger.write_endlog(str(d_py), sc, A.NEUTRON, parts, out, orc.field, orc.point_solids, jobnumber=12)
    L = engine.lib()
    desc, keep = sc.desc()
    dp = lambda a: a.ctypes.data_as(A.c_double_p)
    ip = lambda a: a.ctypes.data_as(A.c_int32_p)
    pin, pout = parts.abi(outputs=False), out.abi()
    for logvars in (None, b"particle Hstart Hend stopID wL"):
        st = L.pt_endlog_write(str(d_cpp).encode(), 12, A.NEUTRON, C.byref(desc), C.byref(pin), C.byref(pout),
                               dp(B0), dp(V0), ip(S0), dp(B1), dp(V1), ip(S1), logvars)
        assert st == A.PT_OK, L.pt_config_error()
        if logvars is None:
            assert open(d_cpp / "000000000012neutronend.out").read() == open(py).read()
    sub = logger.write_endlog(str(d_py), sc, A.NEUTRON, parts, out, orc.field, orc.point_solids, jobnumber=12,
                              logvars=["particle", "Hstart", "Hend", "stopID", "wL"])
    assert open(d_cpp / "000000000012neutronend.out").read() == open(sub).read()
    st = L.pt_endlog_write(str(d_cpp).encode(), 12, A.NEUTRON, C.byref(desc), C.byref(pin), C.byref(pout),
                           dp(B0), dp(V0), ip(S0), dp(B1), dp(V1), ip(S1), b"Hend-Hstart")
    assert st == A.PT_ERR_UNSUPPORTED


def test_cpp_current_solid_matches_python(built):
    """pt_current_solid picks the same solid as logger.current_solid, with
    ignore times and overlapping solids of different priority."""
    import ctypes as C
    from pentrack_gb300 import Scene, engine, scenes
    sc = Scene()
    sc.add_material("a", 100.0)
    sc.add_solid(1, "a")
    sc.add_solid(5, "a", scenes.box_mesh((-1, -1, -1), (1, 1, 1)), ignore=[(2.0, 3.0)])
    sc.add_solid(3, "a", scenes.box_mesh((-2, -2, -2), (2, 2, 2)))
    sc.add_solid(7, "a", scenes.box_mesh((0, 0, 0), (1, 1, 1)), ignore=[(0.0, 1.0), (4.0, 5.0)])
    rng = np.random.default_rng(8)
    n = 5000
    masks = rng.integers(0, 16, n).astype(np.uint64) & ~np.uint64(1)
    t = rng.uniform(-1, 6, n)
    desc, keep = sc.desc()
    out = np.zeros(n, np.int32)
    st = engine.lib().pt_current_solid(C.byref(desc), n, masks.ctypes.data_as(A.c_uint64_p),
                                       t.ctypes.data_as(A.c_double_p), out.ctypes.data_as(A.c_int32_p))
    assert st == A.PT_OK
    assert np.array_equal(out, logger.current_solid(sc, masks, t))
