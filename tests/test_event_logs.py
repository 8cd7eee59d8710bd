"""Hit and snapshot logs (TLogger::PrintHit / PrintSnapshot,
src/logger.cpp:128-235) on the oracle (CPU): in the closed cube every wall
hit is a total reflection out of the vacuum solid into the default one, so
each particle has one hit record per hit (n_hit of the end state) and each
record's velocity after the hit is the specular image of the one before (to
1e-6 m/s: the mirrored velocity is the one at the far end of the final
1e-8 m bisection bracket); a
snapshot is taken at each listed time a particle is still tracked, with the
total energy of its start to 1e-5 (the end states' drift over these 4 s is
3.6e-6); the
writers produce the reference's columns."""
import os

import numpy as np
import pytest

from pentrack_gb300 import _abi as A

SNAPSHOTS = (0.75, 2.25, 3.5)
TRACK_INTERVAL = 0.5  # m


@pytest.fixture(scope="module")
def cube_logs(oracle_mod):
    from pentrack_gb300 import engine, workloads
    sc, params, parts = workloads.cube_storage(n=200, simtime=4.0)
    engine.set_logs(params, hitlog=True, snapshots=SNAPSHOTS, track_interval=TRACK_INTERVAL)
    orc = oracle_mod.Oracle(sc)
    out, st = orc.integrate(params, parts, nthreads=4)
    return sc, params, parts, out, orc.read_log(A.LOG_HIT), orc.read_log(A.LOG_SNAPSHOT), orc


def test_hit_records_match_hits(cube_logs):
    sc, params, parts, out, hits, snaps, orc = cube_logs
    assert hits.shape[1] == A.HIT_RECORD
    assert len(hits) == out.n_hit.sum() > 100
    per = np.bincount(hits[:, 0].astype(np.int64), minlength=parts.n)
    np.testing.assert_array_equal(per, out.n_hit)
    # leaving the vacuum solid (ID 2) into the default solid (ID 1), reflected specularly
    assert np.all(hits[:, 16] == 2) and np.all(hits[:, 17] == 1)
    # Reflect (src/neutron.cpp:99-115) mirrors the velocity at the far end of
    # the final bisection bracket (up to 1e-8 m on), v1 is the one at its start
    n = hits[:, 13:16]
    v1, v2 = hits[:, 5:8], hits[:, 9:12]
    np.testing.assert_allclose(v2, v1 - 2 * (v1 * n).sum(1)[:, None] * n, rtol=0, atol=1e-6)
    assert np.all(np.abs(hits[:, 2:5]) <= 0.5 + 1e-7)


def test_snapshots_at_listed_times(cube_logs, tmp_path):
    from pentrack_gb300 import logger
    sc, params, parts, out, hits, snaps, orc = cube_logs
    assert snaps.shape[1] == A.SNAPSHOT_RECORD
    for ts in SNAPSHOTS:
        alive = out.t > ts
        got = snaps[snaps[:, 1] == ts]
        assert len(got) == alive.sum()
        assert np.all(np.abs(got[:, 2:5]) <= 0.5)
    st, snap = logger.snapshot_states(parts, snaps)
    v = logger.end_variables(sc, A.NEUTRON, st, snap, orc.field, orc.point_solids)
    np.testing.assert_allclose(v["Hend"], v["Hstart"], rtol=1e-5, atol=0)  # as the end states' drift
    p = logger.write_snapshotlog(str(tmp_path), sc, A.NEUTRON, parts, snaps, orc.field, orc.point_solids, jobnumber=3)
    lines = open(p).read().splitlines()
    assert os.path.basename(p) == "000000000003neutronsnapshot.out"
    assert lines[0].split() == list(logger.END_TITLES) and len(lines) == 1 + len(snaps)
    p = logger.write_hitlog(str(tmp_path), A.NEUTRON, hits, jobnumber=3)
    lines = open(p).read().splitlines()
    assert lines[0].split() == list(logger.HIT_TITLES) and len(lines) == 1 + len(hits)
    assert float(lines[1].split()[1]) == hits[0, 0] + 1


def test_track_points(cube_logs, tmp_path):
    """one point at each particle's start and one after every step whose path
    length crossed a multiple of the interval: as many points per particle as
    multiples crossed, plus the start (a step crossing two counts once)"""
    from pentrack_gb300 import logger
    sc, params, parts, out, hits, snaps, orc = cube_logs
    tr = orc.read_log(A.LOG_TRACK)
    assert tr.shape[1] == A.TRACK_RECORD
    per = np.bincount(tr[:, 0].astype(np.int64), minlength=parts.n)
    crossed = np.floor(out.y[8] / TRACK_INTERVAL).astype(np.int64)
    assert np.all(per >= 1) and np.all(per <= crossed + 1) and np.any(per > 1)
    first = tr[np.r_[True, tr[1:, 0] != tr[:-1, 0]]]
    np.testing.assert_array_equal(first[:, 1], parts.t)
    np.testing.assert_array_equal(first[:, 2:5], parts.y[0:3].T)
    assert np.all(tr[:, 9] == 2)  # inside the vacuum cube throughout
    p = logger.write_tracklog(str(tmp_path), sc, A.NEUTRON, tr, orc.field, jobnumber=1)
    lines = open(p).read().splitlines()
    assert lines[0].split() == list(logger.TRACK_TITLES) and len(lines) == 1 + len(tr)
    H = np.array([float(l.split()[10]) for l in lines[1:]])
    H0 = dict(zip(first[:, 0].astype(np.int64), H[np.r_[True, tr[1:, 0] != tr[:-1, 0]]]))
    np.testing.assert_allclose(H, [H0[int(i)] for i in tr[:, 0]], rtol=1e-5)  # each particle keeps its energy


def test_spin_log(oracle_mod, tmp_path):
    """spin records at each Bloch integration's start and at every crossing of
    a multiple of the interval: unit spins, the precession axis |gamma_n| |B|
    (1 uT along z; the v x E and Thomas terms are below 1e-4 of it), times
    increasing per particle, at least one record per interval of tracked time"""
    from pentrack_gb300 import Scene, engine, logger, scenes, workloads
    sc = Scene()
    sc.add_material("wall", 335.0)
    sc.add_material("vacuum", 0.0)
    sc.add_solid(1, "wall")
    sc.add_solid(2, "vacuum", scenes.cylinder_mesh(0.2, -0.06, 0.06, 64))
    ax = (np.linspace(-0.25, 0.25, 6), np.linspace(-0.25, 0.25, 6), np.linspace(-0.1, 0.1, 5))
    sc.add_table3d(*ax, np.zeros((6, 6, 5)), np.zeros((6, 6, 5)), np.full((6, 6, 5), 1e-6))
    sc.add_uniform_e(0.0, 0.0, 1e6)
    ids = np.arange(8, dtype=np.int64)
    pos, (E, ph, th, pol) = scenes.source_cylinder(1004, ids, 0.0, 0.19, -0.05, 0.05, 0.0, 200e-9, polarization=1.0)
    parts = scenes.make_particles(1004, ids, pos, E, ph, th, pol)
    parts.spin[:] = 0.0
    parts.spin[0] = 1.0
    params = workloads.run_params(A.NEUTRON, simtime=0.05, tau=0.0, tmax=9e99, lmax=9e99, bmax=1.0, spintimes=(0.0, 100.0),
                                  seed=1004)
    engine.set_logs(params, spin_interval=0.002)
    orc = oracle_mod.Oracle(sc)
    out, st = orc.integrate(params, parts, nthreads=2)
    sp = orc.read_log(A.LOG_SPIN)
    assert sp.shape[1] == A.SPIN_RECORD and len(sp) >= 8 * 25
    np.testing.assert_allclose(np.sqrt((sp[:, 5:8] ** 2).sum(1)), 1.0, atol=1e-8)
    W = np.sqrt((sp[:, 8:11] ** 2).sum(1))
    B = np.sqrt((sp[:, 11:14] ** 2).sum(1))
    np.testing.assert_allclose(W, abs(scenes.GAMMA_N) * B, rtol=1e-3)
    for i in ids:
        t = sp[sp[:, 0] == i, 1]
        assert np.all(np.diff(t) >= 0) and len(t) >= 25
    p = logger.write_spinlog(str(tmp_path), A.NEUTRON, sp)
    lines = open(p).read().splitlines()
    assert lines[0].split() == list(logger.SPIN_TITLES) and len(lines) == 1 + len(sp)
