"""Sources that need the scene (TSTLVolumeSource, include/source.h:302-331;
TVolumeSource with PhaseSpaceWeighting, src/source.cpp:136-194), with the
oracle's point and field queries standing in for the engine's:
points uniform in an STL solid, start heights distributed as sqrt(H - V),
and start states independent of the batch a particle is created in."""
import numpy as np
import pytest

from pentrack_gb300 import _abi as A
from pentrack_gb300 import sources


def ks_uniform_p(u):
    from scipy import stats
    return stats.kstest(u, "uniform").pvalue


def sphere_scene(R=0.3):
    from pentrack_gb300 import Scene, scenes
    sc = Scene()
    sc.add_material("wall", 250.0)
    sc.add_material("vacuum", 0.0)
    sc.add_solid(1, "wall")
    tris = scenes.sphere_mesh(R, 24, 48)
    sc.add_solid(2, "vacuum", tris)
    return sc, tris


def test_stl_volume_points_uniform_and_batch_independent(oracle_mod):
    sc, tris = sphere_scene()
    orc = oracle_mod.Oracle(sc)
    inside = sources.solid_inside(orc.point_solids, 1)
    ids = np.arange(6000)
    p = sources.stl_volume_points(7, ids, tris, inside)
    assert np.all(inside(p.T))
    r = np.sqrt((p ** 2).sum(0))
    rmax = np.sqrt((np.asarray(tris).reshape(-1, 3) ** 2).sum(1)).max()
    assert np.all(r < rmax)
    # uniform in the (polyhedral, nearly spherical) volume: r^3 nearly uniform
    assert ks_uniform_p((r / rmax) ** 3) > 1e-3
    assert abs(np.mean(p[2])) < 0.01 and abs(np.mean(p[0])) < 0.01
    q = np.hstack([sources.stl_volume_points(7, ids[:2500], tris, inside),
                   sources.stl_volume_points(7, ids[2500:], tris, inside)])
    assert np.array_equal(p, q)


def test_phase_space_weighting_in_gravity(oracle_mod):
    """Cube storage volume without fields: V = m g z, so for a particle of
    total energy H the start height has density sqrt(H - m g z) on
    [-0.5, min(0.5, H / m g)]; its CDF at the sampled heights is uniform."""
    from pentrack_gb300 import workloads, logger
    sc, _, _ = workloads.cube_storage(n=1)
    orc = oracle_mod.Oracle(sc)
    V = sources.rest_energy_potential(sc, A.NEUTRON, orc.field, orc.point_solids)
    pts = sources.box_points((-0.4999, -0.4999, -0.4999), (0.4999, 0.4999, 0.4999))
    parts, vmin = sources.phase_space_volume_source(1001, np.arange(4000), pts, V, 0.0, 60e-9,
                                                    n_min_samples=20000)
    mg = logger.species_constants(A.NEUTRON)["mg"]
    z, ek = parts.y[2], logger.kinetic_energy(A.NEUTRON, parts.y[3:6])
    H = ek + mg * z
    assert vmin < -mg * 0.4999 + 1e-10 and vmin > -mg * 0.5
    assert np.all(ek >= 0) and np.all(H >= vmin - 1e-18) and np.all(np.abs(parts.y[0:3]) < 0.5)
    z0 = -0.4999
    zmax = np.minimum(0.4999, H / mg)
    a = np.maximum(H - mg * z0, 0) ** 1.5
    F = (a - np.maximum(H - mg * z, 0) ** 1.5) / (a - np.maximum(H - mg * zmax, 0) ** 1.5)
    assert ks_uniform_p(F) > 1e-3
    # the same particles from two batches are the same particles
    p1, _ = sources.phase_space_volume_source(1001, np.arange(300), pts, V, 0.0, 60e-9, n_min_samples=20000)
    p2, _ = sources.phase_space_volume_source(1001, np.arange(300, 600), pts, V, 0.0, 60e-9, n_min_samples=20000)
    p12, _ = sources.phase_space_volume_source(1001, np.arange(600), pts, V, 0.0, 60e-9, n_min_samples=20000)
    assert np.array_equal(np.hstack([p1.y, p2.y]), p12.y)


def test_surface_source_on_a_face():
    """TSurfaceSource on the top face of the storage cube: points on the face
    inside the source cylinder, 1e-8 m off along the outward normal, Lambert
    (cos theta sin theta) directions about it, uniform over the face, and
    the normal energy raised by Enormal."""
    from pentrack_gb300 import workloads, logger
    sc, _, _ = workloads.cube_storage(n=1)
    inside, box = sources.cylinder_region(0.0, 0.3, 0.49, 0.51)
    ids = np.arange(5000)
    p = sources.surface_source(5, ids, sc, inside, box, 0.0, 100e-9)
    assert np.allclose(p.y[2], 0.5 + 1e-8, rtol=0, atol=1e-15)
    r2 = p.y[0] ** 2 + p.y[1] ** 2
    assert np.all(r2 < 0.09)
    assert ks_uniform_p(r2 / 0.09) > 1e-3
    v = np.sqrt((p.y[3:6] ** 2).sum(0))
    cz = p.y[5] / v
    assert np.all(cz > 0) and ks_uniform_p(cz ** 2) > 1e-3
    e0 = logger.kinetic_energy(A.NEUTRON, p.y[3:6])
    q = sources.surface_source(5, ids, sc, inside, box, 0.0, 100e-9, enormal=20e-9)
    e1 = logger.kinetic_energy(A.NEUTRON, q.y[3:6])
    np.testing.assert_allclose(e1, e0 + 20e-9, rtol=1e-9)
    assert np.array_equal(q.y[0:3], p.y[0:3])
