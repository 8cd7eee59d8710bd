"""Particle sources that need the scene: STL-volume points and phase-space
weighted volume sources.

TSTLVolumeSource (include/source.h:302-331) draws points uniformly in an STL
solid (TTriangleMesh::RandomPointInVolume, include/trianglemesh.h:241-265:
uniform in the bounding box, kept when inside); TVolumeSource::CreateParticle (src/source.cpp:159-194)
with PhaseSpaceWeighting draws a total energy H from the spectrum (redrawn
below the minimum potential of the volume, found from 100,000 points,
src/source.cpp:136-156), then start points until one with potential V <= H is
accepted with probability sqrt(H - V) / sqrt(H - Vmin), and starts the
particle there with kinetic energy H - V.

The batch form proposes one point per pending particle per round and
evaluates the rounds' points together through the engine's query entry points
(`point_solids` for the inside test, `field` for the potential), so the
geometry and field work runs on the GPU; each particle draws from its own
Philox stream (keyed by the seed and its id, one counter per draw), so its
start state does not depend on the batch it is created in.
"""
import numpy as np

from . import _abi as A
from . import logger
from . import scenes as S

# counter offsets of the source draws within a particle's stream (the
# kinematics helpers of scenes.py use counters below 2000)
_ROUND_STRIDE = 16
_VOL_BASE = 2000        # STL-volume points: 3 coordinates per round
_H_BASE = 1 << 20       # total-energy rounds
_PS_BASE = 1 << 22      # phase-space rounds: time, polarisation, acceptance
_SPEC_BASE = 1 << 60    # spectrum redraws of the total-energy rounds ...
_SPEC_STRIDE = 1 << 12  # ... each round's draws in its own counter block


def _point_base(r):
    """first counter of the volume point drawn in phase-space round r"""
    return (r + 1) << 24


def stl_volume_points(seed, ids, triangles, inside, base=_VOL_BASE, max_rounds=10000):
    """Points uniform in the closed STL solid `triangles` (n, 9): uniform in its
    bounding box, kept when `inside(points)` (n, 3) -> bool says so.  Returns
    (3, len(ids))."""
    ids = np.asarray(ids, dtype=np.int64)
    tri = np.asarray(triangles, dtype=np.float64).reshape(-1, 3, 3)
    lo, hi = tri.min(axis=(0, 1)), tri.max(axis=(0, 1))
    pos = np.full((3, len(ids)), np.nan)
    todo = np.arange(len(ids))
    for r in range(max_rounds):
        if len(todo) == 0:
            return pos
        k = base + r * _ROUND_STRIDE
        p = np.vstack([lo[a] + S._draw(seed, ids[todo], k + a) * (hi[a] - lo[a]) for a in range(3)])
        ok = np.asarray(inside(np.ascontiguousarray(p.T)), dtype=bool)
        pos[:, todo[ok]] = p[:, ok]
        todo = todo[~ok]
    raise RuntimeError(f"no point inside the source volume for {len(todo)} particles after {max_rounds} rounds")


def stl_points(triangles, inside):
    """random_point for phase_space_volume_source: TSTLVolumeSource"""
    return lambda seed, ids, base: stl_volume_points(seed, ids, triangles, inside, base=base)


def cylinder_points(rmin, rmax, zmin, zmax, phimin=0.0, phimax=2 * S.PI):
    """random_point: TCylindricalVolumeSource (include/source.h:219-251), r from
    the linear distribution, azimuth and z uniform"""
    def f(seed, ids, base):
        r = np.sqrt(S._draw(seed, ids, base) * (rmax * rmax - rmin * rmin) + rmin * rmin)
        ph = phimin + S._draw(seed, ids, base + 1) * (phimax - phimin)
        z = zmin + S._draw(seed, ids, base + 2) * (zmax - zmin)
        return np.vstack([r * np.cos(ph), r * np.sin(ph), z])
    return f


def box_points(lo, hi):
    """random_point: TCuboidVolumeSource (include/source.h:186-216)"""
    def f(seed, ids, base):
        return np.vstack([lo[a] + S._draw(seed, ids, base + a) * (hi[a] - lo[a]) for a in range(3)])
    return f


def solid_inside(point_solids, solid_index):
    """The inside test of one scene solid from Engine.point_solids."""
    bit = np.uint64(1) << np.uint64(solid_index)
    return lambda p: (np.asarray(point_solids(p), dtype=np.uint64) & bit) != 0


def rest_energy_potential(scene, kind, field, point_solids):
    """V(t, pos (3, n), pol): the total energy of a particle at rest there
    (TParticle::GetInitialTotalEnergy with Ekin = 0)."""
    def V(t, pos, pol):
        n = pos.shape[1]
        y = np.zeros((9, n))
        y[0:3] = pos
        y[7] = pol
        B, _, U, _ = field(np.column_stack([pos[0], pos[1], pos[2], t]))
        sidx = logger.current_solid(scene, point_solids(np.ascontiguousarray(pos.T)), t)
        return logger.potential_energy(scene, kind, y, B, U, sidx)
    return V


def phase_space_volume_source(seed, ids, random_point, potential, emin, emax, spectrum=None, polarization=0.0,
                              t_range=(0.0, 0.0), theta=(0.0, S.PI), phi=(0.0, 2 * S.PI), species=A.NEUTRON,
                              n_min_samples=100_000, max_rounds=100_000, direction=None, times=None):
    """TVolumeSource with PhaseSpaceWeighting.  `random_point(seed, ids, base)`
    gives points (3, n) in the source volume from draws at counter `base` on,
    `potential(t, pos, pol)` the potential energy there (rest_energy_potential),
    `spectrum(seed, ids, counter)` total energies from draws at `counter` on
    (default uniform on [emin, emax]; round r redraws at _SPEC_BASE +
    r _SPEC_STRIDE, keeping the particle's own id and stream);
    `direction(seed, ids)` -> (phi, theta) and `times(seed, ids, counter)`
    replace the default uniform azimuth, sine-distributed polar angle and
    uniform start time on t_range.  Returns (ParticleSet, Vmin)."""
    ids = np.asarray(ids, dtype=np.int64)
    n = len(ids)
    time_of = times

    def times(sel_ids, k):
        if time_of is not None:
            return time_of(seed, sel_ids, k)
        return t_range[0] + S._draw(seed, sel_ids, k) * (t_range[1] - t_range[0])

    def pols(sel_ids, k):
        return np.where(S._draw(seed, sel_ids, k) < 0.5 * (polarization + 1), 1.0, -1.0)

    # FindPotentialMinimum: a fixed set of sample points, keyed apart from the particles
    probe = (np.int64(1) << np.int64(62)) + np.arange(n_min_samples, dtype=np.int64)
    vmin = float(np.min(potential(times(probe, _PS_BASE + 1), random_point(seed, probe, _point_base(0)),
                                  pols(probe, _PS_BASE + 2))))
    if vmin > emax:
        raise ValueError(f"the spectrum is below the minimal potential energy in the source volume ({emax} eV < {vmin} eV)")
    # total energies above the minimum potential
    H = np.full(n, np.nan)
    todo = np.arange(n)
    for r in range(max_rounds):
        if len(todo) == 0:
            break
        k = _H_BASE + r * _ROUND_STRIDE
        if spectrum is None:
            h = emin + S._draw(seed, ids[todo], k) * (emax - emin)
        else:
            h = spectrum(seed, ids[todo], _SPEC_BASE + r * _SPEC_STRIDE)
        ok = h >= vmin
        H[todo[ok]] = h[ok]
        todo = todo[~ok]
    if len(todo):
        raise RuntimeError(f"no total energy above the minimal potential for {len(todo)} particles")
    # start points accepted with probability sqrt(H - V) / sqrt(H - Vmin)
    pos, t0, pol, ekin = np.full((3, n), np.nan), np.zeros(n), np.zeros(n), np.zeros(n)
    todo = np.arange(n)
    for r in range(max_rounds):
        if len(todo) == 0:
            break
        k = _PS_BASE + (r + 1) * _ROUND_STRIDE
        sid = ids[todo]
        tt, pl = times(sid, k + 1), pols(sid, k + 2)
        p = random_point(seed, sid, _point_base(r + 1))
        v = potential(tt, p, pl)
        u = S._draw(seed, sid, k + 3) * np.sqrt(H[todo] - vmin)
        with np.errstate(invalid="ignore"):
            ok = (H[todo] >= v) & (np.sqrt(H[todo] - v) > u)
        sel = todo[ok]
        pos[:, sel], t0[sel], pol[sel], ekin[sel] = p[:, ok], tt[ok], pl[ok], (H[todo] - v)[ok]
        todo = todo[~ok]
    if len(todo):
        raise RuntimeError(f"no accepted start point for {len(todo)} particles after {max_rounds} rounds")
    if direction is not None:
        ph, th = direction(seed, ids)
    else:
        ph = phi[0] + S._draw(seed, ids, 5) * (phi[1] - phi[0])
        u = S._draw(seed, ids, 6)
        th = np.arccos(np.cos(theta[0]) - u * (np.cos(theta[0]) - np.cos(theta[1])))
    parts = S.make_particles(seed, ids, pos, ekin, ph, th, pol, species=species)
    parts.t[:] = t0
    return parts, vmin


_SURF_BASE = 3000        # surface points: triangle, two barycentric draws per round
REFLECT_TOLERANCE = 1e-8  # include/trianglemesh.h:39


def cylinder_region(rmin, rmax, zmin, zmax, phimin=-S.PI, phimax=S.PI):
    """InSourceVolume of TCylindricalSurfaceSource (include/source.h:279-283)
    and its bounding box (include/source.h:272-274)"""
    def inside(p):
        r = np.sqrt(p[:, 0] * p[:, 0] + p[:, 1] * p[:, 1])
        ph = np.arctan2(p[:, 1], p[:, 0])
        return (r > rmin) & (r < rmax) & (ph > phimin) & (ph < phimax) & (p[:, 2] > zmin) & (p[:, 2] < zmax)
    return inside, ((-rmax, -rmax, zmin), (rmax, rmax, zmax))


def surface_source(seed, ids, scene, in_volume, bbox, emin, emax, enormal=0.0, polarization=0.0, t_range=(0.0, 0.0),
                   spectrum=None, species=A.NEUTRON, max_rounds=100_000):
    """TSurfaceSource::CreateParticle (src/source.cpp:102-131): a point on the
    scene's surfaces (TTriangleMesh::RandomPointOnSurface,
    include/trianglemesh.h:210-232: a solid's mesh by area among those whose
    bounding box meets the source box, a triangle by area, a uniform point on
    it) redrawn until `in_volume(points)` holds, moved off the surface by
    REFLECT_TOLERANCE along the unit face normal; a cos(theta) sin(theta)
    direction about that normal, the normal energy raised by `enormal`.
    `bbox` = ((xmin, ymin, zmin), (xmax, ymax, zmax)) of the source region."""
    ids = np.asarray(ids, dtype=np.int64)
    n = len(ids)
    lo, hi = np.asarray(bbox[0], np.float64), np.asarray(bbox[1], np.float64)
    tris, weights = [], []
    for block, solid in scene.tri_blocks:
        t = np.asarray(block, np.float64).reshape(-1, 3, 3)
        mlo, mhi = t.min(axis=(0, 1)), t.max(axis=(0, 1))
        if np.any(mhi < lo) or np.any(mlo > hi):
            continue  # the reference redraws meshes whose box misses the source box
        tris.append(t)
        weights.append(0.5 * np.sqrt((np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0]) ** 2).sum(1)))
    if not tris:
        raise ValueError("no surface of the scene meets the source region")
    tris, weights = np.concatenate(tris), np.concatenate(weights)
    cum = np.cumsum(weights)
    pos, nrm = np.full((3, n), np.nan), np.full((3, n), np.nan)
    todo = np.arange(n)
    for r in range(max_rounds):
        if len(todo) == 0:
            break
        k = _SURF_BASE + r * _ROUND_STRIDE
        sid = ids[todo]
        j = np.minimum(np.searchsorted(cum, S._draw(seed, sid, k) * cum[-1], side="right"), len(cum) - 1)
        a, b = S._draw(seed, sid, k + 1), S._draw(seed, sid, k + 2)
        flip = a + b > 1
        a, b = np.where(flip, 1 - a, a), np.where(flip, 1 - b, b)
        t = tris[j]
        p = t[:, 0] + a[:, None] * (t[:, 1] - t[:, 0]) + b[:, None] * (t[:, 2] - t[:, 0])
        ok = np.asarray(in_volume(p), dtype=bool)
        nv = np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0])
        nv /= np.sqrt((nv ** 2).sum(1))[:, None]
        sel = todo[ok]
        pos[:, sel], nrm[:, sel] = p[ok].T, nv[ok].T
        todo = todo[~ok]
    if len(todo):
        raise RuntimeError(f"no surface point in the source region for {len(todo)} particles")
    pos = pos + nrm * REFLECT_TOLERANCE
    if spectrum is None:
        E = emin + S._draw(seed, ids, 4) * (emax - emin)
    else:
        E = spectrum(seed, ids)
    ph = 2.0 * S.PI * S._draw(seed, ids, 5)
    th = np.arccos(np.sqrt(1.0 - S._draw(seed, ids, 6)))  # sincos_distribution(0, pi/2), include/mc.h:163-175
    if enormal > 0:
        vn = np.sqrt(E * np.cos(th) * np.cos(th) + enormal)
        vt = np.sqrt(E) * np.sin(th)
        th = np.arctan2(vt, vn)
        E = vn * vn + vt * vt
    v = np.vstack([np.cos(ph) * np.sin(th), np.sin(ph) * np.sin(th), np.cos(th)])
    v = S.rotate_vector(v, nrm)
    ph, th = np.arctan2(v[1], v[0]), np.arccos(np.clip(v[2], -1.0, 1.0))
    pol = np.where(S._draw(seed, ids, 3) < 0.5 * (polarization + 1), 1.0, -1.0)
    parts = S.make_particles(seed, ids, pos, E, ph, th, pol, species=species)
    parts.t[:] = t_range[0] + S._draw(seed, ids, 7) * (t_range[1] - t_range[0])
    return parts
