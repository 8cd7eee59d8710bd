"""The benchmark workloads as synthetic scenes (seeded; no external data).

cube_storage        closed 1 m cube (12 triangles) centred at the origin, gravity
                    only, 335 neV walls, 10,000 UCN, 0-200 neV, 100 s
field_storage       closed cylinder R = 0.2 m, z in [-0.05, 0.05] m, 256 segments
                    (1,024 triangles), 64^3 OPERA3D-style table of the quadrupole
                    B = (7.5 y, 7.5 x, 1e-5) T padded by one cell, 250 neV walls with
                    5 % Lambert and 1e-4 loss per bounce (surface columns on the
                    cylinder's vacuum material, where the reference's OnHit reads
                    them), tau = 880 s, 0-250 neV, 50/50 spin states, 200 s
integration_test    the reference's test/IntegrationTest: OPERA3D and (full=True)
                    OPERA2D linear-gradient tables of dBz/dz = 0.5 T/m each in a
                    hollow unit cube
adjoint_spin        closed cylinder R = 0.2 m, z in [-0.06, 0.06] m, 512 segments
                    (2,048 triangles), B0 = 1 uT along z plus 8 harmonic terms
                    (l <= 2, G ~ N(0, (1e-10 T/m^l)^2)), E = 1e6 V/m along z,
                    specular 335 neV walls, 0-200 neV UCN with spins along x,
                    100 s of Bloch integration
"""
import numpy as np

from . import _abi as A
from . import scenes as S
from .engine import Scene, run_params


def cube_storage(n=10000, seed=1001, simtime=100.0):
    sc = Scene()
    sc.add_material("default", 335.0)
    sc.add_material("vacuum", 0.0)
    sc.add_solid(1, "default")
    sc.add_solid(2, "vacuum", S.box_mesh((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5)))
    ids = np.arange(n, dtype=np.int64)
    pos, (E, ph, th, pol) = S.source_box(seed, ids, (-0.5, -0.5, -0.5), (0.5, 0.5, 0.5), 0.0, 200e-9, polarization=1.0)
    parts = S.make_particles(seed, ids, pos, E, ph, th, pol)
    params = run_params(A.NEUTRON, simtime=simtime, tau=0.0, tmax=9e99, lmax=9e99, bmax=0.1, spintimes=(0, 0), seed=seed)
    return sc, params, parts


def fenced_cube(n=2000, seed=1001, simtime=100.0):
    """The closed unit cube of `cube_storage` with a free-standing block
    (x in [-0.05, 0.05], y in [-0.3, 0.3], z in [-0.45, -0.2]) of the wall
    material inside it.  Particles start on one side of the block; those
    that fly over its edges make chords that cut a corner of the block while
    neither half-chord does, which exercises the dead ends of the bisection
    search (TTracker::iterate_collision returning false)."""
    sc = Scene()
    sc.add_material("default", 335.0)
    sc.add_material("vacuum", 0.0)
    sc.add_solid(1, "default")
    sc.add_solid(2, "vacuum", S.box_mesh((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5)))
    sc.add_solid(3, "default", S.box_mesh((-0.05, -0.3, -0.45), (0.05, 0.3, -0.2)))
    ids = np.arange(n, dtype=np.int64)
    pos, (E, ph, th, pol) = S.source_box(seed, ids, (-0.5, -0.5, -0.1), (-0.1, 0.5, 0.5), 0.0, 200e-9, polarization=1.0)
    parts = S.make_particles(seed, ids, pos, E, ph, th, pol)
    params = run_params(A.NEUTRON, simtime=simtime, tau=0.0, tmax=9e99, lmax=9e99, bmax=0.1, spintimes=(0, 0), seed=seed)
    return sc, params, parts


def quadrupole_table(n=64, r=0.2, h=0.1, grad=7.5, b0=1e-5):
    """Grid of n points per axis over the cylinder's box padded by one cell on
    each side (the reference zeroes B outside a table), sampled from
    B = (grad*y, grad*x, b0): |B_perp| = grad*r."""
    cx = 2 * r / (n - 3)
    cz = h / (n - 3)
    x = -r - cx + cx * np.arange(n)
    z = -h / 2 - cz + cz * np.arange(n)
    X, Y, Z = np.meshgrid(x, x, z, indexing="ij")
    return (x, x.copy(), z), (grad * Y, grad * X, np.full_like(X, b0))


def storage_vacuum(diff_prob, loss_per_bounce):
    """The material of a vacuum solid whose surface is a storage wall.  The
    reference applies the surface columns (diffuse probability, loss per
    bounce, spin flip) of the solid whose surface is hit (TNeutron::OnHit,
    src/neutron.cpp:192): a particle inside the vacuum solid hits that
    solid's own surface, so the wall's surface properties sit on the vacuum
    material while the default medium supplies the Fermi potential step."""
    return ("vacuum", 0.0, 0.0, diff_prob, 0.0, 0.0, 0.0, 0.0, 0.0, loss_per_bounce)


def field_storage_scene(table_n=64, nseg=256):
    sc = Scene()
    sc.add_material("wall", 250.0, 0.0, 0.05, 0.0, 0.0, 0.0, 0.0, 0.0, 1e-4)
    sc.add_material(*storage_vacuum(0.05, 1e-4))
    sc.add_solid(1, "wall")
    sc.add_solid(2, "vacuum", S.cylinder_mesh(0.2, -0.05, 0.05, nseg))
    (x, y, z), (bx, by, bz) = quadrupole_table(table_n)
    sc.add_table3d(x, y, z, bx, by, bz)
    return sc


def field_storage(n=1_000_000, seed=1002, simtime=200.0, table_n=64, engine=None, first_id=0):
    """Scene, run parameters and initial particles.  `engine` (an Engine on the
    same scene) supplies B at the start points for the initial spin."""
    sc = field_storage_scene(table_n)
    ids = np.arange(first_id, first_id + n, dtype=np.int64)
    pos, (E, ph, th, pol) = S.source_cylinder(seed, ids, 0.0, 0.2, -0.05, 0.05, 0.0, 250e-9, polarization=0.0)
    bf = None
    if engine is not None:
        def bf(p):
            q = np.column_stack([p, np.zeros(len(p))])
            return engine.field(q)[0]
    parts = S.make_particles(seed, ids, pos, E, ph, th, pol, spinprojection=0.0, bfield=bf)
    params = run_params(A.NEUTRON, simtime=simtime, tau=880.0, tmax=9e99, lmax=9e99, bmax=0.1, spintimes=(0, 0),
                        seed=seed)
    return sc, params, parts


def hollow_cube_mesh():
    """test/HollowUnitCube.STL: outer box [-0.001, 1.001]^3 and inner box [0, 1]^3
    whose triangles face into the hollow (24 triangles)."""
    outer = S.box_mesh((-0.001, -0.001, -0.001), (1.001, 1.001, 1.001))
    inner = S.box_mesh((0.0, 0.0, 0.0), (1.0, 1.0, 1.0))
    inner = inner.reshape(-1, 3, 3)[:, [0, 2, 1], :].reshape(-1, 9)  # reversed winding
    return np.vstack([outer, inner])


def integration_test(n=1000, seed=7, mesh=None, table=None, full=False):
    """test/IntegrationTest/config.in: the OPERA3D gradient table (dBz/dz =
    0.5 T/m after the 5e-5 scale and cm->m conversion) and, with full=True,
    the OPERA2D one of the same gradient listed before it (1 T/m in total).
    Particles start at (0.1, 0.5, 0.01) with theta_v = 5 deg, E in [10, 150]
    neV, pol +1, inside the hollow of a UCNdet-walled cube."""
    sc = Scene()
    sc.add_material("default", 0.0)
    sc.add_material("UCNdet", 0.1, 1.0)
    sc.add_solid(1, "default")
    sc.add_solid(2, "UCNdet", hollow_cube_mesh() if mesh is None else mesh)
    if full:
        # VerticalLinearGradientField2D.tab: 11 x 11 (r, z) grid 0..100 cm, RBX = 0, RBZ = RV = 100*z[cm]
        r2 = np.linspace(0.0, 1.0, 11)
        R2, Z2 = np.meshgrid(r2, r2, indexing="ij")
        sc.add_table2d(r2, r2.copy(), br=np.zeros_like(Z2), bz=10000.0 * Z2, v=10000.0 * Z2, b_scale=0.00005,
                       e_scale=0.0)
    if table is None:
        # VerticalLinearGradientField3D.tab: 6x6x6 grid 0..100 cm, BZ = 100*z[cm] Gauss units before the 5e-5 scale
        ax = np.linspace(0.0, 1.0, 6)
        X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
        table = ((ax, ax.copy(), ax.copy()), (np.zeros_like(Z), np.zeros_like(Z), 10000.0 * Z))
    (x, y, z), (bx, by, bz) = table
    sc.add_table3d(x, y, z, bx, by, bz, b_scale=0.00005, e_scale=0.0)
    ids = np.arange(n, dtype=np.int64)
    pos, (E, ph, th, pol) = S.source_box(seed, ids, (0.1, 0.5, 0.01), (0.1, 0.5, 0.01), 10e-9, 150e-9,
                                         theta=(5 * S.PI / 180, 5 * S.PI / 180), phi=(0.0, 0.0), polarization=1.0)
    parts = S.make_particles(seed, ids, pos, E, ph, th, pol)
    params = run_params(A.NEUTRON, simtime=10.0, tau=0.0, tmax=9e99, lmax=9e99, bmax=0.1, spintimes=(0, 0), seed=seed)
    return sc, params, parts


def integration_test_acceleration(grad=0.5):
    """a = -g - |mu_n| dBz/dz / m_n, the analytic answer the reference's
    showintegrationresult.cxx checks (-15.5754762729 m/s^2 for 1 T/m)."""
    return -S.GRAV - abs(S.MU_N) * grad / (S.M_N * S.ELE_E)


def mixed_species_scene(nseg=160):
    """The mixed-species scene: a cylinder R = 0.3 m, z in
    [-0.5, 0.5] whose wall is a closed 1 cm shell (solid 2) with a detector
    disc at the top (solid 3, z in [0.495, 0.4999]); particles move in the
    default medium (solid 1) and charged OnStep absorbs them as soon as they
    are in a solid with ID > 1 (src/proton.cpp:25-33).  Fields: a 1 T finite
    solenoid (radius 0.5 m, length 2 m) and E = (0, 0, 3e4 V/m) with the
    reference's V = Ez z.  3 x 4 x nseg triangles (1,920 for nseg = 160)."""
    sc = Scene()
    sc.add_material("vacuum", 0.0)
    sc.add_material("wall", 0.0)
    sc.add_material("detector", 0.0)
    sc.add_solid(1, "vacuum")
    outer = S.cylinder_mesh(0.31, -0.51, 0.51, nseg)
    inner = S.cylinder_mesh(0.3, -0.5, 0.5, nseg).reshape(-1, 3, 3)[:, [0, 2, 1], :].reshape(-1, 9)  # facing inwards
    sc.add_solid(2, "wall", np.vstack([outer, inner]))
    sc.add_solid(3, "detector", S.cylinder_mesh(0.299, 0.495, 0.4999, nseg))
    sc.add_solenoid(0.5, 1.0, 1.0)
    sc.add_uniform_e(0.0, 0.0, 3e4)
    return sc


def mixed_species(n_protons=100_000, n_electrons=100_000, seed=1003, tmax=1e-3):
    """The mixed-species workload: decay protons (E ~ U[0, 750] eV) and electrons (beta
    spectrum on [0, 782] keV), isotropic, uniform in the cylinder; tracked up
    to 1 ms proper time (tmax, which the reference reports as ID_DECAYED).
    Returns the scene and per-species (params, particles) pairs; the species
    run as two calls (the C ABI takes one species per run).  Polarisation 0:
    no magnetic-moment force on the charged particles."""
    sc = mixed_species_scene()
    out = {}
    spec_e = S.spectrum_sampler(S.electron_beta_spectrum, 0.0, 782e3)
    first = 0
    for species, n, emax, spec in ((A.PROTON, n_protons, 750.0, None), (A.ELECTRON, n_electrons, 782e3, spec_e)):
        ids = np.arange(first, first + n, dtype=np.int64)
        first += n
        pos, (E, ph, th, pol) = S.source_cylinder(seed, ids, 0.0, 0.3, -0.5, 0.5, 0.0, emax, polarization=0.0, spectrum=spec)
        parts = S.make_particles(seed, ids, pos, E, ph, th, np.zeros(n), species=species)
        params = run_params(species, simtime=1.0, tau=0.0, tmax=tmax, lmax=9e99, bmax=0.0, spintimes=(), seed=seed)
        out[species] = (params, parts)
    return sc, out


def harmonic_terms_l2(seed=1004, n_terms=8, sigma=1e-10):
    """Eight (l, m) slots of the fifteen with l <= 2, picked deterministically
    from the seed, with coefficients G ~ N(0, (sigma T/m^l)^2)."""
    slots = [(l, m) for l in range(3) for m in range(-l - 1, l + 2)]
    rng = np.random.default_rng(seed)
    pick = sorted(rng.choice(len(slots), n_terms, replace=False))
    return [(slots[k][0], slots[k][1], float(rng.normal(0.0, sigma))) for k in pick]


def adjoint_spin_scene(nseg=512, terms=None, b0=1e-6, ez=1e6):
    """The adjoint-spin scene: closed cylinder R = 0.2 m, z in [-0.06, 0.06]
    (nseg azimuthal segments, 4 nseg triangles), 335 neV specular walls, a
    uniform B0 along z (the harmonic l = 0, m = 0 term, field 0), the harmonic
    terms whose coefficients the gradients are taken with respect to (field 1)
    and the uniform E = (0, 0, ez) (EDMStaticEField)."""
    sc = Scene()
    sc.add_material("wall", 335.0)
    sc.add_material("vacuum", 0.0)
    sc.add_solid(1, "wall")
    sc.add_solid(2, "vacuum", S.cylinder_mesh(0.2, -0.06, 0.06, nseg))
    sc.add_harmonic([(0, 0, b0)])
    sc.add_harmonic(harmonic_terms_l2() if terms is None else terms)
    sc.add_uniform_e(0.0, 0.0, ez)
    return sc


def adjoint_spin(n=10_000, seed=1004, simtime=100.0, terms=None, first_id=0, nseg=512):
    """The adjoint-spin workload: UCN uniform in the cylinder (r < 0.19 m,
    |z| < 0.05 m), 0-200 neV isotropic, polarisation +1, spins along +x
    (the configuration's override of the reference's random azimuth about
    B), Bloch integration over the whole run (spintimes 0 simtime, Bmax 1 T),
    no decay."""
    sc = adjoint_spin_scene(nseg=nseg, terms=terms)
    ids = np.arange(first_id, first_id + n, dtype=np.int64)
    pos, (E, ph, th, pol) = S.source_cylinder(seed, ids, 0.0, 0.19, -0.05, 0.05, 0.0, 200e-9, polarization=1.0)
    parts = S.make_particles(seed, ids, pos, E, ph, th, pol)
    parts.spin[:] = 0.0
    parts.spin[0] = 1.0
    params = run_params(A.NEUTRON, simtime=simtime, tau=0.0, tmax=9e99, lmax=9e99, bmax=1.0, spintimes=(0.0, simtime),
                        seed=seed)
    return sc, params, parts


def multipole_table(n=128, lo=(-1.15, -1.15, -0.55), hi=(1.15, 1.15, 0.55), g1=0.43, g2=0.22, b0=0.05):
    """n^3 grid of the curl- and divergence-free multipole
    B = (g1 y + 2 g2 x y, g1 x + g2 (x^2 - y^2), b0) = grad(g1 x y + g2 (x^2 y - y^3/3) + b0 z),
    |B| <= 1 T over the box."""
    ax = tuple(np.linspace(lo[k], hi[k], n) for k in range(3))
    X, Y, Z = np.meshgrid(*ax, indexing="ij")
    return ax, (g1 * Y + 2 * g2 * X * Y, g1 * X + g2 * (X * X - Y * Y), np.full_like(X, b0))


def large_mesh_scene(table_n=128, nu=500, nv=160, nlat=101, nlon=200):
    """The large-mesh scene: a noise-perturbed torus (R = 1 m, r = 0.1 m,
    2 nu nv triangles) as the guide and a sphere (R = 0.5 m at the origin,
    2 nlon (nlat - 1) triangles) as the bottle, both closed vacuum solids in a
    wall of 10 % diffuse reflection and 3e-5 loss per bounce (200,000
    triangles by default), with gravity and the multipole table.  The two
    volumes are separate closed meshes (a seamless fusion would need a mesh
    boolean the workload generator does not have)."""
    sc = Scene()
    sc.add_material("wall", 250.0, 0.0, 0.1, 0.0, 0.0, 0.0, 0.0, 0.0, 3e-5)
    sc.add_material(*storage_vacuum(0.1, 3e-5))
    sc.add_solid(1, "wall")
    sc.add_solid(2, "vacuum", S.torus_mesh(1.0, 0.1, nu, nv, noise=0.05, seed=1005))
    sc.add_solid(3, "vacuum", S.sphere_mesh(0.5, nlat, nlon))
    ax, comps = multipole_table(table_n)
    sc.add_table3d(*ax, *comps)
    return sc


def large_mesh(n=10_000_000, seed=1005, simtime=100.0, table_n=128, scene=None, engine=None, first_id=0):
    """The large-mesh workload: UCN with E ~ U[0, 300] neV, isotropic, half of them
    uniform in the bottle (r < 0.45 m) and half uniform in the guide's tube
    (within 0.08 m of its centre circle), tau 880 s, 100 s."""
    sc = scene if scene is not None else large_mesh_scene(table_n)
    ids = np.arange(first_id, first_id + n, dtype=np.int64)
    u0, u1, u2 = (S.uniform(seed, ids, S.SOURCE_STREAM + np.uint64(50 + k)) for k in range(3))
    in_ball = (ids % 2) == 0
    # ball: radius by the cube root, direction uniform on the sphere
    rb = 0.45 * np.cbrt(u0)
    ct = 2 * u1 - 1
    st = np.sqrt(1 - ct * ct)
    pb = np.vstack([rb * st * np.cos(2 * np.pi * u2), rb * st * np.sin(2 * np.pi * u2), rb * ct])
    # tube: position along the ring uniform, uniform disc of radius 0.08 in the cross-section
    a = 2 * np.pi * u0
    rd = 0.08 * np.sqrt(u1)
    b = 2 * np.pi * u2
    pt = np.vstack([(1.0 + rd * np.cos(b)) * np.cos(a), (1.0 + rd * np.cos(b)) * np.sin(a), rd * np.sin(b)])
    pos = np.where(in_ball[None, :], pb, pt)
    E, ph, th, pol = S._kinematics(seed, ids, 0.0, 300e-9, (0.0, S.PI), (0.0, 2 * S.PI), 0.0)
    bf = None
    if engine is not None:
        def bf(p):
            q = np.column_stack([p, np.zeros(len(p))])
            return engine.field(q)[0]
    parts = S.make_particles(seed, ids, pos, E, ph, th, pol, spinprojection=0.0, bfield=bf)
    params = run_params(A.NEUTRON, simtime=simtime, tau=880.0, tmax=9e99, lmax=9e99, bmax=0.1, spintimes=(0, 0), seed=seed)
    return sc, params, parts
