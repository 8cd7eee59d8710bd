"""Synthetic scenes, STL/OPERA3D/OPERA2D readers and particle sources.

The workloads named by the benchmark (closed unit cube, field-storage
cylinder with a 64^3 tricubic quadrupole table, ...) are generated here from
seeds; no external dataset is involved.  Initial states use the reference's
source distributions (include/source.h:186-251, include/mc.h:143-213) and
the TParticle constructor's velocity/spin set-up (src/particle.cpp:36-90),
drawn from a Philox4x32-10 stream keyed by (seed, particle id) in a counter
range disjoint from the one the kernels use.
"""
import struct

import numpy as np

from . import _abi as A

# physical constants as exact doubles (generated header include/pt_constants.h)
PI = float.fromhex("0x1.921fb54442d18p+1")
C0 = float.fromhex("0x1.1de784a000000p+28")
M_N = float.fromhex("0x1.673302a9f27acp-27")
M_P = float.fromhex("0x1.66b46eac7abf4p-27")
M_E = float.fromhex("0x1.901732cb621c3p-38")
MU_N = float.fromhex("-0x1.7ec4036197f3ap-87")
ELE_E = float.fromhex("0x1.7a4da04a6daf5p-63")
GRAV = float.fromhex("0x1.39d013a92a305p+3")
GAMMA_N = float.fromhex("-0x1.5d842a2000000p+27")
MASS = {A.NEUTRON: M_N, A.PROTON: M_P, A.ELECTRON: M_E}

SOURCE_STREAM = np.uint64(1) << np.uint64(63)


# ----------------------------------------------------------------------------
# Philox4x32-10, vectorised
def philox4x32_10(c0, c1, c2, c3, k0, k1):
    M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
    W0, W1 = np.uint32(0x9E3779B9), np.uint32(0xBB67AE85)
    x0, x1, x2, x3 = (np.asarray(v, dtype=np.uint32) for v in (c0, c1, c2, c3))
    k0 = np.asarray(k0, dtype=np.uint32)
    k1 = np.asarray(k1, dtype=np.uint32)
    m32 = np.uint64(0xFFFFFFFF)
    for _ in range(10):
        p0 = M0 * x0.astype(np.uint64)
        p1 = M1 * x2.astype(np.uint64)
        y0 = (p1 >> np.uint64(32)).astype(np.uint32) ^ x1 ^ k0
        y1 = (p1 & m32).astype(np.uint32)
        y2 = (p0 >> np.uint64(32)).astype(np.uint32) ^ x3 ^ k1
        y3 = (p0 & m32).astype(np.uint32)
        x0, x1, x2, x3 = y0, y1, y2, y3
        with np.errstate(over="ignore"):
            k0 = (k0 + W0).astype(np.uint32)
            k1 = (k1 + W1).astype(np.uint32)
    return x0, x1, x2, x3


def uniform(seed, ids, draw):
    """53-bit uniforms in [0,1) for particle ids at draw index `draw` (array or scalar)."""
    ids = np.asarray(ids, dtype=np.int64).astype(np.uint64)
    draw = np.broadcast_to(np.asarray(draw, dtype=np.uint64), ids.shape)
    seed = np.uint64(seed)
    o0, o1, _, _ = philox4x32_10(draw & np.uint64(0xFFFFFFFF), draw >> np.uint64(32), ids & np.uint64(0xFFFFFFFF),
                                 ids >> np.uint64(32), seed & np.uint64(0xFFFFFFFF), seed >> np.uint64(32))
    v = (o0.astype(np.uint64) << np.uint64(32)) | o1.astype(np.uint64)
    return (v >> np.uint64(11)).astype(np.float64) * 2.0 ** -53


# ----------------------------------------------------------------------------
# meshes
def read_stl(path):
    """Binary STL as (n, 9) float64 vertices; |v| < 1e-8 snapped to 0
    (TTriangleMesh::ReadFile, src/trianglemesh.cpp:17-57)."""
    with open(path, "rb") as f:
        data = f.read()
    n = struct.unpack("<I", data[80:84])[0]
    if n == 0:
        raise ValueError(f"{path} contains no triangles")
    rec = np.frombuffer(data[84:84 + 50 * n], dtype=np.dtype([("n", "<f4", 3), ("v", "<f4", 9), ("a", "<u2")]))
    if len(rec) != n:
        raise ValueError(f"{path} should contain {n} triangles but read {len(rec)}")
    v = rec["v"].astype(np.float64)
    v[np.abs(v) < 1e-8] = 0.0
    return v


def write_stl(path, tris, name=b"synthetic"):
    tris = np.asarray(tris, dtype=np.float32).reshape(-1, 9)
    with open(path, "wb") as f:
        f.write(name.ljust(80, b" ")[:80])
        f.write(struct.pack("<I", len(tris)))
        for t in tris:
            a, b, c = t[0:3].astype(np.float64), t[3:6].astype(np.float64), t[6:9].astype(np.float64)
            nrm = np.cross(b - a, c - a)
            nrm = nrm / (np.linalg.norm(nrm) or 1.0)
            f.write(struct.pack("<3f", *nrm))
            f.write(t.tobytes())
            f.write(b"\0\0")


def as_stl_precision(tris):
    """Round vertices through float32 as a binary STL stores them."""
    v = np.asarray(tris, dtype=np.float32).astype(np.float64).reshape(-1, 9)
    v[np.abs(v) < 1e-8] = 0.0
    return v


def box_mesh(lo, hi):
    """12 outward-wound triangles of an axis-aligned box."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    P = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                  [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]], dtype=np.float64)
    quads = [(0, 3, 2, 1), (4, 5, 6, 7), (0, 1, 5, 4), (2, 3, 7, 6), (1, 2, 6, 5), (0, 4, 7, 3)]
    tris = []
    for a, b, c, d in quads:
        tris.append(np.concatenate([P[a], P[b], P[c]]))
        tris.append(np.concatenate([P[a], P[c], P[d]]))
    return as_stl_precision(np.array(tris))


def cylinder_mesh(r, z0, z1, nseg, cx=0.0, cy=0.0):
    """Closed cylinder: 2*nseg side triangles plus two nseg-triangle fan caps,
    outward winding."""
    phi = 2 * np.pi * np.arange(nseg) / nseg
    px, py = cx + r * np.cos(phi), cy + r * np.sin(phi)
    tris = []
    for i in range(nseg):
        j = (i + 1) % nseg
        a0, b0 = (px[i], py[i], z0), (px[j], py[j], z0)
        a1, b1 = (px[i], py[i], z1), (px[j], py[j], z1)
        tris.append(a0 + b0 + b1)
        tris.append(a0 + b1 + a1)
        tris.append((cx, cy, z0) + b0 + a0)
        tris.append((cx, cy, z1) + a1 + b1)
    return as_stl_precision(np.array(tris, dtype=np.float64))


def torus_mesh(R, r, nu, nv, noise=0.0, seed=0):
    """Closed torus about the z axis (major radius R, tube radius r) on an
    nu x nv vertex grid, 2 nu nv outward-wound triangles; each vertex moves
    along its tube normal by noise * r * (2u - 1) with u from the vertex's own
    Philox draw, so the mesh stays watertight."""
    iu, iv = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    a, b = 2 * np.pi * iu / nu, 2 * np.pi * iv / nv
    vid = (iu * nv + iv).astype(np.int64).ravel()
    rr = r * (1.0 + noise * (2.0 * uniform(seed, vid, 0) - 1.0)).reshape(nu, nv)
    P = np.stack([(R + rr * np.cos(b)) * np.cos(a), (R + rr * np.cos(b)) * np.sin(a), rr * np.sin(b)], -1)
    tris = []
    for i in range(nu):
        i1 = (i + 1) % nu
        for j in range(nv):
            j1 = (j + 1) % nv
            p00, p10, p11, p01 = P[i, j], P[i1, j], P[i1, j1], P[i, j1]
            tris.append(np.concatenate([p00, p10, p11]))
            tris.append(np.concatenate([p00, p11, p01]))
    return as_stl_precision(np.array(tris))


def sphere_mesh(R, nlat, nlon, center=(0.0, 0.0, 0.0)):
    """Closed UV sphere, outward winding: pole fans plus quads split in two
    (2 nlon (nlat - 1) triangles)."""
    c = np.asarray(center, dtype=np.float64)
    th = np.pi * np.arange(1, nlat) / nlat
    ph = 2 * np.pi * np.arange(nlon) / nlon
    ring = c + R * np.stack([np.sin(th)[:, None] * np.cos(ph)[None, :], np.sin(th)[:, None] * np.sin(ph)[None, :],
                             np.cos(th)[:, None] * np.ones(nlon)[None, :]], -1)
    top, bot = c + np.array([0, 0, R]), c - np.array([0, 0, R])
    tris = []
    for j in range(nlon):
        j1 = (j + 1) % nlon
        tris.append(np.concatenate([top, ring[0, j], ring[0, j1]]))
        tris.append(np.concatenate([bot, ring[-1, j1], ring[-1, j]]))
        for i in range(nlat - 2):
            a, b, cc, d = ring[i, j], ring[i + 1, j], ring[i + 1, j1], ring[i, j1]
            tris.append(np.concatenate([a, b, cc]))
            tris.append(np.concatenate([a, cc, d]))
    return as_stl_precision(np.array(tris))


# ----------------------------------------------------------------------------
# OPERA3D tables
def read_opera3d(path, lengthconv=1.0):
    """OPERA3D table (ReadOperaField3, src/field_3d.cpp:185-310): returns axes and
    (nx, ny, nz) arrays of the columns present (BX, BY, BZ, V)."""
    with open(path) as f:
        head = f.readline().split()
        xl, yl, zl = int(head[0]), int(head[1]), int(head[2])
        cols = []
        while True:
            line = f.readline()
            if line.strip() == "0":
                break
            cols.append(line.split()[1])
        data = np.loadtxt(f)
    if data.ndim == 1:
        data = data.reshape(1, -1)
    if len(data) != xl * yl * zl:
        raise ValueError(f"The header says the size is {xl * yl * zl}, actually it is {len(data)}!")
    xyz = data[:, :3] * lengthconv
    axes = [np.unique(xyz[:, k]) for k in range(3)]
    idx = [np.searchsorted(axes[k], xyz[:, k]) for k in range(3)]
    out = {}
    for ci, name in enumerate(cols[3:]):
        arr = np.zeros((len(axes[0]), len(axes[1]), len(axes[2])))
        arr[idx[0], idx[1], idx[2]] = data[:, 3 + ci]
        out[name.upper()] = arr
    return axes, out


def read_comsol(path, lengthconv=1.0):
    """COMSOL text export (ReadComsolField, src/field_3d.cpp:124-183): lines of
    x y z Bx By Bz separated by spaces, tabs or commas, lines starting with %
    or # skipped; returns the axes and (nx, ny, nz) arrays BX, BY, BZ."""
    rows = []
    with open(path) as f:
        for num, line in enumerate(f, 1):
            if line.startswith("%") or line.startswith("#"):
                continue
            parts = line.replace(",", " ").replace("\t", " ").split()
            if not parts:
                continue
            if len(parts) != 6:
                raise ValueError(f"Error reading line {num} of file {path}")
            rows.append([float(p) for p in parts])
    data = np.array(rows)
    xyz = data[:, :3] * lengthconv
    axes = [np.unique(xyz[:, k]) for k in range(3)]
    if np.prod([len(a) for a in axes]) != len(data):
        raise ValueError(f"{path}: the points do not fill a rectilinear grid")
    idx = [np.searchsorted(axes[k], xyz[:, k]) for k in range(3)]
    out = {}
    for c, name in enumerate(("BX", "BY", "BZ")):
        arr = np.zeros([len(a) for a in axes])
        arr[idx[0], idx[1], idx[2]] = data[:, 3 + c]
        out[name] = arr
    return axes, out


def write_opera3d(path, axes, comps):
    """Write an OPERA3D table in metres (lengthconv 1) with the given columns."""
    X, Y, Z = np.meshgrid(*axes, indexing="ij")
    names = list(comps)
    with open(path, "w") as f:
        f.write(f"{len(axes[0])} {len(axes[1])} {len(axes[2])} 2\n")
        f.write(" 1 X [METRE]\n 2 Y [METRE]\n 3 Z [METRE]\n")
        for i, nme in enumerate(names):
            f.write(f" {4 + i} {nme} [{'VOLT' if nme == 'V' else 'TESLA'}]\n")
        f.write(" 0\n")
        cols = [X.ravel(), Y.ravel(), Z.ravel()] + [np.asarray(comps[k]).ravel() for k in names]
        np.savetxt(f, np.column_stack(cols), fmt="%.17g")


# OPERA2D tables
OPERA2D_COLUMNS = (("RBX", "BR"), ("RBY", "BPHI"), ("RBZ", "BZ"), ("EX", "ER"), ("EY", "EPHI"), ("EZ", "EZ"),
                   ("RV", "V"))


def read_opera2d(path, lengthconv=1.0):
    """OPERA2D table (TabField::ReadTabFile, src/field_2d.cpp:68-190): header
    "m 1 n ...", the coordinate lines (r, an optional " 2 Y [LENGU]", z),
    then the optional column lines RBX, RBY, RBZ, EX, EY, EZ, RV in that
    order, recognised by substring as the reference does, up to " 0".  Rows
    run over z inside r; a z below the previous one starts the next r.
    Returns (r, z) and (nr, nz) arrays named BR, BPHI, BZ, ER, EPHI, EZ, V."""
    with open(path) as f:
        head = f.readline().split()
        m, n = int(head[0]), int(head[2])
        f.readline()
        line = f.readline()
        skipy = not line.startswith(" 2 Y [LENGU]")
        line = f.readline()
        if not skipy:
            line = f.readline()
        cols = []
        for tag, name in OPERA2D_COLUMNS:
            if tag in line:
                cols.append(name)
                line = f.readline()
        if not line.startswith(" 0"):
            raise ValueError(f"{path} not found or corrupt")
        data = np.array(f.read().split(), dtype=np.float64)
    width = (2 if skipy else 3) + len(cols)
    rows = data[: len(data) // width * width].reshape(-1, width)
    r_all, z_all = rows[:, 0] * lengthconv, rows[:, 1 if skipy else 2] * lengthconv
    ri = np.zeros(len(rows), dtype=np.int64)
    zi = np.zeros(len(rows), dtype=np.int64)
    cur_r, cur_z = 0, -1
    zs = {}
    for k in range(len(rows)):
        if cur_z >= 0 and z_all[k] < zs[cur_z]:
            cur_r, cur_z = cur_r + 1, 0
        else:
            cur_z += 1
        zs[cur_z] = z_all[k]
        ri[k], zi[k] = cur_r, cur_z
    if cur_r + 1 != m or cur_z + 1 != n:
        raise ValueError(f"The header says the size is {m} by {n}, actually it is {cur_r + 1} by {cur_z + 1}!")
    r = np.zeros(m)
    z = np.zeros(n)
    r[ri] = r_all
    z[zi] = z_all
    out = {}
    for c, name in enumerate(cols):
        arr = np.zeros((m, n))
        arr[ri, zi] = rows[:, (2 if skipy else 3) + c]
        out[name] = arr
    return (r, z), out


def write_opera2d(path, r, z, comps, lengthunit=1.0):
    """Write an OPERA2D table (columns r, z and the named ones of
    OPERA2D_COLUMNS in their file order); coordinates divided by lengthunit."""
    tags = [(tag, name) for tag, name in OPERA2D_COLUMNS if name in comps]
    R, Z = np.meshgrid(r, z, indexing="ij")
    with open(path, "w") as f:
        f.write(f"{len(r)} 1 {len(z)} 1\n 1 X [LENGU]\n 2 Z [LENGU]\n")
        for i, (tag, name) in enumerate(tags):
            f.write(f" {3 + i} {tag} [{'ENERU' if name == 'V' else 'FLUXU'}]\n")
        f.write(" 0\n")
        cols = [R.ravel() / lengthunit, Z.ravel() / lengthunit] + [np.asarray(comps[name]).ravel() for _, name in tags]
        np.savetxt(f, np.column_stack(cols), fmt="%.17g", delimiter="\t")


# ----------------------------------------------------------------------------
# particle construction
def speed_from_energy(E, m):
    """TParticle ctor (src/particle.cpp:45-52): beta^2 from E/mc^2 with the
    series below round-off."""
    Eom = E / m / C0 / C0
    series = ((((6.0 * Eom - 5.0) * Eom + 4.0) * Eom - 3.0) * Eom + 2.0) * Eom
    rel = 1.0 - 1.0 / (Eom + 1) / (Eom + 1)
    beta2 = np.where(Eom ** 6 < 2 * np.finfo(float).eps, series, rel)
    return C0 * np.sqrt(beta2)


def rotate_vector(v, n):
    """RotateVector(v, n) with CGAL's base1 x axis (src/globals.cpp:40-64), vectorised."""
    v = np.asarray(v, dtype=np.float64)
    n = np.asarray(n, dtype=np.float64)
    a, b, c = np.abs(n[0]), np.abs(n[1]), np.abs(n[2])
    xv = np.zeros_like(n)
    c1 = n[0] == 0
    c2 = ~c1 & (n[1] == 0)
    c3 = ~c1 & ~c2 & (n[2] == 0)
    rest = ~(c1 | c2 | c3)
    r1 = rest & (a <= b) & (a <= c)
    r2 = rest & ~r1 & (b <= a) & (b <= c)
    r3 = rest & ~r1 & ~r2
    xv[0, c1] = 1
    xv[1, c2] = 1
    xv[2, c3] = 1
    xv[1, r1], xv[2, r1] = -n[2, r1], n[1, r1]
    xv[0, r2], xv[2, r2] = -n[2, r2], n[0, r2]
    xv[0, r3], xv[1, r3] = -n[1, r3], n[0, r3]
    xu = xv / np.sqrt((xv ** 2).sum(0))
    zu = n / np.sqrt((n ** 2).sum(0))
    yu = np.cross(zu.T, xu.T).T
    return xu * v[0] + yu * v[1] + zu * v[2]


def make_particles(seed, ids, pos, energy, phi, theta, pol, species=A.NEUTRON, t0=0.0, spinprojection=None,
                   bfield=None):
    """Initial state of TParticle (src/particle.cpp:36-90).  `bfield(pos)` gives
    B at the start points; where |B| > 0 the spin is the spin projection along B
    with a random azimuth (one draw per particle from the source stream)."""
    n = len(ids)
    v = speed_from_energy(np.asarray(energy, dtype=np.float64), MASS[species])
    y = np.zeros((9, n))
    y[0:3] = pos
    y[3] = v * np.cos(phi) * np.sin(theta)
    y[4] = v * np.sin(phi) * np.sin(theta)
    y[5] = v * np.cos(theta)
    y[7] = pol
    spin = np.zeros((5, n))
    if bfield is not None:
        B = np.asarray(bfield(pos.T)).T
        babs = np.sqrt((B ** 2).sum(0))
        sp = pol if spinprojection is None else np.broadcast_to(spinprojection, (n,))
        az = 2.0 * PI * uniform(seed, ids, SOURCE_STREAM + np.uint64(100))
        s = np.vstack([np.sqrt(1 - sp * sp) * np.sin(az), np.sqrt(1 - sp * sp) * np.cos(az), sp * np.ones(n)])
        ok = babs > 0
        if ok.any():
            spin[0:3, ok] = rotate_vector(s[:, ok], B[:, ok])
    from .engine import ParticleSet
    return ParticleSet(n, ids, np.full(n, t0), y, spin)


def _draw(seed, ids, k):
    return uniform(seed, ids, SOURCE_STREAM + np.uint64(k))


def source_box(seed, ids, lo, hi, emin, emax, theta=(0.0, PI), phi=(0.0, 2 * PI), polarization=1.0):
    """TCuboidVolumeSource (include/source.h:186-213) with a flat spectrum, phi
    uniform and theta from sin_distribution (include/mc.h:143-156)."""
    ids = np.asarray(ids, dtype=np.int64)
    pos = np.vstack([lo[k] + _draw(seed, ids, k) * (hi[k] - lo[k]) for k in range(3)])
    return pos, _kinematics(seed, ids, emin, emax, theta, phi, polarization)


def source_cylinder(seed, ids, rmin, rmax, zmin, zmax, emin, emax, theta=(0.0, PI), phi=(0.0, 2 * PI), polarization=1.0,
                    phimin=0.0, phimax=2 * PI, spectrum=None):
    """TCylindricalVolumeSource (include/source.h:219-251): r from the linear
    distribution (include/mc.h:200-213), azimuth and z uniform."""
    ids = np.asarray(ids, dtype=np.int64)
    r = np.sqrt(_draw(seed, ids, 0) * (rmax * rmax - rmin * rmin) + rmin * rmin)
    ph = phimin + _draw(seed, ids, 1) * (phimax - phimin)
    z = zmin + _draw(seed, ids, 2) * (zmax - zmin)
    pos = np.vstack([r * np.cos(ph), r * np.sin(ph), z])
    return pos, _kinematics(seed, ids, emin, emax, theta, phi, polarization, spectrum)


def electron_beta_spectrum(E):
    """ElectronBetaSpectrum (src/globals.cpp:96-101): relative intensity (< 1)
    of neutron-decay electrons at kinetic energy E [eV] (0 <= E <= 782 keV)."""
    q = 0.782
    e = np.asarray(E, dtype=np.float64) * 1e-6
    mec2 = M_E * C0 * C0 / ELE_E * 1e-6
    return 8.2 * np.sqrt(e * e + 2 * e * mec2) * (q - e) ** 2 * (e + mec2)


def spectrum_sampler(f, emin, emax, tries=256, first_draw=1000):
    """Rejection sampling of the spectrum f (max < 1) on [emin, emax], as the
    reference's source does for its spectrum formula; draw pairs come from the
    particle's own Philox stream, so samples do not depend on the batch.
    The sampler's draws start at counter `first_draw` and use at most
    2 x `tries` counters."""
    def sample(seed, ids, first_draw=first_draw):
        ids = np.asarray(ids, dtype=np.int64)
        E = np.full(len(ids), np.nan)
        todo = np.ones(len(ids), bool)
        for k in range(tries):
            if not todo.any():
                break
            e = emin + _draw(seed, ids, first_draw + 2 * k) * (emax - emin)
            u = _draw(seed, ids, first_draw + 2 * k + 1)
            acc = todo & (u < f(e))
            E[acc] = e[acc]
            todo &= ~acc
        if todo.any():
            raise RuntimeError(f"spectrum sampling did not converge for {int(todo.sum())} particles")
        return E
    return sample


def _kinematics(seed, ids, emin, emax, theta, phi, polarization, spectrum=None):
    u = _draw(seed, ids, 3)
    pol = np.where(u < 0.5 * (polarization + 1), 1.0, -1.0)  # polarization_distribution (include/mc.h:22-48)
    if spectrum is None:
        E = emin + _draw(seed, ids, 4) * (emax - emin)
    else:
        E = spectrum(seed, ids)
    ph = phi[0] + _draw(seed, ids, 5) * (phi[1] - phi[0])
    u = _draw(seed, ids, 6)
    th = np.arccos(np.cos(theta[0]) - u * (np.cos(theta[0]) - np.cos(theta[1])))  # inversetransform_sin
    return E, ph, th, pol
