"""Python host binding of the engine's C ABI.

Mirrors the reference's host-side objects for the tracking path:
  Scene        -- what TGeometry(TConfig&) + TFieldManager(TConfig&) hold
                  (src/geometry.cpp:93-137, src/fields.cpp:19-136)
  Engine       -- a device context (pt_create) with IntegrateParticles, the
                  batched form of TTracker::IntegrateParticle (include/tracking.h:46-47)
  ParticleSet  -- the SoA start/end states the reference keeps per TParticle
The library is loaded from this package directory; there is no CPU fallback:
every call goes through libpentrack_gpu.so and fails loudly without it.
"""
import ctypes as C
import os

import numpy as np

from . import _abi as A

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


class EngineError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{A.STATUS.get(status, status)}: {msg}")
        self.status = status


def lib():
    """Load the in-tree engine library (built by pentrack_gb300.build)."""
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "libpentrack_gpu.so")
        if not os.path.exists(path):
            raise RuntimeError(f"engine library {path} is missing: run pentrack_gb300.build.build_engine() first")
        _LIB = C.CDLL(path)
        A.declare(_LIB)
    return _LIB


def _dp(a):
    return a.ctypes.data_as(A.c_double_p) if a is not None else None


def _ip(a):
    return a.ctypes.data_as(A.c_int32_p) if a is not None else None


def _lp(a):
    return a.ctypes.data_as(A.c_int64_p) if a is not None else None


# ----------------------------------------------------------------------------
class Scene:
    """Raw scene inputs: triangles per solid, materials, solids and fields.

    Solid 0 is the default solid (ID 1), as in the reference's [GEOMETRY]
    section where ID 1 names the medium outside every STL (src/geometry.cpp:125-128).
    """

    def __init__(self):
        self.materials = []       # list of 9-tuples (materials.in columns)
        self.material_names = []
        self.solids = []          # dicts: id, material, ignore (list of (t0, t1))
        self.tri_blocks = []      # (triangles (n,9) float64, solid index)
        self.fields = []          # dicts

    # --- materials / solids -------------------------------------------------
    def add_material(self, name, fermi_real, fermi_imag=0.0, diff_prob=0.0, spinflip_prob=0.0, rms_roughness=0.0,
                     correl_length=0.0, internal_bfield=0.0, modified_lambert_prob=0.0, loss_per_bounce=0.0):
        self.materials.append((fermi_real, fermi_imag, diff_prob, spinflip_prob, rms_roughness, correl_length,
                               internal_bfield, modified_lambert_prob, loss_per_bounce))
        self.material_names.append(name)
        return len(self.materials) - 1

    def material_index(self, name):
        return self.material_names.index(name)

    def add_solid(self, sid, material, triangles=None, ignore=()):
        if isinstance(material, str):
            material = self.material_index(material)
        if not self.solids and sid != 1:
            raise ValueError("the first solid must be the default solid with ID 1")
        self.solids.append({"id": int(sid), "material": int(material), "ignore": list(ignore)})
        idx = len(self.solids) - 1
        if triangles is not None:
            tri = np.ascontiguousarray(np.asarray(triangles, dtype=np.float64).reshape(-1, 9))
            self.tri_blocks.append((tri, idx))
        return idx

    # --- fields -------------------------------------------------------------
    def add_table3d(self, x, y, z, bx=None, by=None, bz=None, v=None, b_scale=1.0, e_scale=1.0, boundary_width=0.0,
                    box=None):
        """TabField3 on a rectilinear grid; arrays shaped (nx, ny, nz).  The
        container box defaults to the table's extent (src/field_3d.cpp:306-309)."""
        x, y, z = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z))
        f = {"type": A.FIELD_TAB3D, "x": x, "y": y, "z": z, "b_scale": b_scale, "e_scale": e_scale,
             "boundary_width": boundary_width}
        for k, arr in (("bx", bx), ("by", by), ("bz", bz), ("v", v)):
            f[k] = None if arr is None else np.ascontiguousarray(arr, dtype=np.float64).reshape(-1)
        f["box"] = box if box is not None else (x.max(), x.min(), y.max(), y.min(), z.max(), z.min())
        self.fields.append(f)

    def add_table2d(self, r, z, br=None, bphi=None, bz=None, v=None, er=None, ephi=None, ez=None, b_scale=1.0,
                    e_scale=1.0):
        """TabField (OPERA2D / 2Dtable): a field rotationally symmetric about
        the z axis on an (r, z) grid; arrays shaped (nr, nz).  E_r, E_phi,
        E_z columns take precedence over the potential.  The reference wraps
        it in a container without a box (src/field_2d.cpp:65)."""
        r, z = (np.ascontiguousarray(a, dtype=np.float64) for a in (r, z))
        f = {"type": A.FIELD_TAB2D, "x": r, "z": z, "b_scale": b_scale, "e_scale": e_scale, "boundary_width": 0.0,
             "box": (0, 0, 0, 0, 0, 0)}
        for k, arr in (("bx", br), ("by", bphi), ("bz", bz), ("v", v), ("er", er), ("ephi", ephi), ("ez", ez)):
            f[k] = None if arr is None else np.ascontiguousarray(arr, dtype=np.float64).reshape(-1)
        self.fields.append(f)

    def add_harmonic(self, coeffs, offset=(0.0, 0.0, 0.0), b_scale=1.0, boundary_width=0.0, box=(0, 0, 0, 0, 0, 0)):
        """HarmonicExpansionBField: coeffs = [(l, m, G), ...]."""
        l = np.array([c[0] for c in coeffs], dtype=np.int32)
        m = np.array([c[1] for c in coeffs], dtype=np.int32)
        g = np.array([c[2] for c in coeffs], dtype=np.float64)
        self.fields.append({"type": A.FIELD_HARMONIC, "l": l, "m": m, "g": g, "offset": offset, "b_scale": b_scale,
                            "e_scale": 0.0, "boundary_width": boundary_width, "box": box})

    def add_solenoid(self, radius, half_length, b_center, center=(0.0, 0.0, 0.0), b_scale=1.0, boundary_width=0.0,
                     box=(0, 0, 0, 0, 0, 0)):
        """Finite ideal solenoid along z (closed form, include/pt_solenoid.h):
        sheet current on rho = radius, |z - zc| <= half_length, field b_center
        [T] at its centre."""
        self.fields.append({"type": A.FIELD_SOLENOID, "offset": center, "radius": radius, "half_length": half_length,
                            "b_center": b_center, "b_scale": b_scale, "e_scale": 0.0, "boundary_width": boundary_width,
                            "box": box})

    def add_uniform_e(self, ex, ey, ez, e_scale=1.0):
        """EDMStaticEField (src/edmfields.cpp:181-187): no box, B scale 0."""
        self.fields.append({"type": A.FIELD_UNIFORM_E, "e": (ex, ey, ez), "b_scale": 0.0, "e_scale": e_scale,
                            "boundary_width": 0.0, "box": (0, 0, 0, 0, 0, 0)})

    # --- ABI ------------------------------------------------------------------
    def desc(self):
        """Build a pt_scene_desc; the returned object keeps every array alive."""
        keep = []
        tris = [b[0] for b in self.tri_blocks]
        sids = [np.full(len(b[0]), b[1], dtype=np.int32) for b in self.tri_blocks]
        T = np.ascontiguousarray(np.concatenate(tris)) if tris else np.zeros((0, 9))
        S = np.ascontiguousarray(np.concatenate(sids)) if sids else np.zeros(0, np.int32)
        keep += [T, S]
        mats = (A.Material * max(1, len(self.materials)))()
        for i, m in enumerate(self.materials):
            mats[i] = A.Material(*m)
        sol = (A.Solid * len(self.solids))()
        for i, s in enumerate(self.solids):
            ig = np.ascontiguousarray(np.array(s["ignore"], dtype=np.float64).reshape(-1))
            keep.append(ig)
            sol[i] = A.Solid(s["id"], s["material"], len(s["ignore"]), 0, _dp(ig) if len(ig) else None)
        flds = (A.Field * max(1, len(self.fields)))()
        for i, f in enumerate(self.fields):
            F = A.Field()
            F.type = f["type"]
            F.b_scale, F.e_scale = f["b_scale"], f["e_scale"]
            F.xmax, F.xmin, F.ymax, F.ymin, F.zmax, F.zmin = f["box"]
            F.boundary_width = f["boundary_width"]
            if f["type"] == A.FIELD_TAB3D:
                F.nx, F.ny, F.nz = len(f["x"]), len(f["y"]), len(f["z"])
                F.x, F.y, F.z = _dp(f["x"]), _dp(f["y"]), _dp(f["z"])
                F.bx, F.by, F.bz, F.v = (_dp(f[k]) for k in ("bx", "by", "bz", "v"))
                keep += [f[k] for k in ("x", "y", "z", "bx", "by", "bz", "v")]
            elif f["type"] == A.FIELD_TAB2D:
                F.nx, F.ny, F.nz = len(f["x"]), 1, len(f["z"])
                F.x, F.z = _dp(f["x"]), _dp(f["z"])
                F.bx, F.by, F.bz, F.v, F.er, F.ephi, F.ez = (_dp(f[k]) for k in ("bx", "by", "bz", "v", "er", "ephi", "ez"))
                keep += [f[k] for k in ("x", "z", "bx", "by", "bz", "v", "er", "ephi", "ez")]
            elif f["type"] == A.FIELD_HARMONIC:
                F.n_coeff = len(f["l"])
                F.l, F.m, F.g = _ip(f["l"]), _ip(f["m"]), _dp(f["g"])
                F.offset[:] = f["offset"]
                keep += [f["l"], f["m"], f["g"]]
            elif f["type"] == A.FIELD_UNIFORM_E:
                F.e[:] = f["e"]
            elif f["type"] == A.FIELD_SOLENOID:
                F.offset[:] = f["offset"]
                F.sol_radius, F.sol_half_length, F.sol_bcenter = f["radius"], f["half_length"], f["b_center"]
            flds[i] = F
        d = A.SceneDesc(len(T), _dp(T), _ip(S), len(self.solids), len(self.materials), sol, mats, len(self.fields), 0,
                        flds)
        return d, (keep, mats, sol, flds)


# ----------------------------------------------------------------------------
class ParticleSet:
    """SoA particle states: y is (9, n) = x, y, z, vx, vy, vz, proper time,
    polarisation, path length (include/particle.h:21); spin is (5, n)."""

    OUT_FIELDS = (("stop_id", np.int32), ("solid", np.int32), ("n_hit", np.int32), ("n_step", np.int32),
                  ("n_spinflip", np.int32), ("h_max", np.float64), ("noflip_prob", np.float64), ("tau", np.float64),
                  ("h_start", np.float64), ("n_accepted", np.int64), ("n_rejected", np.int64))

    def __init__(self, n, id=None, t=None, y=None, spin=None):
        self.n = int(n)
        self.id = np.ascontiguousarray(np.arange(n, dtype=np.int64) if id is None else id, dtype=np.int64)
        self.t = np.ascontiguousarray(np.zeros(n) if t is None else t, dtype=np.float64)
        self.y = np.ascontiguousarray(np.zeros((9, n)) if y is None else y, dtype=np.float64)
        self.spin = np.ascontiguousarray(np.zeros((5, n)) if spin is None else spin, dtype=np.float64)
        for name, dt in self.OUT_FIELDS:
            setattr(self, name, np.zeros(n, dtype=dt))

    @classmethod
    def empty(cls, n):
        """A set with uninitialised arrays (every field is an output of pt_batch_read)."""
        p = cls.__new__(cls)
        p.n = int(n)
        p.id = np.empty(n, np.int64)
        p.t = np.empty(n)
        p.y = np.empty((9, n))
        p.spin = np.empty((5, n))
        for name, dt in cls.OUT_FIELDS:
            setattr(p, name, np.empty(n, dtype=dt))
        return p

    def copy(self):
        p = ParticleSet(self.n, self.id.copy(), self.t.copy(), self.y.copy(), self.spin.copy())
        for name, _ in self.OUT_FIELDS:
            setattr(p, name, getattr(self, name).copy())
        return p

    def subset(self, idx):
        p = ParticleSet(len(idx), self.id[idx], self.t[idx], self.y[:, idx], self.spin[:, idx])
        return p

    def head(self, m):
        """the first m particles, outputs included (copies)"""
        p = ParticleSet(m, self.id[:m].copy(), self.t[:m].copy(), self.y[:, :m].copy(), self.spin[:, :m].copy())
        for name, _ in self.OUT_FIELDS:
            setattr(p, name, getattr(self, name)[:m].copy())
        return p

    def abi(self, outputs=True):
        P = A.Particles()
        P.n = self.n
        P.id, P.t, P.y, P.spin = _lp(self.id), _dp(self.t), _dp(self.y), _dp(self.spin)
        if outputs:
            P.stop_id, P.solid, P.n_hit, P.n_step, P.n_spinflip = (_ip(getattr(self, k)) for k in
                                                                   ("stop_id", "solid", "n_hit", "n_step", "n_spinflip"))
            P.h_max, P.noflip_prob, P.tau, P.h_start = (_dp(getattr(self, k)) for k in ("h_max", "noflip_prob", "tau", "h_start"))
            P.n_accepted, P.n_rejected = _lp(self.n_accepted), _lp(self.n_rejected)
        return P


def run_params(species=A.NEUTRON, simtime=100.0, tau=0.0, tmax=9e99, lmax=9e99, bmax=0.0, spintimes=(), flipspin=0,
               seed=1, mode=A.MODE_PLAIN, precision=A.PREC_FP64, steps_per_launch=0, block_size=0):
    """pt_run_params from the reference's [GLOBAL] simtime and particle options
    (tau, tmax, lmax, Bmax, spintimes, flipspin; src/tracking.cpp:19-60)."""
    st = np.ascontiguousarray(np.array(spintimes, dtype=np.float64).reshape(-1))
    p = A.RunParams()
    p.species, p.mode, p.field_precision, p.flipspin = species, mode, precision, flipspin
    p.simtime, p.tau, p.tmax, p.lmax, p.bmax = simtime, tau, tmax, lmax, bmax
    p.n_spintimes = len(st)
    p.spintimes = _dp(st) if len(st) else None
    p.steps_per_launch = steps_per_launch
    p.seed = seed
    p.block_size = block_size
    p._keep = st
    return p


def set_logs(p, hitlog=False, snapshots=None, track_interval=0.0, spin_interval=0.0, capacity=0):
    """Turn on the hit log, (with snapshot times) the snapshot log, (with a
    path-length interval [m]) the track log and (with a time interval [s])
    the spin log of a run (the particle options hitlog, snapshotlog /
    snapshots, tracklog / trackloginterval and spinlog / spinloginterval of
    src/logger.cpp:128-284); read them after the run with Engine.read_log."""
    p.hitlog = int(bool(hitlog))
    p.spinlog = int(spin_interval > 0)
    p.spinloginterval = float(spin_interval)
    p.tracklog = int(track_interval > 0)
    p.trackloginterval = float(track_interval)
    ts = np.ascontiguousarray(np.array(() if snapshots is None else snapshots, dtype=np.float64).reshape(-1))
    p.snapshotlog = int(len(ts) > 0)
    p.n_snapshots = len(ts)
    p.snapshots = _dp(ts) if len(ts) else None
    p.log_capacity = capacity
    p._keep_snap = ts
    return p


class ConfigScene:
    """The scene of a PENTrack config.in as the library's config front end
    reads it (pt_config_load: [GEOMETRY], [MATERIALS] / materials_file,
    [FIELDS], [FORMULAS]; files relative to the config)."""

    def __init__(self, path):
        h = C.c_void_p()
        st = lib().pt_config_load(os.fsencode(str(path)), C.byref(h))
        if st != A.PT_OK:
            raise EngineError(st, lib().pt_config_error().decode())
        self.h = h
        self.path = str(path)

    def desc(self):
        return lib().pt_config_scene_desc(self.h).contents, self

    def __del__(self):
        if getattr(self, "h", None):
            lib().pt_config_free(self.h)
            self.h = None


def config_run_params(path, species="neutron", max_spintimes=64):
    """pt_run_params from [GLOBAL] simtime and the species' particle options."""
    p = A.RunParams()
    buf = np.zeros(max_spintimes)
    st = lib().pt_config_run_params(os.fsencode(str(path)), species.encode(), C.byref(p), _dp(buf), max_spintimes)
    if st != A.PT_OK:
        raise EngineError(st, lib().pt_config_error().decode())
    p._keep = buf
    return p


class Engine:
    """One device context: the scene on the GPU plus the tracking kernels."""

    def __init__(self, scene, device=0):
        L = lib()
        self._desc, self._keep = scene.desc()
        h = C.c_void_p()
        st = L.pt_create(C.byref(self._desc), device, C.byref(h))
        if st != A.PT_OK:
            raise EngineError(st, L.pt_last_error(None).decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().pt_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != A.PT_OK and st != A.PT_ERR_CANCELLED:
            raise EngineError(st, lib().pt_last_error(self.h).decode())
        return st

    def integrate(self, params, particles, out=None):
        """Track every particle to its stop ID (host arrays in and out).  `out`
        (a ParticleSet of the same size, e.g. with pinned arrays) receives the
        end states; by default fresh arrays are allocated."""
        if out is None:
            out = ParticleSet.empty(particles.n)
        elif out.n != particles.n:
            raise ValueError("output set has a different size")
        stats = A.Stats()
        pin, pout = particles.abi(outputs=False), out.abi()
        self.last_status = self._check(lib().pt_integrate(self.h, C.byref(params), C.byref(pin), C.byref(pout), C.byref(stats)))
        return out, stats.as_dict()

    def batch(self, params, particles):
        return Batch(self, params, particles)

    def adjoint(self, params, particles, field, dl_dspin, dl_dy=None, checkpoint_interval=1024, out=None):
        """pt_adjoint: dL/dG for the coefficients of harmonic field `field`,
        given dL/d(end spin) (5, n) and optionally dL/d(end state) (9, n) per
        particle.  Returns (dL_dG, end states of the forward pass, stats)."""
        n = particles.n
        dsp = np.ascontiguousarray(dl_dspin, dtype=np.float64).reshape(5, n)
        dy = None if dl_dy is None else np.ascontiguousarray(dl_dy, dtype=np.float64).reshape(9, n)
        nc = len(self._field_coeffs(field))
        g = np.zeros(nc)
        if out is None:
            out = ParticleSet.empty(n)
        stats = A.Stats()
        pin, pout = particles.abi(outputs=False), out.abi()
        self._check(lib().pt_adjoint(self.h, C.byref(params), C.byref(pin), field, checkpoint_interval, _dp(dsp),
                                     _dp(dy) if dy is not None else None, _dp(g), C.byref(pout), C.byref(stats)))
        return g, out, stats.as_dict()

    def _field_coeffs(self, field):
        f = self._desc.fields[field]
        if f.type != A.FIELD_HARMONIC:
            raise ValueError("pt_adjoint differentiates a harmonic-expansion field")
        return [f.g[k] for k in range(f.n_coeff)]

    def mr(self, what, v, normal, Estep, b, w, transmit=False, integral=False, theta=None, phi=None):
        """pt_mr_eval over contacts: v, normal (n, 3); Estep, b, w (n,) or
        scalars; what = "dist" (with theta, phi), "prob" or "max"."""
        v = np.ascontiguousarray(np.atleast_2d(v), dtype=np.float64)
        n = len(v)
        arr = lambda a: np.ascontiguousarray(np.broadcast_to(np.asarray(a, dtype=np.float64), (n,)))  # noqa: E731
        nr = np.ascontiguousarray(np.broadcast_to(np.asarray(normal, dtype=np.float64), (n, 3)))
        E, bb, ww = arr(Estep), arr(b), arr(w)
        th = arr(0.0 if theta is None else theta)
        ph = arr(0.0 if phi is None else phi)
        out = np.zeros(n)
        k = {"dist": 0, "prob": 1, "max": 2}[what]
        self._check(lib().pt_mr_eval(self.h, k, int(transmit), int(integral), n, _dp(v), _dp(nr), _dp(E), _dp(bb), _dp(ww),
                                     _dp(th), _dp(ph), _dp(out)))
        return out

    def neutron_decay(self, seed, neutrons, which=None):
        """pt_neutron_decay: the protons and electrons of the decayed neutrons of
        a tracked set (stop ID ID_DECAYED, or the indices `which`), made on the
        device; the same draws and formulas as secondaries.neutron_decay."""
        idx = np.nonzero(neutrons.stop_id == A.ID_DECAYED)[0] if which is None else np.asarray(which)
        m = len(idx)
        ids = np.ascontiguousarray(neutrons.id[idx])
        t = np.ascontiguousarray(neutrons.t[idx])
        y = np.ascontiguousarray(neutrons.y[:, idx])
        pp, pe = ParticleSet(m), ParticleSet(m)
        a, b = pp.abi(outputs=False), pe.abi(outputs=False)
        self._check(lib().pt_neutron_decay(self.h, seed, m, _lp(ids), _dp(t), _dp(y), C.byref(a), C.byref(b)))
        return pp, pe

    def integrate_secondaries(self, neutron, proton, electron, particles):
        """pt_integrate_secondaries: neutrons, then the protons and electrons of
        those that decayed, in one call; returns the three end-state sets and
        the summed stats."""
        n = particles.n
        out, op, oe = ParticleSet.empty(n), ParticleSet.empty(n), ParticleSet.empty(n)
        st, nd = A.Stats(), C.c_int64(0)
        pin = particles.abi(outputs=False)
        a, b, c = out.abi(), op.abi(), oe.abi()
        self._check(lib().pt_integrate_secondaries(self.h, C.byref(neutron), C.byref(proton), C.byref(electron), C.byref(pin),
                                                   C.byref(a), C.byref(b), C.byref(c), C.byref(nd), C.byref(st)))
        m = nd.value
        return out, op.head(m), oe.head(m), st.as_dict()

    def field(self, xyzt, precision=A.PREC_FP64, grad=True):
        """B, dB/dx, V, E at (x, y, z, t) rows; grad=False evaluates B on the
        value-only path and returns dB None."""
        q = np.ascontiguousarray(xyzt, dtype=np.float64).reshape(-1, 4)
        n = len(q)
        B, V, E = np.zeros((n, 3)), np.zeros(n), np.zeros((n, 3))
        dB = np.zeros((n, 3, 3)) if grad else None
        self._check(lib().pt_field_eval(self.h, n, _dp(q), precision, _dp(B), _dp(dB) if grad else None, _dp(V), _dp(E)))
        return B, dB, V, E

    def collisions(self, segs, max_hits=8):
        s = np.ascontiguousarray(segs, dtype=np.float64).reshape(-1, 6)
        n = len(s)
        cnt = np.zeros(n, np.int32)
        ss, nn, sid, dn = np.zeros((n, max_hits)), np.zeros((n, max_hits, 3)), np.zeros((n, max_hits), np.int32), np.zeros((n, max_hits))
        self._check(lib().pt_segment_collisions(self.h, n, _dp(s), max_hits, _ip(cnt), _dp(ss), _dp(nn), _ip(sid), _dp(dn)))
        return cnt, ss, nn, sid, dn

    def collisions_noalloc(self, segs, max_hits=8):
        """pt_segment_collisions_noalloc: the same query through the entry
        point that uses the library's static device scratch (at most 8 MiB:
        52 n + 44 n max_hits bytes) instead of allocating."""
        s = np.ascontiguousarray(segs, dtype=np.float64).reshape(-1, 6)
        n = len(s)
        cnt = np.zeros(n, np.int32)
        ss, nn, sid, dn = np.zeros((n, max_hits)), np.zeros((n, max_hits, 3)), np.zeros((n, max_hits), np.int32), np.zeros((n, max_hits))
        self._check(lib().pt_segment_collisions_noalloc(self.h, n, _dp(s), max_hits, _ip(cnt), _dp(ss), _dp(nn), _ip(sid), _dp(dn)))
        return cnt, ss, nn, sid, dn

    def source_volume(self, ids, seed, species=A.NEUTRON, shape=A.SOURCE_BOX, lo=(0, 0, 0), hi=(0, 0, 0),
                      cylinder=(0, 0, 0, 0, 0, 0), solid=0, phase_space=False, emin=0.0, emax=0.0, polarization=0.0,
                      t_range=(0.0, 0.0), theta=(0.0, np.pi), phi=(0.0, 2 * np.pi), n_min_samples=100_000,
                      max_rounds=100_000, enormal=0.0, region=None):
        """pt_source_volume: initial states of the particles `ids` from a
        cuboid (lo, hi), cylindrical (cylinder = rmin, rmax, phimin, phimax,
        zmin, zmax) or STL volume (scene solid index `solid`, points proposed
        in the box lo..hi), optionally phase-space weighted, or from the
        scene's surfaces inside a cylindrical region (SOURCE_SURFACE_CYLINDER,
        `cylinder` as above) or inside an STL (SOURCE_SURFACE_STL: `region`
        an Engine on the same device whose scene holds the STL as solid
        index 1), with the normal energy raised by `enormal`, generated on the
        device.
        Returns (ParticleSet, minimum potential or -inf)."""
        ids = np.ascontiguousarray(ids, dtype=np.int64)
        n = len(ids)
        sp = A.SourceParams()
        sp.species, sp.shape, sp.seed = species, shape, int(seed)
        for a in range(3):
            sp.lo[a], sp.hi[a] = lo[a], hi[a]
        sp.rmin, sp.rmax, sp.phimin, sp.phimax, sp.zmin, sp.zmax = cylinder
        sp.solid, sp.phase_space = solid, int(bool(phase_space))
        sp.emin, sp.emax, sp.polarization = emin, emax, polarization
        sp.tmin, sp.tmax = t_range
        sp.thetamin, sp.thetamax = theta
        sp.phimin_v, sp.phimax_v = phi
        sp.n_min_samples, sp.max_rounds = n_min_samples, max_rounds
        sp.enormal = enormal
        sp.region = region.h if region is not None else None
        out = ParticleSet(n, ids.copy())
        vmin = C.c_double(0)
        P = out.abi(outputs=False)
        self._check(lib().pt_source_volume(self.h, C.byref(sp), n, _lp(out.id), C.byref(P), C.byref(vmin)))
        return out, vmin.value

    def read_log(self, kind):
        """pt_log_read: the records of the last run's hit log (kind LOG_HIT,
        columns of A.HIT_RECORD), snapshot log (LOG_SNAPSHOT) or track log
        (LOG_TRACK), sorted by
        particle and time, as an (n, width) array; and the number of events
        (more than n when the log's capacity was exceeded)."""
        width = {A.LOG_HIT: A.HIT_RECORD, A.LOG_SNAPSHOT: A.SNAPSHOT_RECORD, A.LOG_TRACK: A.TRACK_RECORD,
                 A.LOG_SPIN: A.SPIN_RECORD}[kind]
        total = C.c_int64(0)
        self._check(lib().pt_log_read(self.h, kind, 0, None, C.byref(total)))
        rec = np.zeros((max(total.value, 0), width))
        if total.value > 0:
            self._check(lib().pt_log_read(self.h, kind, total.value, _dp(rec), C.byref(total)))
        order = np.lexsort((rec[:, 1], rec[:, 0])) if len(rec) else np.arange(0)
        return rec[order], int(total.value)

    def point_solids(self, pts):
        p = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
        m = np.zeros(len(p), np.uint64)
        self._check(lib().pt_point_solids(self.h, len(p), _dp(p), m.ctypes.data_as(A.c_uint64_p)))
        return m

    def cancel(self):
        lib().pt_cancel(self.h)


class Batch:
    """Device-resident particle batch (pt_batch_*): advance in lab-time windows."""

    def __init__(self, engine, params, particles):
        self.engine = engine
        self.n = particles.n
        self._template = particles
        h = C.c_void_p()
        pin = particles.abi(outputs=False)
        engine._check(lib().pt_batch_create(engine.h, C.byref(params), C.byref(pin), C.byref(h)))
        self.h = h

    def advance(self, t_pause=float("inf"), max_steps=0):
        """Advance live particles until they stop, reach lab time t_pause at a
        step boundary, or (max_steps > 0) complete max_steps accepted steps."""
        st = A.Stats()
        self.engine._check(lib().pt_batch_advance_steps(self.engine.h, self.h, t_pause, max_steps, C.byref(st)))
        return st.as_dict()

    def read(self):
        out = self._template.copy()
        p = out.abi()
        self.engine._check(lib().pt_batch_read(self.engine.h, self.h, C.byref(p)))
        return out

    def close(self):
        if getattr(self, "h", None):
            lib().pt_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
