"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it:
it is the checker of the GPU engine and never part of the product path.
"""
import ctypes as C
import os

import numpy as np

from pentrack_gb300 import _abi as A

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "libpto.so")
        if not os.path.exists(path):
            raise RuntimeError("oracle library missing: run `make -C oracle`")
        L = C.CDLL(path)
        vp = C.c_void_p
        P = C.POINTER
        dp = A.c_double_p
        L.pto_create.argtypes = [P(A.SceneDesc), P(vp)]
        L.pto_create.restype = C.c_int
        L.pto_destroy.argtypes = [vp]
        L.pto_last_error.restype = C.c_char_p
        L.pto_track.argtypes = [vp, P(A.RunParams), P(A.Particles), P(A.Particles), C.c_int, P(A.Stats)]
        L.pto_field.argtypes = [vp, C.c_int64, dp, dp, dp, dp, dp]
        L.pto_segment_collisions.argtypes = [vp, C.c_int64, dp, C.c_int32, A.c_int32_p, dp, dp, A.c_int32_p, dp]
        L.pto_point_solids.argtypes = [vp, C.c_int64, dp, A.c_uint64_p]
        L.pto_spline_derivs.argtypes = [C.c_int32, dp, dp, dp]
        L.pto_spline1d_calc.argtypes = [C.c_int32, dp, dp, C.c_int32, dp, dp]
        L.pto_mr.argtypes = [C.c_int32, C.c_int32, C.c_int32, dp, dp, C.c_double, C.c_double, C.c_double, C.c_double,
                             C.c_double]
        L.pto_mr.restype = C.c_double
        L.pto_tricubic_coeff.argtypes = [dp, dp]
        L.pto_tricubic_eval.argtypes = [dp, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int, dp]
        L.pto_philox4x32_10.argtypes = [P(C.c_uint32), P(C.c_uint32), P(C.c_uint32)]
        L.pto_uniform.argtypes = [C.c_uint64, C.c_int64, C.c_uint64]
        L.pto_uniform.restype = C.c_double
        L.pto_detpow.argtypes = [C.c_double, C.c_double]
        L.pto_detpow.restype = C.c_double
        L.pto_dopri5_selftest.argtypes = [C.c_double, dp, C.c_double, C.c_int, dp, dp]
        L.pto_log_read.argtypes = [vp, C.c_int32, C.c_int64, dp]
        L.pto_log_read.restype = C.c_int64
        _LIB = L
    return _LIB


def ref_lib():
    """oracle/_ref/libptref.so (reference ALGLIB + libtricubic), or None."""
    global _REF
    if _REF is None:
        path = os.path.join(HERE, "_ref", "libptref.so")
        if not os.path.exists(path):
            return None
        R = C.CDLL(path)
        R.ref_spline_derivs.argtypes = [C.c_int, A.c_double_p, A.c_double_p, A.c_double_p]
        R.ref_tricubic_coeff.argtypes = [A.c_double_p, A.c_double_p]
        R.ref_tricubic_eval.argtypes = [A.c_double_p, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int]
        R.ref_tricubic_eval.restype = C.c_double
        R.ref_spline1d_calc.argtypes = [C.c_int, A.c_double_p, A.c_double_p, C.c_int, A.c_double_p, A.c_double_p]
        R.ref_spline2d.argtypes = [C.c_int, A.c_double_p, C.c_int, A.c_double_p, A.c_double_p, C.c_int, A.c_double_p,
                                   A.c_double_p, A.c_double_p]
        _REF = R
    return _REF


def _dp(a):
    return a.ctypes.data_as(A.c_double_p)


class Oracle:
    def __init__(self, scene):
        self._desc, self._keep = scene.desc()
        h = C.c_void_p()
        st = lib().pto_create(C.byref(self._desc), C.byref(h))
        if st != 0:
            raise RuntimeError("oracle: " + lib().pto_last_error().decode())
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            lib().pto_destroy(self.h)
            self.h = None

    def integrate(self, params, particles, nthreads=None):
        out = particles.copy()
        stats = A.Stats()
        nthreads = nthreads or os.cpu_count()
        lib().pto_track(self.h, C.byref(params), C.byref(particles.abi(outputs=False)), C.byref(out.abi()), nthreads,
                        C.byref(stats))
        return out, stats.as_dict()

    def read_log(self, kind):
        """records of the last integrate call's hit log (A.LOG_HIT) or snapshot
        log (A.LOG_SNAPSHOT), sorted by particle and time"""
        width = {A.LOG_HIT: A.HIT_RECORD, A.LOG_SNAPSHOT: A.SNAPSHOT_RECORD, A.LOG_TRACK: A.TRACK_RECORD,
                 A.LOG_SPIN: A.SPIN_RECORD}[kind]
        n = lib().pto_log_read(self.h, kind, 0, None)
        rec = np.zeros((n, width))
        if n:
            lib().pto_log_read(self.h, kind, n, _dp(rec))
        order = np.lexsort((rec[:, 1], rec[:, 0])) if n else np.arange(0)
        return rec[order]

    def field(self, xyzt, grad=True):
        q = np.ascontiguousarray(xyzt, dtype=np.float64).reshape(-1, 4)
        n = len(q)
        B, V, E = np.zeros((n, 3)), np.zeros(n), np.zeros((n, 3))
        dB = np.zeros((n, 3, 3)) if grad else None
        lib().pto_field(self.h, n, _dp(q), _dp(B), _dp(dB) if grad else None, _dp(V), _dp(E))
        return B, dB, V, E

    def collisions(self, segs, max_hits=8):
        s = np.ascontiguousarray(segs, dtype=np.float64).reshape(-1, 6)
        n = len(s)
        cnt = np.zeros(n, np.int32)
        ss, nn, sid, dn = np.zeros((n, max_hits)), np.zeros((n, max_hits, 3)), np.zeros((n, max_hits), np.int32), np.zeros((n, max_hits))
        lib().pto_segment_collisions(self.h, n, _dp(s), max_hits, cnt.ctypes.data_as(A.c_int32_p), _dp(ss), _dp(nn),
                                     sid.ctypes.data_as(A.c_int32_p), _dp(dn))
        return cnt, ss, nn, sid, dn

    def point_solids(self, pts):
        p = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
        m = np.zeros(len(p), np.uint64)
        lib().pto_point_solids(self.h, len(p), _dp(p), m.ctypes.data_as(A.c_uint64_p))
        return m


def mr(what, v, normal, Estep, b, w, transmit=False, integral=False, theta=0.0, phi=0.0):
    """MicroRoughness of one wall contact: what = "dist" (MRDist), "prob"
    (MRProb) or "max" (MRDistMax)"""
    v = np.ascontiguousarray(v, dtype=np.float64)
    n = np.ascontiguousarray(normal, dtype=np.float64)
    k = {"dist": 0, "prob": 1, "max": 2}[what]
    return lib().pto_mr(k, int(transmit), int(integral), _dp(v), _dp(n), Estep, b, w, theta, phi)


def spline1d_calc(x, y, pts):
    """the oracle's cubic spline through (x, y) (spline1dbuildcubic) at pts (spline1dcalc)"""
    x, y, p = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, pts))
    out = np.zeros_like(p)
    lib().pto_spline1d_calc(len(x), _dp(x), _dp(y), len(p), _dp(p), _dp(out))
    return out


def spline_derivs(x, y):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    d = np.zeros_like(x)
    lib().pto_spline_derivs(len(x), _dp(x), _dp(y), _dp(d))
    return d


def tricubic_coeff(x64):
    x = np.ascontiguousarray(x64, dtype=np.float64)
    a = np.zeros(64)
    lib().pto_tricubic_coeff(_dp(x), _dp(a))
    return a


def tricubic_eval(a64, x, y, z, dx=0, dy=0, dz=0):
    a = np.ascontiguousarray(a64, dtype=np.float64)
    o = np.zeros(1)
    lib().pto_tricubic_eval(_dp(a), x, y, z, dx, dy, dz, _dp(o))
    return o[0]


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().pto_philox4x32_10(c, k, o)
    return list(o)
