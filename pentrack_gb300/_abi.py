"""ctypes mirror of include/pentrack_gpu.h (the engine's C ABI)."""
import ctypes as C

c_double_p = C.POINTER(C.c_double)
c_int32_p = C.POINTER(C.c_int32)
c_int64_p = C.POINTER(C.c_int64)
c_uint64_p = C.POINTER(C.c_uint64)

PT_OK = 0
STATUS = {
    0: "PT_OK", -1: "PT_ERR_INVALID", -2: "PT_ERR_UNSUPPORTED", -3: "PT_ERR_OOM", -4: "PT_ERR_CUDA",
    -5: "PT_ERR_TIMEOUT", -6: "PT_ERR_CANCELLED", -7: "PT_ERR_IO", -8: "PT_ERR_NO_DEVICE",
}
PT_ERR_INVALID, PT_ERR_UNSUPPORTED, PT_ERR_OOM, PT_ERR_CUDA, PT_ERR_TIMEOUT = -1, -2, -3, -4, -5
PT_ERR_CANCELLED, PT_ERR_IO, PT_ERR_NO_DEVICE = -6, -7, -8

# stop IDs: include/globals.h:13-23 of the reference
ID_UNKNOWN, ID_NOT_FINISH, ID_HIT_BOUNDARIES, ID_ODEINT_ERROR, ID_DECAYED = 0, -1, -2, -3, -4
ID_INITIAL_NOT_FOUND, ID_CGAL_ERROR, ID_GEOMETRY_ERROR = -5, -6, -7
ID_ABSORBED_IN_MATERIAL, ID_ABSORBED_ON_SURFACE = 1, 2

NEUTRON, PROTON, ELECTRON = 0, 1, 2
FIELD_TAB3D, FIELD_HARMONIC, FIELD_UNIFORM_E, FIELD_SOLENOID, FIELD_TAB2D = 1, 2, 3, 4, 5
MODE_PLAIN, MODE_BATCHED, MODE_PHASED = 0, 1, 2
PREC_FP64, PREC_FP32 = 0, 1
SCHED_AUTO, SCHED_PHASED, SCHED_PERSISTENT, SCHED_PERSISTENT_WIDE, SCHED_PHASED_WIDE = 0, 1, 2, 3, 4


class Material(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "fermi_real", "fermi_imag", "diff_prob", "spinflip_prob", "rms_roughness", "correl_length",
        "internal_bfield", "modified_lambert_prob", "loss_per_bounce")]


class Solid(C.Structure):
    _fields_ = [("id", C.c_uint32), ("material", C.c_int32), ("n_ignore", C.c_int32), ("reserved", C.c_int32),
                ("ignore_times", c_double_p)]


class Field(C.Structure):
    _fields_ = [
        ("type", C.c_int32), ("reserved0", C.c_int32),
        ("b_scale", C.c_double), ("e_scale", C.c_double),
        ("xmax", C.c_double), ("xmin", C.c_double), ("ymax", C.c_double), ("ymin", C.c_double),
        ("zmax", C.c_double), ("zmin", C.c_double), ("boundary_width", C.c_double),
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("reserved1", C.c_int32),
        ("x", c_double_p), ("y", c_double_p), ("z", c_double_p),
        ("bx", c_double_p), ("by", c_double_p), ("bz", c_double_p), ("v", c_double_p),
        ("offset", C.c_double * 3), ("n_coeff", C.c_int32), ("reserved2", C.c_int32),
        ("l", c_int32_p), ("m", c_int32_p), ("g", c_double_p),
        ("e", C.c_double * 3),
        ("sol_radius", C.c_double), ("sol_half_length", C.c_double), ("sol_bcenter", C.c_double),
        ("er", c_double_p), ("ephi", c_double_p), ("ez", c_double_p),
    ]


class SceneDesc(C.Structure):
    _fields_ = [
        ("n_triangles", C.c_int64), ("triangles", c_double_p), ("triangle_solid", c_int32_p),
        ("n_solids", C.c_int32), ("n_materials", C.c_int32),
        ("solids", C.POINTER(Solid)), ("materials", C.POINTER(Material)),
        ("n_fields", C.c_int32), ("reserved", C.c_int32), ("fields", C.POINTER(Field)),
    ]


class RunParams(C.Structure):
    _fields_ = [
        ("species", C.c_int32), ("mode", C.c_int32), ("field_precision", C.c_int32), ("flipspin", C.c_int32),
        ("simtime", C.c_double), ("tau", C.c_double), ("tmax", C.c_double), ("lmax", C.c_double), ("bmax", C.c_double),
        ("n_spintimes", C.c_int32), ("steps_per_launch", C.c_int32), ("spintimes", c_double_p),
        ("seed", C.c_uint64), ("block_size", C.c_int32), ("max_launches", C.c_int32), ("timeout_s", C.c_double),
        ("max_run", C.c_int32), ("period_iters", C.c_int32), ("scheduler", C.c_int32), ("reserved3", C.c_int32),
        ("hitlog", C.c_int32), ("snapshotlog", C.c_int32), ("snapshots", c_double_p), ("n_snapshots", C.c_int32),
        ("reserved4", C.c_int32), ("log_capacity", C.c_int64),
        ("tracklog", C.c_int32), ("reserved5", C.c_int32), ("trackloginterval", C.c_double),
        ("spinlog", C.c_int32), ("reserved6", C.c_int32), ("spinloginterval", C.c_double),
        ("interpolatefields", C.c_int32), ("reserved7", C.c_int32),
    ]


class Particles(C.Structure):
    _fields_ = [
        ("n", C.c_int64), ("id", c_int64_p), ("t", c_double_p), ("y", c_double_p), ("spin", c_double_p),
        ("stop_id", c_int32_p), ("solid", c_int32_p), ("n_hit", c_int32_p), ("n_step", c_int32_p),
        ("n_spinflip", c_int32_p), ("reserved", c_int32_p),
        ("h_max", c_double_p), ("noflip_prob", c_double_p), ("tau", c_double_p), ("h_start", c_double_p),
        ("n_accepted", c_int64_p), ("n_rejected", c_int64_p),
    ]


SOURCE_BOX, SOURCE_CYLINDER, SOURCE_SOLID, SOURCE_SURFACE_CYLINDER, SOURCE_SURFACE_STL = 0, 1, 2, 3, 4
LOG_HIT, LOG_SNAPSHOT, LOG_TRACK, LOG_SPIN = 0, 1, 2, 3
HIT_RECORD, SNAPSHOT_RECORD, TRACK_RECORD, SPIN_RECORD = 18, 22, 10, 14


class SourceParams(C.Structure):
    _fields_ = [
        ("species", C.c_int32), ("shape", C.c_int32), ("seed", C.c_uint64),
        ("lo", C.c_double * 3), ("hi", C.c_double * 3),
        ("rmin", C.c_double), ("rmax", C.c_double), ("phimin", C.c_double), ("phimax", C.c_double),
        ("zmin", C.c_double), ("zmax", C.c_double),
        ("solid", C.c_int32), ("phase_space", C.c_int32),
        ("emin", C.c_double), ("emax", C.c_double), ("polarization", C.c_double), ("tmin", C.c_double),
        ("tmax", C.c_double), ("thetamin", C.c_double), ("thetamax", C.c_double), ("phimin_v", C.c_double),
        ("phimax_v", C.c_double), ("n_min_samples", C.c_int64), ("max_rounds", C.c_int32), ("reserved", C.c_int32),
        ("enormal", C.c_double), ("region", C.c_void_p),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("kernel_ms", C.c_double), ("span_ms", C.c_double), ("wall_ms", C.c_double), ("particle_seconds", C.c_double),
        ("launches", C.c_int64), ("active", C.c_int64),
        ("rk_accepted", C.c_int64), ("rk_rejected", C.c_int64), ("rhs_evals", C.c_int64), ("field_evals", C.c_int64),
        ("hits", C.c_int64), ("bisection_levels", C.c_int64),
        ("bvh_nodes", C.c_int64), ("tri_tests", C.c_int64), ("subsegments", C.c_int64), ("dense_evals", C.c_int64),
        ("dominant_kernel_ms", C.c_double), ("dominant_launches", C.c_int64), ("dominant_kernel", C.c_char * 48),
        ("try_ms", C.c_double), ("post_ms", C.c_double), ("slow_ms", C.c_double),
        ("bisect_max", C.c_int64),
        ("cand_calls", C.c_int64), ("cand_overflow", C.c_int64), ("cand_sum", C.c_int64), ("tri32_tests", C.c_int64),
        ("bisect_ms", C.c_double), ("bisect_dead", C.c_int64), ("spin_steps", C.c_int64), ("tail_ms", C.c_double), ("aux_launches", C.c_int64),
        ("graph_launches", C.c_int64), ("sched_outer_iters", C.c_int64), ("sched_inner_iters", C.c_int64),
        ("adj_forward_ms", C.c_double), ("adj_reverse_ms", C.c_double),
        ("scheduler", C.c_int64), ("tune_ns_per_try", C.c_double * 4),
    ]

    def as_dict(self):
        d = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            if isinstance(v, bytes):
                v = v.decode()
            elif hasattr(v, "_length_"):
                v = list(v)
            d[name] = v
        return d


def declare(lib):
    """Attach argument/return types of every exported entry point."""
    P = C.POINTER
    vp = C.c_void_p
    sig = {
        "pt_create": (C.c_int32, [P(SceneDesc), C.c_int32, P(vp)]),
        "pt_destroy": (None, [vp]),
        "pt_last_error": (C.c_char_p, [vp]),
        "pt_cancel": (C.c_int32, [vp]),
        "pt_integrate": (C.c_int32, [vp, P(RunParams), P(Particles), P(Particles), P(Stats)]),
        "pt_batch_create": (C.c_int32, [vp, P(RunParams), P(Particles), P(vp)]),
        "pt_batch_advance": (C.c_int32, [vp, vp, C.c_double, P(Stats)]),
        "pt_batch_advance_steps": (C.c_int32, [vp, vp, C.c_double, C.c_int32, P(Stats)]),
        "pt_batch_read": (C.c_int32, [vp, vp, P(Particles)]),
        "pt_batch_destroy": (None, [vp]),
        "pt_field_eval": (C.c_int32, [vp, C.c_int64, c_double_p, C.c_int32, c_double_p, c_double_p, c_double_p, c_double_p]),
        "pt_segment_collisions": (C.c_int32, [vp, C.c_int64, c_double_p, C.c_int32, c_int32_p, c_double_p, c_double_p,
                                              c_int32_p, c_double_p]),
        "pt_adjoint": (C.c_int32, [vp, P(RunParams), P(Particles), C.c_int32, C.c_int32, c_double_p, c_double_p,
                                   c_double_p, P(Particles), P(Stats)]),
        "pt_segment_collisions_noalloc": (C.c_int32, [vp, C.c_int64, c_double_p, C.c_int32, c_int32_p, c_double_p,
                                                      c_double_p, c_int32_p, c_double_p]),
        "pt_point_solids": (C.c_int32, [vp, C.c_int64, c_double_p, c_uint64_p]),
        "pt_source_volume": (C.c_int32, [vp, P(SourceParams), C.c_int64, c_int64_p, P(Particles), c_double_p]),
        "pt_mr_eval": (C.c_int32, [vp, C.c_int32, C.c_int32, C.c_int32, C.c_int64, c_double_p, c_double_p, c_double_p,
                                   c_double_p, c_double_p, c_double_p, c_double_p, c_double_p]),
        "pt_neutron_decay": (C.c_int32, [vp, C.c_uint64, C.c_int64, c_int64_p, c_double_p, c_double_p, P(Particles),
                                         P(Particles)]),
        "pt_integrate_secondaries": (C.c_int32, [vp, P(RunParams), P(RunParams), P(RunParams), P(Particles), P(Particles),
                                                 P(Particles), P(Particles), c_int64_p, P(Stats)]),
        "pt_log_read": (C.c_int32, [vp, C.c_int32, C.c_int64, c_double_p, c_int64_p]),
        "pt_probe_fp64": (C.c_int32, [vp, c_double_p]),
        "pt_version": (C.c_char_p, []),
        "pt_config_load": (C.c_int32, [C.c_char_p, P(vp)]),
        "pt_config_scene_desc": (P(SceneDesc), [vp]),
        "pt_config_free": (None, [vp]),
        "pt_config_run_params": (C.c_int32, [C.c_char_p, C.c_char_p, P(RunParams), c_double_p, C.c_int32]),
        "pt_config_error": (C.c_char_p, []),
        "pt_current_solid": (C.c_int32, [P(SceneDesc), C.c_int64, c_uint64_p, c_double_p, c_int32_p]),
        "pt_endlog_write": (C.c_int32, [C.c_char_p, C.c_int64, C.c_int32, P(SceneDesc), P(Particles), P(Particles),
                                        c_double_p, c_double_p, c_int32_p, c_double_p, c_double_p, c_int32_p,
                                        C.c_char_p]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return sig
