"""End-of-track log in the reference's text layout.

TLogger::Print with the suffix "end" (src/logger.cpp:42-126) collects, per
tracked particle, its start and end states with energies, field values,
solids and counters; TTextLogger::DoLog (src/logger.cpp:314-334) writes them
to <jobnumber, 12 digits><particle name>end.out: one header line of the
variable names, then one line per particle, every value written with 15
significant digits and followed by a space.  The variables and their default
order are the reference's; `logvars` selects a subset by name (the
reference's ExprTk formulas and logfilter are not evaluated here).

The energies follow TParticle::GetKineticEnergy / GetPotentialEnergy
(src/particle.cpp:237-269) plus TNeutron's material potential
(src/neutron.cpp:378-380) with the same operations as the kernels, and the
start and end solids are point queries at the logged positions, as
geom.GetSolid is in the reference's Print.  Fields and solids come from
callables, normally Engine.field and Engine.point_solids.
"""
import os

import numpy as np

from . import _abi as A

END_TITLES = ("jobnumber", "particle",
              "tstart", "xstart", "ystart", "zstart", "vxstart", "vystart", "vzstart", "polstart",
              "Sxstart", "Systart", "Szstart", "Hstart", "Estart", "Bstart", "Ustart", "solidstart",
              "tend", "xend", "yend", "zend", "vxend", "vyend", "vzend", "polend",
              "Sxend", "Syend", "Szend", "Hend", "Eend", "Bend", "Uend",
              "solidend", "stopID", "Nspinflip", "spinflipprob", "Nhit", "Nstep", "propert", "trajlength", "Hmax", "wL")

SPECIES_NAME = {A.NEUTRON: "neutron", A.PROTON: "proton", A.ELECTRON: "electron"}

_CONSTANTS = None


def species_constants(kind):
    """Mass, charge, magnetic moment and the derived energy constants of a
    species, read from include/pt_constants.h (the values the kernels use)."""
    global _CONSTANTS
    if _CONSTANTS is None:
        path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "pt_constants.h")
        _CONSTANTS = {}
        with open(path) as f:
            for line in f:
                parts = line.split()
                if len(parts) >= 3 and parts[0] == "#define" and parts[1].startswith("PT_"):
                    try:
                        _CONSTANTS[parts[1]] = float.fromhex(parts[2])
                    except ValueError:
                        pass
    pre = "PT_" + SPECIES_NAME[kind].upper() + "_"
    return {k: _CONSTANTS[pre + k.upper()] for k in ("m", "q", "mu", "mu_over_e", "q_over_e", "mc2", "mg")}


def kinetic_energy(kind, v):
    """TParticle::GetKineticEnergy [eV] of velocities v (3, n)."""
    c = species_constants(kind)
    beta2 = (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) / _CONSTANTS["PT_C0_SQ"]
    b4 = beta2 * beta2
    series = (0.5 + (3.0 / 8.0 + (5.0 / 16.0 + 35.0 / 128.0 * beta2) * beta2) * beta2) * beta2
    with np.errstate(invalid="ignore", divide="ignore"):
        exact = 1.0 / np.sqrt(1.0 - beta2) - 1.0
    return c["mc2"] * np.where(b4 * b4 * beta2 < 2.220446049250313e-16, series, exact)


def potential_energy(scene, kind, y, B, V, solid_index):
    """TParticle::GetPotentialEnergy [eV] (+ the material potential of the
    solid for neutrons) for states y (9, n), fields B (n, 3), V (n)."""
    c = species_constants(kind)
    r = np.zeros(y.shape[1])
    if c["mu"] != 0:
        r = r + (-y[7] * c["mu_over_e"]) * np.sqrt(B[:, 0] * B[:, 0] + B[:, 1] * B[:, 1] + B[:, 2] * B[:, 2])
    if c["q"] != 0:
        r = r + c["q_over_e"] * V
    r = r + c["mg"] * y[2]
    if kind == A.NEUTRON:
        mats = np.array([scene.materials[s["material"]] for s in scene.solids], dtype=np.float64)
        fermi, bint = mats[solid_index, 0], mats[solid_index, 6]
        r = r + (fermi * 1e-9 - bint * c["mu_over_e"] * y[7])
    return r


def current_solid(scene, masks, t):
    """Index of the solid a point belongs to (TGeometry::GetSolid): the default
    solid plus every solid whose bit is set in `masks` (Engine.point_solids),
    in index order, the highest ID among those not ignored at time t winning
    (TTracker::GetCurrentsolid's rule)."""
    n = len(masks)
    ids = np.array([s["id"] for s in scene.solids])
    best = np.zeros(n, dtype=np.int64)
    best_ign = np.zeros(n, dtype=bool)
    masks = np.asarray(masks, dtype=np.uint64)
    for s in range(1, len(scene.solids)):
        inside = (masks >> np.uint64(s)) & np.uint64(1) == np.uint64(1)
        ign = np.zeros(n, dtype=bool)
        for t0, t1 in scene.solids[s]["ignore"]:
            ign |= (t >= t0) & (t < t1)
        take = inside & (best_ign | (~ign & (ids[best] < ids[s])))
        best = np.where(take, s, best)
        best_ign = np.where(take, ign, best_ign)
    return best


def end_variables(scene, kind, start, end, field, point_solids, jobnumber=0, particle=None):
    """Every variable of the end log, name -> array over particles.  `start`
    and `end` are ParticleSets (the tracked inputs and pt_integrate's outputs),
    `field(xyzt)` returns (B, dB, V, E) and `point_solids(p)` the solid masks;
    `particle` defaults to id + 1 (the reference numbers particles from 1)."""
    n = start.n
    c = species_constants(kind)
    ids = np.array([s["id"] for s in scene.solids])

    def at(t, y):
        B, _, V, _ = field(np.column_stack([y[0], y[1], y[2], t]))
        sidx = current_solid(scene, point_solids(np.ascontiguousarray(y[0:3].T)), t)
        return B, V, sidx

    B0, V0, s0 = at(start.t, start.y)
    B1, V1, s1 = at(end.t, end.y)
    E0, E1 = kinetic_energy(kind, start.y[3:6]), kinetic_energy(kind, end.y[3:6])
    H0 = E0 + potential_energy(scene, kind, start.y, B0, V0, s0)
    H1 = E1 + potential_energy(scene, kind, end.y, B1, V1, s1)
    with np.errstate(invalid="ignore", divide="ignore"):
        wl = np.where(end.spin[3] > 0, end.spin[4] / np.where(end.spin[3] > 0, end.spin[3], 1.0), 0.0)
    v = {"jobnumber": np.full(n, float(jobnumber)),
         "particle": (start.id + 1).astype(np.float64) if particle is None else np.asarray(particle, np.float64),
         "m": np.full(n, c["m"]), "q": np.full(n, c["q"]), "mu": np.full(n, c["mu"]),
         "tstart": start.t, "Hstart": H0, "Estart": E0, "Bstart": np.sqrt((B0 * B0).sum(1)), "Ustart": V0,
         "solidstart": ids[s0].astype(np.float64),
         "tend": end.t, "Hend": H1, "Eend": E1, "Bend": np.sqrt((B1 * B1).sum(1)), "Uend": V1,
         "solidend": ids[s1].astype(np.float64),
         "stopID": end.stop_id.astype(np.float64), "Nspinflip": end.n_spinflip.astype(np.float64),
         "spinflipprob": 1 - end.noflip_prob, "Nhit": end.n_hit.astype(np.float64),
         "Nstep": end.n_step.astype(np.float64), "propert": end.y[6], "trajlength": end.y[8],
         "Hmax": end.h_max, "wL": wl}
    for k, name in enumerate(("x", "y", "z", "vx", "vy", "vz")):
        v[name + "start"] = start.y[k]
        v[name + "end"] = end.y[k]
    v["polstart"], v["polend"] = start.y[7], end.y[7]
    for k, name in enumerate(("Sx", "Sy", "Sz")):
        v[name + "start"] = start.spin[k]
        v[name + "end"] = end.spin[k]
    return v


def write_log(directory, jobnumber, particle_name, suffix, titles, columns):
    """TTextLogger::DoLog for a whole table: the header and one row per
    particle, values as C++ streams write doubles at precision 15."""
    path = os.path.join(directory, f"{int(jobnumber):012d}{particle_name}{suffix}.out")
    cols = [np.asarray(c, dtype=np.float64) for c in columns]
    with open(path, "w") as f:
        f.write("".join(t + " " for t in titles) + "\n")
        for row in zip(*cols):
            f.write("".join("%.15g " % x for x in row) + "\n")
    return path


def write_endlog(directory, scene, kind, start, end, field, point_solids, jobnumber=0, logvars=None, particle=None):
    """The end log of one species' particles; `logvars` (names, as the
    config's endlogvars) selects and orders the columns.  Returns the path."""
    v = end_variables(scene, kind, start, end, field, point_solids, jobnumber, particle)
    titles = tuple(logvars) if logvars else END_TITLES
    unknown = [t for t in titles if t not in v]
    if unknown:
        raise ValueError(f"end log variables not available (formulas are not evaluated): {unknown}")
    return write_log(directory, jobnumber, SPECIES_NAME[kind], "end", titles, [v[t] for t in titles])


HIT_TITLES = ("jobnumber", "particle", "t", "x", "y", "z", "v1x", "v1y", "v1z", "pol1", "v2x", "v2y", "v2z", "pol2",
              "nx", "ny", "nz", "solid1", "solid2")


def write_hitlog(directory, kind, records, jobnumber=0):
    """The hit log (TLogger::PrintHit, src/logger.cpp:202-235) from the hit
    records of Engine.read_log(LOG_HIT): one row per hit that changed the
    particle's solid, in the order of the records (by particle, then time);
    particle numbers as in the end log (id + 1).  Returns the path."""
    r = np.asarray(records, dtype=np.float64).reshape(-1, 18)
    cols = [np.full(len(r), float(jobnumber)), r[:, 0] + 1] + [r[:, k] for k in range(1, 18)]
    return write_log(directory, jobnumber, SPECIES_NAME[kind], "hit", HIT_TITLES, cols)


TRACK_TITLES = ("jobnumber", "particle", "polarisation", "t", "x", "y", "z", "vx", "vy", "vz", "H", "E",
                "Bx", "dBxdx", "dBxdy", "dBxdz", "By", "dBydx", "dBydy", "dBydz", "Bz", "dBzdx", "dBzdy", "dBzdz",
                "Ex", "Ey", "Ez", "V")


def write_tracklog(directory, scene, kind, records, field, jobnumber=0):
    """The track log (TLogger::PrintTrack, src/logger.cpp:143-200) from the
    track records of Engine.read_log(LOG_TRACK): per record the state, the
    field and its Jacobian, E and V there, and the kinetic and total energy
    (with the potential of the recorded current solid).  Returns the path."""
    r = np.asarray(records, dtype=np.float64).reshape(-1, 10)
    n = len(r)
    y = np.zeros((9, n))
    y[0:6] = r[:, 2:8].T
    y[7] = r[:, 8]
    B, dB, V, E = field(np.column_stack([y[0], y[1], y[2], r[:, 1]]))
    index = {int(s["id"]): k for k, s in enumerate(scene.solids)}
    sidx = np.array([index[int(i)] for i in r[:, 9]], dtype=np.int64)
    Ek = kinetic_energy(kind, y[3:6])
    H = Ek + potential_energy(scene, kind, y, B, V, sidx)
    cols = [np.full(n, float(jobnumber)), r[:, 0] + 1, y[7], r[:, 1], y[0], y[1], y[2], y[3], y[4], y[5], H, Ek]
    for i in range(3):
        cols += [B[:, i], dB[:, i, 0], dB[:, i, 1], dB[:, i, 2]]
    cols += [E[:, 0], E[:, 1], E[:, 2], V]
    return write_log(directory, jobnumber, SPECIES_NAME[kind], "track", TRACK_TITLES, cols)


SPIN_TITLES = ("jobnumber", "particle", "t", "x", "y", "z", "Sx", "Sy", "Sz", "Wx", "Wy", "Wz", "Bx", "By", "Bz")


def write_spinlog(directory, kind, records, jobnumber=0):
    """The spin log (TLogger::PrintSpin, src/logger.cpp:237-284) from the
    spin records of Engine.read_log(LOG_SPIN).  Returns the path."""
    r = np.asarray(records, dtype=np.float64).reshape(-1, 14)
    cols = [np.full(len(r), float(jobnumber)), r[:, 0] + 1] + [r[:, k] for k in range(1, 14)]
    return write_log(directory, jobnumber, SPECIES_NAME[kind], "spin", SPIN_TITLES, cols)


def snapshot_states(start, records):
    """(start subset, ParticleSet at the snapshots) from snapshot records of
    Engine.read_log(LOG_SNAPSHOT): for each record the particle's start state
    and its state, spin and counters at the snapshot time."""
    from .engine import ParticleSet
    r = np.asarray(records, dtype=np.float64).reshape(-1, 22)
    index = {int(i): k for k, i in enumerate(start.id)}
    rows = np.array([index[int(i)] for i in r[:, 0]], dtype=np.int64)
    st = start.subset(rows)
    snap = ParticleSet(len(r), st.id.copy(), r[:, 1].copy(), r[:, 2:11].T.copy(), r[:, 11:16].T.copy())
    snap.stop_id[:] = r[:, 16]
    snap.n_spinflip[:] = r[:, 17]
    snap.noflip_prob[:] = r[:, 18]
    snap.n_hit[:] = r[:, 19]
    snap.n_step[:] = r[:, 20]
    snap.h_max[:] = r[:, 21]
    return st, snap


def write_snapshotlog(directory, scene, kind, start, records, field, point_solids, jobnumber=0, logvars=None):
    """The snapshot log (TLogger::PrintSnapshot -> Print(..., "snapshot"),
    src/logger.cpp:128-141): the end log's columns with the state at each
    snapshot time in place of the end state.  Returns the path."""
    st, snap = snapshot_states(start, records)
    v = end_variables(scene, kind, st, snap, field, point_solids, jobnumber)
    titles = tuple(logvars) if logvars else END_TITLES
    return write_log(directory, jobnumber, SPECIES_NAME[kind], "snapshot", titles, [v[t] for t in titles])


def log_settings(config_path, particle_name, suffix="end"):
    """(enabled, logvars) of one log from a config.in: `<suffix>log` and
    `<suffix>logvars` of [PARTICLES], overridden by the particle's own
    section (as TTracker reads the particle options, src/tracking.cpp:19-60);
    logvars None means the default columns."""
    from .config_source import read_config
    cfg = read_config(config_path)
    opts = dict(cfg.get("PARTICLES", {}))
    opts.update(cfg.get(particle_name, {}))
    on = opts.get(suffix + "log", "0").split()
    names = opts.get(suffix + "logvars", "").split()
    return bool(on) and float(on[0]) != 0, (names or None)

