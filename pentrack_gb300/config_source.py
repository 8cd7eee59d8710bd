"""The [SOURCE] section of a PENTrack config.in as a particle generator.

CreateParticleSource (src/source.cpp:204-229) picks the source by
`sourcemode` (boxvolume, cylvolume, STLvolume, cylsurface, STLsurface);
TParticleSource (src/source.cpp:18-84) reads the particle type, ActiveTime
with optional pulseGap / pulseWidth (a piecewise-constant start-time
distribution), polarization, and the distributions `spectrum` on
[Emin, Emax], `phi_v` on [phi_v_min, phi_v_max] and `theta_v` on
[theta_v_min, theta_v_max] (degrees), each an ExprTk formula in x turned
into a piecewise-linear distribution (parse_distribution,
include/mc.h:281-335).  The formulas are evaluated here by a restricted
expression evaluator (numbers, x, + - * / ^, parentheses, the usual
functions, pi, and the reference's ProtonBetaSpectrum, ElectronBetaSpectrum
and MaxwellBoltzSpectrum); their piecewise-linear tables use a fixed grid of
4,096 intervals.

Geometry-dependent parts go through callables: `inside_stl(triangles)`
returns the inside test of a source STL (normally an Engine on a scene that
holds only that solid), and PhaseSpaceWeighting needs `field`,
`point_solids` and the scene, as in sources.py.
"""
import ast
import math
import os

import numpy as np

from . import _abi as A
from . import scenes as S
from . import secondaries
from . import sources

SPECIES = {"neutron": A.NEUTRON, "proton": A.PROTON, "electron": A.ELECTRON}
CONV = S.PI / 180.0


def read_config(path):
    """TConfig::ReadFromFile (src/config.cpp:14-53): sections of `key rest of
    line`, comments after '#', a key defined twice in a section is an error."""
    cfg, sec = {}, None
    with open(path) as f:
        for line in f:
            s = line.strip(" \t\r\n")
            if not s:
                continue
            if s[0] == "[":
                sec = None if s[1:2] == "/" else (s[1:s.index("]")] if "]" in s else s[1:])
                if sec is not None:
                    cfg.setdefault(sec, {})
                continue
            if s[0] == "#" or sec is None:
                continue
            parts = s.split(None, 1)
            key, rest = parts[0], (parts[1] if len(parts) > 1 else "").split("#", 1)[0]
            if key in cfg[sec]:
                raise ValueError(f"Variable {key} in config file is ambiguous!")
            cfg[sec][key] = rest
    return cfg


# ---------------------------------------------------------------- formulas
_FUNCS = {"sqrt": np.sqrt, "exp": np.exp, "log": np.log, "log10": np.log10, "sin": np.sin, "cos": np.cos,
          "tan": np.tan, "asin": np.arcsin, "acos": np.arccos, "atan": np.arctan, "abs": np.abs, "pow": np.power,
          "min": np.minimum, "max": np.maximum, "sinh": np.sinh, "cosh": np.cosh, "tanh": np.tanh,
          "ProtonBetaSpectrum": secondaries.proton_beta_spectrum, "ElectronBetaSpectrum": S.electron_beta_spectrum}
_CONSTS = {"pi": math.pi, "e": math.e}
BOLTZ = 8.617343e-5  # boltzconst [eV/K], include/globals.h


def maxwell_boltz_spectrum(T, E):
    """MaxwellBoltzSpectrum (src/globals.cpp:106-109), normalised to its maximum"""
    kT = BOLTZ * T
    return 2 * np.sqrt(E / S.PI) / np.sqrt(kT * kT * kT) * np.exp(-E / kT) / (2 * np.sqrt(0.5 / S.PI) / kT * np.exp(-0.5))


_FUNCS["MaxwellBoltzSpectrum"] = maxwell_boltz_spectrum


def formula(expr):
    """f(x) for an ExprTk-style formula in x ('^' is the power operator);
    anything but numbers, x, the listed functions and constants and
    arithmetic is refused."""
    tree = ast.parse(expr.replace("^", "**").strip(), mode="eval")
    allowed = (ast.Expression, ast.BinOp, ast.UnaryOp, ast.Call, ast.Name, ast.Constant, ast.Load, ast.Add, ast.Sub,
               ast.Mult, ast.Div, ast.Pow, ast.USub, ast.UAdd, ast.Mod)
    for node in ast.walk(tree):
        if not isinstance(node, allowed):
            raise ValueError(f"unsupported element {type(node).__name__} in formula '{expr}'")
        if isinstance(node, ast.Call) and not (isinstance(node.func, ast.Name) and node.func.id in _FUNCS):
            raise ValueError(f"unknown function in formula '{expr}'")
        if isinstance(node, ast.Name) and node.id not in _FUNCS and node.id not in _CONSTS and node.id != "x":
            raise ValueError(f"unknown name '{node.id}' in formula '{expr}'")
        if isinstance(node, ast.Constant) and not isinstance(node.value, (int, float)):
            raise ValueError(f"unsupported constant in formula '{expr}'")
    code = compile(tree, "<formula>", "eval")

    def f(x):
        env = dict(_CONSTS)
        env.update(_FUNCS)
        env["x"] = np.asarray(x, dtype=np.float64)
        return np.broadcast_to(np.asarray(eval(code, {"__builtins__": {}}, env), dtype=np.float64), env["x"].shape)
    return f


def distribution(expr, lo, hi, n=4096):
    """Inverse CDF u -> x of the piecewise-linear distribution of the formula
    on [lo, hi] (a constant 1 when the formula is empty)."""
    if hi <= lo:
        return lambda u: np.full(np.shape(u), lo, dtype=np.float64)
    x = np.linspace(lo, hi, n + 1)
    w = np.ones_like(x) if not expr.strip() else np.maximum(formula(expr)(x), 0.0)
    seg = 0.5 * (w[1:] + w[:-1]) * np.diff(x)
    cdf = np.concatenate([[0.0], np.cumsum(seg)])
    if cdf[-1] <= 0:
        raise ValueError(f"formula '{expr}' has no positive weight on [{lo}, {hi}]")
    cdf /= cdf[-1]

    total = seg.sum()

    def inv(u):
        # within interval k the weight is w0 + m t (0 <= t <= dx); the mass
        # c up to t solves m t^2 / 2 + w0 t = c, taken in its stable form
        u = np.asarray(u, dtype=np.float64)
        k = np.clip(np.searchsorted(cdf, u, side="right") - 1, 0, n - 1)
        c = np.maximum(u - cdf[k], 0.0) * total
        w0, dx = w[k], x[k + 1] - x[k]
        m = (w[k + 1] - w0) / dx
        den = w0 + np.sqrt(np.maximum(w0 * w0 + 2 * m * c, 0.0))
        with np.errstate(invalid="ignore", divide="ignore"):
            t = np.where(den > 0, 2 * c / den, 0.0)
        return x[k] + np.clip(t, 0.0, dx)
    return inv


def time_distribution(active, gap=0.0, width=0.0):
    """The start-time distribution of TParticleSource (src/source.cpp:40-84):
    all at 0, uniform over ActiveTime, or pulses of `width` every `gap`."""
    if active == 0:
        return lambda u: np.zeros(np.shape(u))
    if gap > 0 and active > 0:
        edges = []
        i = 0.0
        while i < active:
            if width == 0:
                edges.append((i, np.nextafter(i, np.inf), 1.0))
            elif i + width > active:
                edges.append((i, active, (active - i) / width))
            else:
                edges.append((i, i + width, 1.0))
            i += gap
        lo = np.array([e[0] for e in edges])
        hi = np.array([e[1] for e in edges])
        p = np.array([e[2] for e in edges])  # piecewise-constant density: weight per unit time
        mass = p * (hi - lo)
        cum = np.concatenate([[0.0], np.cumsum(mass)])
        cum /= cum[-1]

        def inv(u):
            u = np.asarray(u, dtype=np.float64)
            k = np.clip(np.searchsorted(cum, u, side="right") - 1, 0, len(lo) - 1)
            f = (u - cum[k]) / np.where(cum[k + 1] > cum[k], cum[k + 1] - cum[k], 1.0)
            return lo[k] + f * (hi[k] - lo[k])
        return inv
    return lambda u: np.asarray(u, dtype=np.float64) * active


# ---------------------------------------------------------------- sources
def _floats(s, n):
    v = [float(x) for x in s.split()[:n]]
    return v + [0.0] * (n - len(v))


def source_from_config(config_path, n, seed, first_id=0, inside_stl=None, scene=None, field=None, point_solids=None):
    """(species, ParticleSet) of n particles from the config's [SOURCE]
    section, ids first_id .. first_id + n - 1."""
    cfg = read_config(config_path)
    sc = cfg.get("SOURCE", {})
    get = lambda k, d="": sc.get(k, d).strip()
    mode = get("sourcemode").split()[0] if get("sourcemode") else ""
    kind = SPECIES.get(get("particle").split()[0] if get("particle") else "neutron")
    if kind is None:
        raise ValueError(f"unsupported particle '{get('particle')}'")
    ids = np.arange(first_id, first_id + n, dtype=np.int64)
    emin, emax = float(get("Emin", "0") or 0), float(get("Emax", "0") or 0)
    spec = distribution(get("spectrum"), emin, emax)
    phi_d = distribution(get("phi_v"), float(get("phi_v_min", "0") or 0) * CONV, float(get("phi_v_max", "0") or 0) * CONV)
    th_d = distribution(get("theta_v"), float(get("theta_v_min", "0") or 0) * CONV,
                        float(get("theta_v_max", "0") or 0) * CONV)
    pol = float(get("polarization", "0") or 0)
    tdist = time_distribution(float(get("ActiveTime", "0") or 0),
                              float(get("pulseGap", "0") or 0) if "pulseWidth" in sc and "pulseGap" in sc else 0.0,
                              float(get("pulseWidth", "0") or 0) if "pulseWidth" in sc and "pulseGap" in sc else 0.0)
    draw = lambda k, sel=ids: S._draw(seed, sel, k)
    spectrum = lambda sd, sel, k=4: spec(S._draw(sd, sel, k))
    stl = None
    if mode in ("STLvolume", "STLsurface"):
        path = get("STLfile").split()[0]
        path = path if os.path.isabs(path) else os.path.join(os.path.dirname(os.path.abspath(config_path)), path)
        stl = S.read_stl(path)
        if inside_stl is None:
            raise ValueError("STL sources need inside_stl (the inside test of the source solid)")
    if mode in ("boxvolume", "cylvolume", "STLvolume"):
        if mode == "boxvolume":
            x0, x1, y0, y1, z0, z1 = _floats(get("parameters"), 6)
            rp = sources.box_points((x0, y0, z0), (x1, y1, z1))
        elif mode == "cylvolume":
            r0, r1, p0, p1, z0, z1 = _floats(get("parameters"), 6)
            rp = sources.cylinder_points(r0, r1, z0, z1, p0 * CONV, p1 * CONV)
        else:
            rp = sources.stl_points(stl, inside_stl(stl))
        if int(float(get("PhaseSpaceWeighting", "0") or 0)):
            if scene is None or field is None or point_solids is None:
                raise ValueError("PhaseSpaceWeighting needs the scene, field and point_solids")
            V = sources.rest_energy_potential(scene, kind, field, point_solids)
            parts, _ = sources.phase_space_volume_source(
                seed, ids, rp, V, emin, emax, spectrum=spectrum, polarization=pol, species=kind,
                direction=lambda sd, sel: (phi_d(S._draw(sd, sel, 5)), th_d(S._draw(sd, sel, 6))),
                times=lambda sd, sel, k: tdist(S._draw(sd, sel, k)))
            return kind, parts
        pos = rp(seed, ids, sources._point_base(0))
        E, ph, th = spec(draw(4)), phi_d(draw(5)), th_d(draw(6))
        p = np.where(draw(3) < 0.5 * (pol + 1), 1.0, -1.0)
        parts = S.make_particles(seed, ids, pos, E, ph, th, p, species=kind)
        parts.t[:] = tdist(draw(7))
        return kind, parts
    if mode in ("cylsurface", "STLsurface"):
        if scene is None:
            raise ValueError("surface sources need the scene")
        if mode == "cylsurface":
            r0, r1, p0, p1, z0, z1 = _floats(get("parameters"), 6)
            inside, box = sources.cylinder_region(r0, r1, z0, z1, p0 * CONV, p1 * CONV)
        else:
            t = np.asarray(stl).reshape(-1, 3, 3)
            inside, box = inside_stl(stl), (t.min(axis=(0, 1)), t.max(axis=(0, 1)))
        parts = sources.surface_source(seed, ids, scene, inside, box, emin, emax,
                                       enormal=float(get("Enormal", "0") or 0), polarization=pol, spectrum=spectrum,
                                       species=kind)
        parts.t[:] = tdist(draw(7))
        return kind, parts
    raise ValueError(f"Could not load source {mode}!")
