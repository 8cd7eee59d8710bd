#!/usr/bin/env python3
"""Benchmark: particle-seconds tracked per second on the field-storage workload.

Workload (the configuration the headline metric is quoted on): 1e6 UCN per
GPU in a closed cylinder R = 0.2 m, H = 0.1 m (256 segments, 1,024 triangles),
64^3 tricubic table of the quadrupole |B| = 1.5 T r/0.2 m + 10 uT along z,
+-mu grad|B| force with 50/50 spin states, 250 neV walls with 5 % Lambert and
1e-4 loss per bounce, tau = 880 s, 0-250 neV isotropic, FP64 state.  One step
is one step-batch: every live particle advances a fixed number of accepted
RK steps (default 32) with all wall hits, decays and losses they contain;
results are bit-identical to one uninterrupted run.  Synthetic, seeded
inputs (no dataset).

  value     device time of the timed step-batches (inputs resident in HBM)
  e2e       pt_integrate on a fresh chunk of the workload from pinned host
            buffers over the same lab-time span as one step-batch, H2D/D2H
            and initialisation inside the timed region
  cpu       the oracle on all host cores over the same lab-time span

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-s tracked/s at stated energy drift: batched vs plain GPU form, 1 GB300"
SCHED_NAMES = ["autotuning", "phase split (168 registers)", "persistent (168 registers)", "persistent (255 registers)",
               "phase split (255 registers)"]
UNIT = "particle-s/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=None, help="particles per GPU (default 1e6; 1e7 for large_mesh)")
    p.add_argument("--workload", default="field_storage", choices=["field_storage", "large_mesh", "adjoint_spin"],
                   help="field_storage: the headline configuration; large_mesh: the 200k-triangle, 128^3 scale-up")
    p.add_argument("--batch-steps", type=int, default=32, help="accepted RK steps per particle per bench step")
    p.add_argument("--precision", default="fp32", choices=["fp64", "fp32"],
                   help="field evaluation: fp64, or fp32 = FP32 node table (linear base + FP32 Hermite remainder)")
    p.add_argument("--mode", default="batched", choices=["plain", "batched", "phased"],
                   help="batched: persistent lanes + device-scheduled CUDA graph; phased: host-driven phase split")
    p.add_argument("--scheduler", type=int, default=0, choices=[0, 1, 2, 3, 4],
                   help="batched/phased forms: 0 autotuned, 1 phase split, 2 persistent, 3 persistent (255 registers), "
                        "4 phase split (255 registers); the phased form uses the 255-register try kernel for 4")
    p.add_argument("--no-plain", action="store_true", help="skip the plain-form comparison run")
    p.add_argument("--no-phased", action="store_true", help="skip the host-driven phase-split comparison run")
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="target CPU time of the baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-fp64-line", action="store_true", help="skip the FP64-field batched sub-record")
    p.add_argument("--no-adjoint", action="store_true", help="skip the adjoint-spin forward / adjoint cost sub-record")
    p.add_argument("--e2e-steps", type=int, default=2)
    p.add_argument("--full-run", action="store_true",
                   help="field_storage: track --n UCN over the whole 200 s in the batched and the plain form (one call "
                        "each, to completion) instead of step-batches")
    p.add_argument("--spin-window", type=float, default=0.5,
                   help="adjoint_spin workload: lab time every particle advances per bench step (s)")
    return p.parse_args()


# ----------------------------------------------------------------------------
def pci_bus_id(device):
    """PCI bus ID of CUDA device `device` (cudaDeviceGetPCIBusId, read-only):
    nvidia-smi numbers GPUs in PCI order and ignores CUDA_VISIBLE_DEVICES, so
    the clock sampler selects the GPU by bus ID."""
    import ctypes
    for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            rt = ctypes.CDLL(name)
        except OSError:
            continue
        buf = ctypes.create_string_buffer(64)
        if rt.cudaDeviceGetPCIBusId(buf, 64, int(device)) == 0:
            return buf.value.decode()
    return None


class Clocks:
    """nvidia-smi clock / throttle sampling during the timed region, on the
    GPU with the CUDA device's PCI bus ID."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.bus_id = pci_bus_id(device)
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            sel = self.bus_id if self.bus_id else str(self.device)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", sel, f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "pci_bus_id": self.bus_id}
        if self.proc is None:
            return out
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return out
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for k, nme in enumerate(names):
                if r[5 + k].lower() == "active":
                    reasons.add(nme)
        out["sm_mhz"] = statistics.median(sm) if sm else None
        out["sm_max_mhz"] = max(mx) if mx else None
        out["reasons"] = sorted(reasons)
        out["samples"] = len(rows)
        return out


# ----------------------------------------------------------------------------
def algorithmic_work(st, precision):
    """FP64/FP32 flops of one call from the device event counters, per unit of
    work: RK try 650 + 6 RHS; RHS = 60 (equation of motion) + 1,248 (tricubic
    B and grad B, 3 x (64 + 3 x 48) FMA); B-only table value 384; dense-output
    state 150; BVH node test 24; segment-triangle test 60."""
    tries = st["rk_accepted"] + st["rk_rejected"]
    rhs = st["rhs_evals"]
    bonly = max(0, st["field_evals"] - rhs)
    field_flops = rhs * 1248 + bonly * 384
    other64 = tries * 650 + rhs * 60 + st["dense_evals"] * 150 + st["bvh_nodes"] * 24 + st["tri_tests"] * 60
    if precision == "fp32":
        return other64, field_flops
    return other64 + field_flops, 0


def make_workload(args, n, engine=None, first_id=0, simtime=None, scene=None):
    from pentrack_gb300 import workloads
    kw = {} if simtime is None else {"simtime": simtime}
    if args.workload == "large_mesh":
        return workloads.large_mesh(n=n, engine=engine, first_id=first_id, scene=scene, **kw)
    if args.workload == "adjoint_spin":
        return workloads.adjoint_spin(n=n, first_id=first_id, **kw)
    return workloads.field_storage(n=n, engine=engine, first_id=first_id, **kw)


def make_scene(args):
    from pentrack_gb300 import workloads
    return workloads.large_mesh_scene() if args.workload == "large_mesh" else workloads.field_storage_scene()


def setup_ours(args, rank):
    from pentrack_gb300 import Engine, _abi as A, replicas
    device = int(os.environ.get("LOCAL_RANK", 0))
    scene = make_scene(args)
    engine = Engine(scene, device=device)
    first, count = replicas.shard(args.n, rank)
    _, params, parts = make_workload(args, count, engine=engine, first_id=first, scene=scene)
    params.field_precision = A.PREC_FP32 if args.precision == "fp32" else A.PREC_FP64
    params.mode = {"batched": A.MODE_BATCHED, "phased": A.MODE_PHASED, "plain": A.MODE_PLAIN}[args.mode]
    params.scheduler = args.scheduler
    return engine, params, parts, device


def plain_run(args, rank):
    """The plain GPU form on the same workload and precision: one fixed
    step-batch launch (one lane per particle) per bench step."""
    from pentrack_gb300 import _abi as A
    import torch
    engine, params, parts, device = setup_ours(args, rank)
    params.mode = A.MODE_PLAIN
    batch = engine.batch(params, parts)
    for _ in range(args.warmup):
        batch.advance(max_steps=args.batch_steps)
    torch.cuda.synchronize(device)
    psec = ms = 0.0
    for _ in range(args.steps):
        st = batch.advance(max_steps=args.batch_steps)
        psec += st["particle_seconds"]
        ms += st["span_ms"]
    return {"value": psec / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / args.steps,
            "events": {"rk_accepted": st["rk_accepted"], "hits": st["hits"]}}


def form_run(args, rank, mode):
    """Another scheduling form on the same workload and precision (the
    host-driven phase split), timed like the headline."""
    from pentrack_gb300 import _abi as A
    import torch
    engine, params, parts, device = setup_ours(args, rank)
    params.mode = {"phased": A.MODE_PHASED, "plain": A.MODE_PLAIN, "batched": A.MODE_BATCHED}[mode]
    batch = engine.batch(params, parts)
    for _ in range(args.warmup):
        batch.advance(max_steps=args.batch_steps)
    torch.cuda.synchronize(device)
    psec = ms = 0.0
    steps = max(3, args.steps // 2)
    launches = 0
    for _ in range(steps):
        st = batch.advance(max_steps=args.batch_steps)
        psec += st["particle_seconds"]
        ms += st["span_ms"]
        launches += st["launches"] + st["aux_launches"]
    return {"value": psec / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / steps, "steps": steps,
            "gpu_launches_per_step_batch": launches / steps}


def adjoint_run(args, rank, n=1024, simtime=0.5, K=1024):
    """The adjoint-spin configuration (B0 = 1 uT + eight l <= 2 harmonic terms,
    E = 1e6 V/m, specular walls, spins along x) on a subset: the forward
    pass (pt_integrate, FP64 field, Bloch integration) and the adjoint
    (pt_adjoint, gradient of the mean phase with respect to the eight
    coefficients, checkpoints every K Bloch steps), each timed on the device;
    the cost ratio adjoint / forward is the configuration's figure."""
    from pentrack_gb300 import Engine, _abi as A, workloads, spin_gradients as SG
    device = int(os.environ.get("LOCAL_RANK", 0))
    terms = workloads.harmonic_terms_l2()
    sc, params, parts = workloads.adjoint_spin(n=n, simtime=simtime, terms=terms, first_id=rank * n)
    e = Engine(sc, device=device)
    params.mode = A.MODE_PLAIN
    params.field_precision = A.PREC_FP64
    e.integrate(params, parts)  # warm-up
    out, st = e.integrate(params, parts)
    fwd_ms = st["kernel_ms"]
    g, _, ast = e.adjoint(params, parts, 1, SG.observable_cotangents(out, "phase"), checkpoint_interval=K)
    adj_ms = ast["adj_forward_ms"] + ast["adj_reverse_ms"]
    return {"workload": f"adjoint spin: {n} UCN x {simtime} s, cylinder R=0.2 m H=0.12 m (2048 triangles), "
                        f"B0 1 uT + 8 harmonic terms l<=2, E 1e6 V/m, spins along x",
            "checkpoint_interval": K, "forward_ms": fwd_ms, "adjoint_ms": adj_ms,
            "adjoint_forward_pass_ms": ast["adj_forward_ms"], "adjoint_reverse_ms": ast["adj_reverse_ms"],
            "cost_ratio": adj_ms / fwd_ms, "spin_steps": st["spin_steps"],
            "spin_steps_per_s": st["spin_steps"] / (fwd_ms / 1e3), "dphase_dG": [float(x) for x in g]}


def field_fp64_run(args, rank):
    """The batched form in the FP64 field mode (the tricubic evaluated in FP64
    as the reference does) on the same workload: the FP32 field mode's gain
    made visible in the same line."""
    from pentrack_gb300 import _abi as A
    import torch
    engine, params, parts, device = setup_ours(args, rank)
    params.field_precision = A.PREC_FP64
    batch = engine.batch(params, parts)
    for _ in range(args.warmup):
        batch.advance(max_steps=args.batch_steps)
    torch.cuda.synchronize(device)
    psec = ms = 0.0
    steps = max(3, args.steps // 2)
    for _ in range(steps):
        st = batch.advance(max_steps=args.batch_steps)
        psec += st["particle_seconds"]
        ms += st["span_ms"]
    out = batch.read()
    return {"value": psec / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / steps, "steps": steps,
            "energy_drift": energy_drift(engine.field, parts, out)}


def cpu_baseline(args, T, n_hint=2048):
    """The oracle (FP64 CPU restatement of the reference path) on all host cores,
    on the first ids of the same workload tracked over 0-T s, T the lab-time
    span the GPU run covered."""
    from oracle import pyoracle
    from pentrack_gb300 import Engine, workloads
    cores = os.cpu_count()
    scene = make_scene(args)
    orc = pyoracle.Oracle(scene)
    eng = None
    try:
        eng = Engine(scene)
    except Exception:
        pass
    m = n_hint
    total_ps, total_s = 0.0, 0.0
    while True:
        _, params, parts = make_workload(args, m, engine=eng, simtime=T, scene=scene)
        t0 = time.perf_counter()
        out, st = orc.integrate(params, parts, nthreads=cores)
        dt = time.perf_counter() - t0
        total_ps, total_s = st["particle_seconds"], dt
        if dt >= 0.5 * args.cpu_seconds or m >= 1 << 20:
            break
        m = int(min(1 << 20, m * max(2.0, args.cpu_seconds / max(dt, 1e-3))))
    return {"value": total_ps / total_s, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"oracle on {cores} threads: first {m} UCN of the workload tracked over 0-{T:g} s "
                      f"({total_ps:.4g} particle-s in {total_s:.2f} s)",
            "energy_drift": energy_drift(orc.field, parts, out)}


def energy_drift(field, parts, out):
    """(H_end - H_start)/(t_end - t_start) per particle [eV/s] for particles
    still stored: H = Ekin + m g z - pol mu |B| (+ Fermi potential, 0 inside);
    `field` evaluates B at (x, y, z, t) rows (the engine's FP64 field, or the
    oracle's for the oracle's own run)."""
    from pentrack_gb300 import scenes
    # stored to the end of the window: still active (0) or stopped at the window's end (ID_NOT_FINISH)
    live = (out.stop_id == 0) | (out.stop_id == -1)
    if live.sum() == 0:
        return None
    idx = np.nonzero(live)[0][:20000]
    m = scenes.M_N
    c2 = scenes.C0 ** 2

    def H(t, y):
        v2 = (y[3:6] ** 2).sum(0)
        q = np.column_stack([y[0], y[1], y[2], t])
        B = field(q)[0]
        return 0.5 * m * v2 * (1 + 0.75 * v2 / c2) + m * scenes.GRAV * y[2] - y[7] * (scenes.MU_N / scenes.ELE_E) * np.sqrt((B ** 2).sum(1))

    h0 = H(parts.t[idx], parts.y[:, idx])
    h1 = H(out.t[idx], out.y[:, idx])
    rate = np.abs(h1 - h0) / np.maximum(out.t[idx] - parts.t[idx], 1e-30)
    return {"median_eV_per_s": float(np.median(rate)), "p99_eV_per_s": float(np.percentile(rate, 99)),
            "particles": int(len(idx))}


def e2e_run(args, engine, params, rank, T):
    """The reference-facing call: pt_integrate with host (pinned) buffers, a
    fresh chunk of the workload per step tracked over 0-T s (T = the lab-time
    span of one device step-batch)."""
    from pentrack_gb300 import workloads
    import torch
    n = args.n

    def pinned(a):
        tt = torch.empty(a.shape, dtype=torch.from_numpy(a).dtype, pin_memory=True)
        tt.numpy()[...] = a
        return tt.numpy()

    def pinned_set(seed_first):
        from pentrack_gb300 import ParticleSet
        _, p, parts = make_workload(args, n, engine=engine, first_id=seed_first, simtime=T)
        for k in ("id", "t", "y", "spin"):
            setattr(parts, k, pinned(getattr(parts, k)))
        out = ParticleSet.empty(n)  # caller-owned pinned output buffers
        for k in ("id", "t", "y", "spin") + tuple(f for f, _ in ParticleSet.OUT_FIELDS):
            setattr(out, k, pinned(getattr(out, k)))
        return p, parts, out

    h2d = d2h = 0
    total_ps, total_s, dev_ms = 0.0, 0.0, 0.0
    for k in range(1 + args.e2e_steps):
        p, parts, dst = pinned_set(10_000_000 * (k + 1) + rank * n)
        p.field_precision, p.mode = params.field_precision, params.mode
        t0 = time.perf_counter()
        out, st = engine.integrate(p, parts, out=dst)
        dt = time.perf_counter() - t0
        if k == 0:
            continue
        total_ps += st["particle_seconds"]
        total_s += dt
        dev_ms += st["span_ms"]
        h2d = n * (8 + 8 + 72 + 40)
        d2h = n * (8 + 8 + 72 + 40 + 4 * 4 + 8 * 6)
    return {"value": total_ps / total_s, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "steps": args.e2e_steps, "call": "pt_integrate (host buffers, full H2D/D2H per step)",
            "ms_per_step": total_s * 1e3 / args.e2e_steps, "tracking_device_ms_per_step": dev_ms / args.e2e_steps}


def load_traffic(kernel):
    """DRAM bytes per RK try of the try kernel, from the committed ncu capture
    (profiles/<kernel>_field_storage_traffic.json); None when absent."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_field_storage_traffic.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return None


def run_ours(args, rank, world):
    import torch
    engine, params, parts, device = setup_ours(args, rank)
    from pentrack_gb300 import lib
    import ctypes
    peak = ctypes.c_double(0)
    lib().pt_probe_fp64(engine.h, ctypes.byref(peak))
    batch = engine.batch(params, parts)
    for _ in range(args.warmup):
        batch.advance(max_steps=args.batch_steps)
    dist = world > 1
    if dist:
        torch.distributed.barrier()
    torch.cuda.synchronize(device)
    clocks = Clocks(device)
    clocks.start()
    agg = None
    try_kernel = "k_run" if args.mode == "batched" else "k_try"
    t0 = time.perf_counter()
    for _ in range(args.steps):
        st = batch.advance(max_steps=args.batch_steps)
        if str(st["dominant_kernel"]).startswith(("k_try", "k_run")):
            try_kernel = st["dominant_kernel"]
        if agg is None:
            agg = dict(st)
        else:
            for k, v in st.items():
                if isinstance(v, (int, float)) and k not in ("active", "scheduler"):
                    agg[k] += v
            agg["active"] = st["active"]
    torch.cuda.synchronize(device)
    elapsed = time.perf_counter() - t0
    clk = clocks.stop()
    psec = agg["particle_seconds"]
    device_ms = agg["span_ms"]
    if dist:
        from pentrack_gb300 import replicas
        device_s, psec_all = replicas.reduce_timing(device_ms / 1e3, psec, device=f"cuda:{device}")
        torch.distributed.barrier()
    else:
        device_s, psec_all = device_ms / 1e3, psec
    out_state = batch.read()
    if rank != 0:
        return None
    live = out_state.stop_id == 0
    span_total = float(np.median(out_state.t[live] - parts.t[live])) if live.any() else 1.0
    span_step = span_total / (args.warmup + args.steps)
    f64, f32 = algorithmic_work(agg, args.precision)
    tries = agg["rk_accepted"] + agg["rk_rejected"]
    field_per_rhs = 1248
    # one RK try: stage algebra, error norm and step control (650) plus six
    # equations of motion (60 each) in FP64; the tricubic B and grad B (1,248
    # per right-hand side) in FP64 or, in the FP32 field mode, in FP32
    try_f64 = tries * (650 + 6 * 60) + (0 if args.precision == "fp32" else tries * 6 * field_per_rhs)
    try_f32 = tries * 6 * field_per_rhs if args.precision == "fp32" else 0
    state_bytes = None
    if args.mode in ("batched", "phased"):
        first = "k_run" if str(agg["dominant_kernel"]).startswith("k_run") else "k_try"
        kern = {first: agg["try_ms"], "k_post": agg["post_ms"], "k_slow": agg["slow_ms"], "k_bisect": agg["bisect_ms"],
                "k_plain_tail": agg["tail_ms"]}
        dom = max(kern, key=kern.get)
        launches = max(1, agg["dominant_launches"])
        avg_launch_s = kern[dom] / 1e3 / launches
        # k_run: its tries are counted (a lower bound on its work: the fast
        # step completion and its BVH query add to it); k_try: exactly its tries
        dom_f64 = try_f64 if dom == first else f64
        dom_f32 = try_f32 if dom == first else f32
        achieved = dom_f64 / launches / avg_launch_s / 1e12
        # the FP32-table-only instances are k_run_tab32 / k_try_tab32
        agg["dominant_kernel"] = try_kernel if dom == first else dom
        if args.mode == "phased":
            # per-particle state a try must move: reads t, y, dydt, dt, ntry, nacc,
            # nrej, list entry (188 B), writes dt, ntry, nacc, nrej (28 B); an
            # accepted try also writes yn, dyn, k3..k6, tn, flags, the B cache slot
            # and a list entry (504 B), a rejected one a list entry (4 B)
            acc = agg["rk_accepted"] / max(1, tries)
            state_bytes = (188 + 28 + 504 * acc + 4 * (1 - acc)) * tries / launches
    else:
        launches = max(1, agg["dominant_launches"])
        avg_launch_s = agg["dominant_kernel_ms"] / 1e3 / launches
        achieved = f64 / launches / avg_launch_s / 1e12
        dom_f64, dom_f32 = f64, f32
    traffic = None
    if args.workload == "field_storage" and agg["dominant_kernel"].startswith(("k_try", "k_run")):
        t = load_traffic(agg["dominant_kernel"])
        if t:
            # per launch like `achieved`: bytes per try x tries per average launch
            traffic = (t["dram_read_bytes_per_try"] + t["dram_write_bytes_per_try"]) * tries / launches
    line = {
        "metric": METRIC,
        "value": psec_all / device_s,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": device_s * 1e3 / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f64 state, f32 field",
        "data": "synthetic (seeded Philox sources; analytic quadrupole table)",
        "config": {"workload": (f"field storage: {args.n} UCN/GPU, cylinder R=0.2 m H=0.1 m (1024 triangles), "
                                f"64^3 tricubic quadrupole, 250 neV walls 5% Lambert 1e-4 loss, tau 880 s")
                               if args.workload == "field_storage" else
                               (f"large mesh: {args.n} UCN/GPU, noisy torus R=1 m r=0.1 m + sphere R=0.5 m (200,000 "
                                f"triangles), 128^3 tricubic multipole, 10% Lambert 3e-5 loss, tau 880 s"),
                   "step": f"one step-batch: every live particle advances {args.batch_steps} accepted RK steps",
                   "form": args.mode, "field_precision": args.precision,
                   "l2": "per-step particle state > L2 (350 B x 1e6); field table L2-resident by design",
                   "parallelism": f"replicas x{world}", "lab_time_per_step_s": span_step},
        "gpu_launches": int(agg["launches"] + agg["aux_launches"]),
        "gpu_launches_detail": {"timed_kernels": int(agg["launches"]), "bookkeeping_kernels": int(agg["aux_launches"]),
                                "graph_launches": int(agg["graph_launches"]),
                                "scheduler_iterations": int(agg["sched_outer_iters"]),
                                "slow_rounds": int(agg["sched_inner_iters"]),
                                "per_step_batch": (agg["launches"] + agg["aux_launches"]) / args.steps},
        "wall_s": elapsed,
        "clocks": clk,
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
                     "frac": achieved / peak.value if peak.value else None,
                     "peak_source": "measured: pt_probe_fp64 DFMA kernel on this GPU",
                     "traffic": traffic, "state_bytes_per_launch": state_bytes,
                     "kernel": agg["dominant_kernel"], "launches": int(launches),
                     "avg_launch_ms": avg_launch_s * 1e3,
                     "fp64_flops_per_launch": dom_f64 / launches, "fp32_flops_per_launch": dom_f32 / launches},
        "events": {k: agg[k] for k in ("rk_accepted", "rk_rejected", "rhs_evals", "field_evals", "hits",
                                        "bisection_levels", "bvh_nodes", "tri_tests", "subsegments", "dense_evals",
                                        "bisect_max", "bisect_dead", "cand_calls", "cand_overflow", "cand_sum", "tri32_tests")},
        "live_particles": int(agg["active"]),
        "scheduler": {"chosen": SCHED_NAMES[int(st["scheduler"])],
                      "autotune_ns_per_try": {SCHED_NAMES[k + 1]: st["tune_ns_per_try"][k] for k in range(4)}},
        "phase_ms": {("k_run" if str(agg["dominant_kernel"]).startswith("k_run") else "k_try"): agg["try_ms"], "k_post": agg["post_ms"],
                     "k_slow": agg["slow_ms"], "k_bisect": agg["bisect_ms"], "k_plain_tail": agg["tail_ms"]},
    }
    if not args.no_plain and args.mode == "batched":
        line["plain_form"] = plain_run(args, rank)
    if not args.no_phased and args.mode == "batched":
        line["phased_form"] = form_run(args, rank, "phased")
    line["energy_drift"] = energy_drift(engine.field, parts, out_state)
    if not args.no_fp64_line and args.precision == "fp32" and args.mode == "batched":
        line["field_fp64"] = field_fp64_run(args, rank)
    if not args.no_adjoint:
        line["adjoint_spin"] = adjoint_run(args, rank)
    if not args.no_e2e:
        try:
            line["e2e"] = e2e_run(args, engine, params, rank, span_step)
        except Exception as ex:  # report, never hide
            line["e2e"] = {"error": str(ex)}
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args, span_total)
        # the energy drift of the FP64 CPU oracle over the same lab-time span, beside the GPU's
        line["energy_drift"] = {"gpu": line["energy_drift"], "oracle": line["cpu_baseline"]["energy_drift"],
                                "unit": "eV/s per particle, |H_end - H_start| / (t_end - t_start), stored UCN"}
    return line


# Bloch (LOOP D) work per accepted Bloch step, FP64 flops: six precession-axis
# evaluations (dense-output coefficients 36 + trajectory state 108 + the two
# harmonic polynomials of B and grad B 140 + equation of motion 60 + BMT and
# Thomas axis 70 + spin derivative 20) and the stage algebra and error norm
# (about 290)
BLOCH_FLOPS = 6 * 434 + 290


def run_spin(args, rank, world):
    """--workload adjoint_spin: the adjoint-spin configuration at its stated
    size (10,000 UCN per GPU in the cylinder R = 0.2 m, H = 0.12 m of 512
    segments; B0 = 1 uT + eight l <= 2 harmonic terms; E = 1e6 V/m; specular
    walls; spins along x; Bloch integration along every trajectory step, FP64
    field) in bounded steps: each bench step advances every particle by
    --spin-window s of its 100 s (pt_batch_advance_steps with a lab-time
    pause), timed with CUDA events on the engine's stream.  Reports
    particle-s/s, Bloch steps/s and the FP64 roofline of k_plain_spin."""
    import torch
    import ctypes
    from pentrack_gb300 import Engine, _abi as A, workloads, lib
    device = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(device)
    sc, params, parts = workloads.adjoint_spin(n=args.n, simtime=100.0, first_id=rank * args.n)
    e = Engine(sc, device=device)
    params.mode = A.MODE_PLAIN
    params.field_precision = A.PREC_FP64
    peak = ctypes.c_double(0)
    lib().pt_probe_fp64(e.h, ctypes.byref(peak))
    batch = e.batch(params, parts)
    w = args.spin_window
    for k in range(args.warmup):
        batch.advance(t_pause=(k + 1) * w)
    dist = world > 1
    if dist:
        torch.distributed.barrier()
    torch.cuda.synchronize(device)
    clocks = Clocks(device)
    clocks.start()
    psec = ms = 0.0
    spin = launches = 0
    t0 = time.perf_counter()
    for k in range(args.steps):
        st = batch.advance(t_pause=(args.warmup + k + 1) * w)
        psec += st["particle_seconds"]
        ms += st["kernel_ms"]
        spin += st["spin_steps"]
        launches += st["launches"]
    torch.cuda.synchronize(device)
    elapsed = time.perf_counter() - t0
    clk = clocks.stop()
    device_s = ms / 1e3
    if dist:
        from pentrack_gb300 import replicas
        device_s, psec_all = replicas.reduce_timing(device_s, psec, device=f"cuda:{device}")
        torch.distributed.barrier()
    else:
        psec_all = psec
    if rank != 0:
        return None
    achieved = spin * BLOCH_FLOPS / (ms / 1e3) / 1e12
    line = {
        "metric": "particle-s tracked/s with Bloch spin integration, 1 GB300", "value": psec_all / device_s,
        "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": device_s * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded Philox sources; harmonic coefficients drawn N(0, 1e-10 T/m^l))",
        "config": {"workload": f"adjoint spin: {args.n} UCN/GPU x 100 s, cylinder R=0.2 m H=0.12 m (2048 triangles), "
                               "B0 1 uT + 8 harmonic terms l<=2, E 1e6 V/m, specular walls, spins along x",
                   "step": f"every particle advances {w:g} s of lab time with Bloch integration",
                   "form": "plain (k_plain_spin)", "field_precision": "fp64",
                   "l2": "state 1.6 KB x 1e4 particles is L2-resident; the kernel is FP64-pipe bound",
                   "parallelism": f"replicas x{world}"},
        "bloch_steps_per_s": spin / (ms / 1e3), "bloch_steps": int(spin),
        "gpu_launches": int(launches), "wall_s": elapsed, "clocks": clk,
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
                     "frac": achieved / peak.value if peak.value else None,
                     "peak_source": "measured: pt_probe_fp64 DFMA kernel on this GPU",
                     "kernel": "k_plain_spin", "fp64_flops_per_bloch_step": BLOCH_FLOPS, "traffic": None},
    }
    if not args.no_e2e:
        try:
            line["e2e"] = e2e_run(args, e, params, rank, w)
        except Exception as ex:  # report, never hide
            line["e2e"] = {"error": str(ex)}
    if not args.no_cpu_baseline:
        ref = run_reference_spin(argparse.Namespace(warmup=0, steps=2), 1, os.cpu_count())
        line["cpu_baseline"] = dict(ref["cpu_baseline"], bloch_steps_per_s=ref["bloch_steps_per_s"])
    return line


def run_full(args, rank, world):
    """--full-run: the field-storage workload over its whole 200 s, every UCN
    tracked to its end (decay, absorption, loss through the boundary or the
    end of the run) in one pt_integrate call per form, the regime where
    trajectory lengths are most uneven (absorbed UCN within ms, stored ones
    the full 200 s).  Device time of each call (CUDA events / %globaltimer
    spans on the engine's stream) and wall time; particle-s/s of each form."""
    import torch
    from pentrack_gb300 import Engine, _abi as A, workloads
    device = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(device)
    sc = workloads.field_storage_scene()
    e = Engine(sc, device=device)
    res = {}
    for form, mode in (("batched", A.MODE_BATCHED), ("plain", A.MODE_PLAIN)):
        _, params, parts = workloads.field_storage(n=args.n, simtime=200.0, first_id=rank * args.n, engine=e)
        params.field_precision = A.PREC_FP32 if args.precision == "fp32" else A.PREC_FP64
        params.mode = mode
        torch.cuda.synchronize(device)
        t0 = time.perf_counter()
        out, st = e.integrate(params, parts)
        torch.cuda.synchronize(device)
        wall = time.perf_counter() - t0
        dev_s = st["span_ms"] / 1e3
        ids, counts = np.unique(out.stop_id, return_counts=True)
        res[form] = {"value": st["particle_seconds"] / dev_s, "unit": UNIT, "device_s": dev_s, "wall_s": wall,
                     "particle_seconds": st["particle_seconds"], "rk_steps": int(st["rk_accepted"]),
                     "stop_ids": {int(k): int(c) for k, c in zip(ids, counts)},
                     "gpu_launches": int(st["launches"] + st["aux_launches"])}
        if form == "batched":
            res[form]["scheduler"] = SCHED_NAMES[int(st["scheduler"])]
    if rank != 0:
        return None
    return {"metric": METRIC, "value": res["batched"]["value"], "unit": UNIT, "n_gpus": world, "steps": 1, "warmup": 0,
            "ms_per_step": res["batched"]["device_s"] * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f64 state, f32 field",
            "data": "synthetic (seeded Philox sources; analytic quadrupole table)",
            "config": {"workload": f"field storage, full run: {args.n} UCN/GPU over 0-200 s, every UCN to its end",
                       "step": "one pt_integrate call per form", "field_precision": args.precision,
                       "parallelism": f"replicas x{world}"},
            "batched": res["batched"], "plain": res["plain"],
            "batched_over_plain": res["batched"]["value"] / res["plain"]["value"]}


def run_reference(args, rank, world):
    """The reference path's CPU implementation (the oracle port: the reference
    itself cannot be built without Boost/CGAL) on all host cores."""
    if rank != 0:
        return None
    from oracle import pyoracle
    from pentrack_gb300 import workloads
    cores = os.cpu_count()
    if args.workload == "adjoint_spin":
        return run_reference_spin(args, world, cores)
    scene = workloads.field_storage_scene()
    orc = pyoracle.Oracle(scene)
    m = 4096
    T = 0.06 * (args.warmup + args.steps)  # about the lab time 32 accepted RK steps cover in this workload
    total_ps = total_s = 0.0
    for k in range(args.warmup + args.steps):
        _, params, parts = workloads.field_storage(n=m, simtime=T, first_id=k * m)
        t0 = time.perf_counter()
        out, st = orc.integrate(params, parts, nthreads=cores)
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            total_ps += st["particle_seconds"]
            total_s += dt
    value = total_ps / total_s
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_s * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded Philox sources; analytic quadrupole table)", "impl": "reference",
            "config": {"workload": "field storage (same scene); per step 4096 UCN tracked over "
                                   f"0-{T:g} s", "parallelism": f"{cores} host threads"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{args.steps} x 4096 UCN over 0-{T:g} s on {cores} threads"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_reference_spin(args, world, cores):
    """The oracle on the adjoint-spin configuration: per step a fresh 512 UCN
    of the workload tracked with Bloch integration over 0-1 s on all host
    threads."""
    from oracle import pyoracle
    from pentrack_gb300 import workloads
    m, T = 512, 1.0
    total_ps = total_s = 0.0
    spin = 0
    orc = None
    for k in range(args.warmup + args.steps):
        sc, params, parts = workloads.adjoint_spin(n=m, simtime=T, first_id=k * m)
        orc = orc or pyoracle.Oracle(sc)
        t0 = time.perf_counter()
        out, st = orc.integrate(params, parts, nthreads=cores)
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            total_ps += st["particle_seconds"]
            total_s += dt
            spin += st["spin_steps"]
    value = total_ps / total_s
    sample = f"{args.steps} x {m} UCN over 0-{T:g} s with Bloch integration on {cores} threads"
    return {"metric": "particle-s tracked/s with Bloch spin integration, 1 GB300", "value": value, "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_s * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Philox sources; harmonic coefficients drawn N(0, 1e-10 T/m^l))", "impl": "reference",
            "config": {"workload": "adjoint spin (same scene); " + sample, "parallelism": f"{cores} host threads"},
            "bloch_steps_per_s": spin / total_s,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    args = parse()
    if args.n is None:
        args.n = {"large_mesh": 10_000_000, "adjoint_spin": 10_000}.get(args.workload, 1_000_000)
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if world > 1:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        torch.distributed.init_process_group("nccl")
    from pentrack_gb300 import build
    if args.impl == "ours":
        build.build_engine()
    build.build_oracle()
    if args.impl == "reference":
        line = run_reference(args, rank, world)
    elif args.workload == "adjoint_spin":
        line = run_spin(args, rank, world)
    elif args.full_run:
        line = run_full(args, rank, world)
    else:
        line = run_ours(args, rank, world)
    if rank == 0 and line is not None:
        print(json.dumps(line))
    if world > 1:
        import torch
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
