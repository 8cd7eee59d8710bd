"""Build recipe for the engine's shared library (sm_103a) and, for tests, the oracle.

The engine is compiled in-tree with nvcc: pentrack_gb300/libpentrack_gpu.so.
The host translation unit and the CUDA translation unit compile in parallel.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libpentrack_gpu.so")
BUILD_DIR = os.path.join(HERE, "_build")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", f"-I{os.path.join(ROOT, 'include')}"]

SOURCES = ["pt_api.cu", "pt_k_phase.cu", "pt_k_run.cu", "pt_k_adjoint.cu", "pt_k_slow.cu", "pt_k_plain.cu", "pt_k_query.cu", "pt_k_source.cu", "pt_scene.cpp", "pt_host.cpp"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build_engine(force=False, verbose=False):
    os.makedirs(BUILD_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".h"))]
    headers += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    srcs = [os.path.join(CSRC, s) for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    objs = [os.path.join(BUILD_DIR, os.path.basename(s) + ".o") for s in srcs]
    if not force and not _stale(LIB, srcs + headers + [__file__]):
        return LIB
    jobs = []
    for s, o in zip(srcs, objs):
        if force or _stale(o, [s] + headers):
            # device code: no automatic contraction; the integrator's fused
            # multiply-adds are explicit (identical chains in the oracle)
            extra = ["-fmad=false"] if s.endswith(".cu") else []
            jobs.append([NVCC] + ARCH + COMMON + extra + ["-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for r in ex.map(_run, jobs):
            if verbose and r.stderr:
                sys.stderr.write(r.stderr)
    _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    return LIB


def reference_tree():
    """The reference source tree the oracle recipe compiles ALGLIB/libtricubic
    from: $PENTRACK_REFERENCE, else the read-only mount of the build container;
    None when absent (as on a machine that only runs the prebuilt checker)."""
    path = os.environ.get("PENTRACK_REFERENCE", "/root/reference")
    return path if os.path.isdir(path) else None


def build_oracle(force=False):
    """Compile the CPU oracle (test infrastructure) and, when the reference
    tree is present, the reference's ALGLIB/libtricubic under oracle/_ref."""
    odir = os.path.join(ROOT, "oracle")
    args = ["make", "-C", odir, "-j4", "all"]
    if force:
        args.insert(3, "-B")
    _run(args)
    ref = reference_tree()
    if ref:
        _run(["make", "-C", odir, "-j8", "ref", f"REF={ref}"])


if __name__ == "__main__":
    build_engine(force="--force" in sys.argv, verbose=True)
    build_oracle()
    print("built", LIB)
