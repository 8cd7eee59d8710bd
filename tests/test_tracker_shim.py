"""The header-only TTrackerGPU (include/pentrack_tracker_gpu.hpp), whose
IntegrateParticle has the signature of TTracker::IntegrateParticle
(include/tracking.h:46-47), compiled against stand-ins of the PENTrack types
(tests/cpp/stub_pentrack.h) and linked to the engine library.

CPU: the shim compiles, reads the particle options the reference's
IntegrateParticle reads (src/tracking.cpp:19-60) and, without a GPU, reports
pt_create's error.  GPU: particles tracked one at a time through the shim end
bit-identical to Engine.integrate on the same config (plain form)."""
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

CONFIG = """[GLOBAL]
simtime 5

[MATERIALS]
default 335 0 0 0 0 0
vacuum  0 0 0 0 0 0

[GEOMETRY]
1 ignored default
2 cube.STL vacuum

[FIELDS]
"""


@pytest.fixture(scope="module")
def shim_exe(built, tmp_path_factory):
    d = tmp_path_factory.mktemp("shim")
    exe = d / "shim"
    lib = os.path.join(ROOT, "pentrack_gb300")
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(HERE, "cpp"),
           os.path.join(HERE, "cpp", "shim_main.cpp"), "-o", str(exe), f"-L{lib}", "-lpentrack_gpu", f"-Wl,-rpath,{lib}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _case(d, n=8, simtime=5.0):
    from pentrack_gb300 import scenes, workloads
    (d / "config.in").write_text(CONFIG.replace("simtime 5", f"simtime {simtime}"))
    scenes.write_stl(d / "cube.STL", scenes.box_mesh((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5)))
    _, params, parts = workloads.cube_storage(n=n, simtime=simtime)
    lines = [f"{simtime}"]
    for i in range(n):
        lines.append(" ".join([str(int(parts.id[i])), repr(float(parts.t[i]))] + [repr(float(v)) for v in parts.y[:, i]]))
    (d / "particles.txt").write_text("\n".join(lines) + "\n")
    return params, parts


def _run(exe, d):
    r = subprocess.run([str(exe), str(d / "config.in"), str(d / "particles.txt")], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout.splitlines()


def test_shim_reads_particle_options_and_reports_errors(shim_exe, tmp_path):
    import torch
    _case(tmp_path)
    out = _run(shim_exe, tmp_path)
    p = out[0].split()
    assert p[0] == "params"
    assert [float(x) for x in p[1:6]] == [100.0, 880.0, 9e99, 5e3, 0.1]
    assert int(p[6]) == 1 and int(p[7]) == 4 and [float(x) for x in p[8:12]] == [0.0, 10.0, 20.0, 30.0]
    if not torch.cuda.is_available():
        assert out[1].startswith("error") and "device" in out[1]


@pytest.mark.gpu
def test_shim_integrate_particle_matches_engine(shim_exe, tmp_path):
    from pentrack_gb300 import ConfigScene, Engine, _abi as A
    params, parts = _case(tmp_path)
    lines = [l.split() for l in _run(shim_exe, tmp_path) if l.startswith("end")]
    assert len(lines) == parts.n
    sc = ConfigScene(tmp_path / "config.in")
    e = Engine(sc)
    params.mode = A.MODE_PLAIN
    params.seed = 1001
    out, _ = e.integrate(params, parts)
    for i, l in enumerate(lines):
        assert int(l[1]) == out.id[i]
        assert int(l[2]) == out.stop_id[i]
        assert float(l[4]) == out.t[i]
        assert np.array_equal(np.array([float(x) for x in l[5:14]]), out.y[:, i])
        assert int(l[3]) == (2 if np.all(np.abs(out.y[0:3, i]) < 0.5) else 1)
