"""The C-ABI library loads and exports every entry point include/pentrack_gpu.h declares."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h") or h == "pt_constants.h":
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(pt_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("pt_create", "pt_destroy", "pt_integrate", "pt_batch_advance", "pt_last_error", "pt_cancel"):
        assert s in syms


def test_library_exports_every_declared_symbol(built):
    from pentrack_gb300 import engine
    L = engine.lib()
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, missing
    assert b"sm_103a" in L.pt_version()


def test_struct_sizes_match_header(built):
    """The ctypes mirror has the same layout as the C structs (checked through
    offsets that the C side reports implicitly via a round trip)."""
    from pentrack_gb300 import _abi as A
    assert ctypes.sizeof(A.Material) == 9 * 8
    assert ctypes.sizeof(A.Solid) == 24
    assert ctypes.sizeof(A.Particles) == 17 * 8
    assert A.Field.ez.offset + 8 == ctypes.sizeof(A.Field)


def test_create_without_device_fails_cleanly(built):
    """On a host without a GPU pt_create reports PT_ERR_NO_DEVICE instead of
    falling back to a CPU path."""
    from pentrack_gb300 import Engine, EngineError, workloads
    if os.environ.get("CUDA_VISIBLE_DEVICES", None) == "" or not os.path.exists("/dev/nvidiactl"):
        sc, _, _ = workloads.cube_storage(n=1)
        with pytest.raises(EngineError) as e:
            Engine(sc)
        assert e.value.status in (-8, -4)
    else:
        pytest.skip("a GPU is present")


def test_ctypes_layout_equals_the_c_compilers(tmp_path):
    """Every field offset and struct size of the ctypes mirror equals what a C
    compiler computes from include/pentrack_gpu.h."""
    import shutil
    import subprocess
    from pentrack_gb300 import _abi as A
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = {"pt_material": A.Material, "pt_solid": A.Solid, "pt_field": A.Field, "pt_scene_desc": A.SceneDesc,
               "pt_run_params": A.RunParams, "pt_particles": A.Particles, "pt_stats": A.Stats,
               "pt_source_params": A.SourceParams}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "pentrack_gpu.h"', "int main(void) {"]
    expect = []
    for cname, cls in structs.items():
        lines.append(f'printf("%zu\\n", sizeof({cname}));')
        expect.append(ctypes.sizeof(cls))
        for f in cls._fields_:
            lines.append(f'printf("%zu\\n", offsetof({cname}, {f[0]}));')
            expect.append(getattr(cls, f[0]).offset)
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert got == expect
