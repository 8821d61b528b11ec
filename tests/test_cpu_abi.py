"""The C ABI: the library loads on a machine without a GPU, exports every
symbol include/*.h declares (the reference's 16 among them), and its records
have the reference's byte layout. CPU only: no compute call."""
import ctypes as C
import os
import re
import subprocess

import pytest

import simstack_gb300 as sg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# the reference sources: SIMSTACK_REF_DIR, else the staged copy (oracle/Makefile `stage`)
REF_SRC = os.environ.get("SIMSTACK_REF_DIR", os.path.join(ROOT, "baseline", "_ref"))


def declared_exports():
    names = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            text = "\n".join(l for l in open(os.path.join(ROOT, "include", fn)) if not l.lstrip().startswith("#"))
            names += re.findall(r"SGB_API\s+[\w\s\*]+?\b(\w+)\s*\(", text)
    return sorted(set(names))


def test_library_loads_and_exports_every_declared_symbol():
    L = C.CDLL(sg.LIB_PATH)
    names = declared_exports()
    assert len(names) > 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_reference_export_names_present():
    L = C.CDLL(sg.LIB_PATH)
    for name in sg.REFERENCE_EXPORTS:
        assert hasattr(L, name), name
    assert set(sg.REFERENCE_EXPORTS) <= set(declared_exports())


def test_record_layouts():
    """Sizes and offsets of the boundary records (src/gpu/gpu_api.h:30-44, kin_mech.h:42-120)."""
    assert C.sizeof(sg.KinMech) == 30044 and C.sizeof(sg.KinReaction) == 54
    assert C.sizeof(sg.KinMethod) == 200 and C.sizeof(sg.KinControl) == 56
    assert C.sizeof(sg.GpuKinLaunch) == 120 and C.sizeof(sg.GpuInfo) == 168
    assert sg.GpuKinLaunch.padded.offset == 96 and sg.GpuKinLaunch.precision.offset == 104
    assert sg.GpuKinLaunch.duration.offset == 112 and sg.GpuInfo.total_bytes.offset == 144


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF_SRC, "src", "gpu")), reason="reference sources not present")
def test_layouts_against_reference_headers(tmp_path):
    """Compile a probe against the reference's own headers and against include/simstack_gpu.h."""
    fields = ("sizeof(KinMech)", "sizeof(KinMethod)", "sizeof(KinControl)", "sizeof(GpuKinLaunch)", "sizeof(GpuInfo)",
              "offsetof(GpuKinLaunch, padded)", "offsetof(GpuKinLaunch, lane_count)", "offsetof(GpuKinLaunch, precision)",
              "offsetof(GpuKinLaunch, duration)", "offsetof(GpuInfo, multiprocessors)", "offsetof(GpuInfo, arena_bytes)",
              "offsetof(KinMech, nnz)", "offsetof(KinMech, lu_div)", "offsetof(KinMech, lu_sub)", "offsetof(KinMech, upper)",
              "offsetof(KinMethod, gamma0)", "offsetof(KinControl, max_steps)")
    body = "int main(){" + "".join(f'printf("%zu\\n", (size_t)({f}));' for f in fields) + "return 0;}"
    ref = tmp_path / "ref.cpp"
    ref.write_text("#define BASE_DEBUG_H\n#define TIMED_BLOCK(n)\n#define TIMED_FUNCTION()\nstruct DebugTable;\n"
                   "#include <stdio.h>\n#include <stddef.h>\n#include \"sim_platform.h\"\n#include \"sim/kinetics/kin_mech.h\"\n" + body)
    ours = tmp_path / "ours.cpp"
    ours.write_text("#include <stdio.h>\n#include <stddef.h>\n#include \"simstack_gpu.h\"\n" + body)
    outs = []
    for src, inc, extra in ((ref, os.path.join(REF_SRC, "src"), ["-DSIM_SIMD=0"]), (ours, os.path.join(ROOT, "include"), [])):
        exe = str(src) + ".bin"
        subprocess.run(["g++", "-std=c++20", "-w", *extra, f"-I{inc}", str(src), "-o", exe], check=True)
        outs.append(subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split())
    assert outs[0] == outs[1]


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF_SRC, "src", "platform")), reason="reference sources not present")
def test_reference_loader_resolves_every_export(tmp_path):
    """The reference's own loader (linux_gpu.cpp) dlopens this library and resolves all
    16 exports; without a GPU it then stops at gpu_init, as it would for its own module."""
    src = tmp_path / "load.cpp"
    src.write_text(
        "#define BASE_DEBUG_H\n#define TIMED_BLOCK(n)\n#define TIMED_FUNCTION()\nstruct DebugTable;\n"
        "#include <stdio.h>\n#include <dlfcn.h>\n#include \"sim_platform.h\"\n#include \"platform/linux_gpu.cpp\"\n"
        "int main(int c, char **v){ GpuAPI api; b32 ok = linux_load_gpu_module(v[1], 1 << 20, &api); printf(\"loaded=%d\\n\", ok); return 0; }\n")
    exe = str(tmp_path / "load")
    subprocess.run(["g++", "-std=c++20", "-w", "-DSIM_SIMD=0", f"-I{os.path.join(REF_SRC, 'src')}", str(src), "-o", exe, "-ldl"],
                   check=True)
    out = subprocess.run([exe, sg.LIB_PATH], capture_output=True, text=True)
    text = out.stdout + out.stderr
    assert "missing export" not in text
    assert "loaded=1" in text or "gpu_init failed" in text
