"""Build recipe of the GB300 kinetics module (no cmake, no setuptools).

    python -m simstack_gb300.build

1. compiles and runs the build-time generator (csrc/kin_codegen.cpp + mech.cpp),
   which writes straight-line device code for the shipped mechanism into
   _build/gen/air_ops.cuh;
2. compiles every translation unit in parallel -- one nvcc per precision of the
   generated kernels, the table-driven kernels, the probes and the exports,
   g++ for the host code -- for sm_103a only;
3. links simstack_gb300/libsimstack_gpu.so (in-tree, git-ignored).

Flags that carry the bit-identity contract: -fmad=false (device: no FMA the
source does not ask for; explicit fma() still fuses) and -ffp-contract=off
(host: the rate constants and the generator).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(ROOT, "_build")
GEN = os.path.join(BUILD, "gen")
LIB = os.path.join(PKG, "libsimstack_gpu.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC = os.environ.get("NVCC", "nvcc")
CXX = os.environ.get("CXX", "g++")

NV_FLAGS = ["-std=c++17", "-O3", ARCH, "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
            "-Xptxas", "-v", f"-I{GEN}", f"-I{CSRC}"]
# Extra preprocessor definitions for build-time variants (e.g. SGB_NOINLINE_OPS).
NV_FLAGS += [f"-D{d}" for d in os.environ.get("SGB_DEFINES", "").split() if d]
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wno-unused-function"]


def _run(cmd: list[str], log: str) -> None:
    out = subprocess.run(cmd, capture_output=True, text=True)
    with open(log, "w") as f:
        f.write(" ".join(cmd) + "\n" + out.stdout + out.stderr)
    if out.returncode != 0:
        raise RuntimeError(f"build step failed ({' '.join(cmd[:3])} ...):\n{out.stdout}{out.stderr}")


def _sources_newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, jobs: int | None = None) -> str:
    os.makedirs(GEN, exist_ok=True)
    # objects built with other flags (SGB_DEFINES variants) are rebuilt
    stamp = os.path.join(BUILD, "flags.txt")
    flags = " ".join(NV_FLAGS + CXX_FLAGS)
    if not os.path.exists(stamp) or open(stamp).read() != flags:
        force = True
        with open(stamp, "w") as f:
            f.write(flags)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "simstack_gpu.h"))
    # 1. generator
    gen_bin = os.path.join(BUILD, "kin_codegen")
    gen_srcs = [os.path.join(CSRC, "kin_codegen.cpp"), os.path.join(CSRC, "mech.cpp")]
    if force or _sources_newer(gen_bin, gen_srcs + headers):
        _run([CXX, "-std=c++17", "-O1", "-ffp-contract=off", *gen_srcs, "-o", gen_bin], os.path.join(BUILD, "codegen.log"))
    air_ops = os.path.join(GEN, "air_ops.cuh")
    _run([gen_bin, air_ops], os.path.join(BUILD, "codegen_run.log"))
    # 2. objects
    units = [
        ("kern_air_p0.o", [NVCC, *NV_FLAGS, "-DSGB_PREC=0", "-c", os.path.join(CSRC, "kern_air.cu")]),
        ("kern_air_p1.o", [NVCC, *NV_FLAGS, "-DSGB_PREC=1", "-c", os.path.join(CSRC, "kern_air.cu")]),
        ("kern_air_p2.o", [NVCC, *NV_FLAGS, "-DSGB_PREC=2", "-c", os.path.join(CSRC, "kern_air.cu")]),
        ("kern_air_p3.o", [NVCC, *NV_FLAGS, "-DSGB_PREC=3", "-c", os.path.join(CSRC, "kern_air.cu")]),
        ("kern_air_p4.o", [NVCC, *NV_FLAGS, "-DSGB_PREC=4", "-c", os.path.join(CSRC, "kern_air.cu")]),
        ("kern_table_p3.o", [NVCC, *NV_FLAGS, "-DSGB_PREC=3", "-c", os.path.join(CSRC, "kern_table.cu")]),
        ("kern_table_p4.o", [NVCC, *NV_FLAGS, "-DSGB_PREC=4", "-c", os.path.join(CSRC, "kern_table.cu")]),
        ("kern_table_p0.o", [NVCC, *NV_FLAGS, "-DSGB_PREC=0", "-c", os.path.join(CSRC, "kern_table.cu")]),
        ("kern_table_p1.o", [NVCC, *NV_FLAGS, "-DSGB_PREC=1", "-c", os.path.join(CSRC, "kern_table.cu")]),
        ("kern_table_p2.o", [NVCC, *NV_FLAGS, "-DSGB_PREC=2", "-c", os.path.join(CSRC, "kern_table.cu")]),
        ("kern_probe.o", [NVCC, *NV_FLAGS, "-c", os.path.join(CSRC, "kern_probe.cu")]),
        ("gpu_module.o", [NVCC, *NV_FLAGS, "-c", os.path.join(CSRC, "gpu_module.cu")]),
        ("static_scratch.o", [NVCC, *NV_FLAGS, "-c", os.path.join(CSRC, "static_scratch.cu")]),
        ("serve.o", [NVCC, *NV_FLAGS, "-c", os.path.join(CSRC, "serve.cu")]),
        ("dbd_driver.o", [NVCC, *NV_FLAGS, "-c", os.path.join(CSRC, "dbd_driver.cu")]),
        ("nft_transport.o", [NVCC, *NV_FLAGS, "-c", os.path.join(CSRC, "nft_transport.cu")]),
        ("kern_coop.o", [NVCC, *NV_FLAGS, "-c", os.path.join(CSRC, "kern_coop.cu")]),
        ("coop_build.o", [CXX, *CXX_FLAGS, "-c", os.path.join(CSRC, "coop_build.cpp")]),
        ("mech.o", [CXX, *CXX_FLAGS, "-c", os.path.join(CSRC, "mech.cpp")]),
        ("host_api.o", [CXX, *CXX_FLAGS, "-c", os.path.join(CSRC, "host_api.cpp")]),
    ]
    objs = []
    todo = []
    for name, cmd in units:
        obj = os.path.join(BUILD, name)
        objs.append(obj)
        src = cmd[-1]
        deps = [src, air_ops] + headers
        if force or _sources_newer(obj, deps):
            todo.append((cmd + ["-o", obj], os.path.join(BUILD, name + ".log")))
    with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo) or 1, os.cpu_count() or 4)) as ex:
        for fut in [ex.submit(_run, c, l) for c, l in todo]:
            fut.result()
    # 3. link
    if force or todo or not os.path.exists(LIB):
        _run([NVCC, ARCH, "-shared", "-o", LIB, *objs], os.path.join(BUILD, "link.log"))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
