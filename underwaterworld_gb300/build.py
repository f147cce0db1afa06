"""Build libuww_gb300.so (sm_103a) in-tree, and the CPU oracle.

``python -m underwaterworld_gb300.build`` or ``build()`` from Python.  Every
CUDA translation unit is compiled in parallel with
``-gencode arch=compute_103a,code=sm_103a``; the objects are linked into
``underwaterworld_gb300/_build/libuww_gb300.so`` with the CUDA runtime linked
statically, so the library needs no torch and no extra shared objects.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libuww_gb300.so"

SOURCES = ["uww_build.cu", "uww_api.cu", "uww_noalloc.cu", "uww_adjoint.cu", "uww_tune.cu", "uww_sample.cu", "uww_query.cu", "uww_schedule.cu", "uww_shade.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              f"-I{ROOT / 'include'}", f"-I{CSRC}"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libuww_gb300")
    return cand


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False, extra_flags=()) -> Path:
    OUT.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "uww.h"]
    cc = nvcc()
    objs = []
    jobs = []
    for src in SOURCES:
        s = CSRC / src
        o = OUT / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s, *headers]):
            cmd = [cc, *ARCH, *NVCC_FLAGS, *extra_flags, "-c", str(s), "-o", str(o)]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode:
                raise RuntimeError(f"nvcc failed: {' '.join(cmd)}")
    if force or jobs or _stale(LIB, objs):
        cmd = [cc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-cudart", "static",
               "-Xcompiler", "-fPIC"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link of libuww_gb300.so failed")
    build_host()
    build_probe(force=force)
    return LIB


PROBE_LIB = OUT / "libuww_bench_probe.so"


def build_probe(force: bool = False) -> Path:
    """The benchmark's measurement kernels (FP32 peak, host-write bandwidth),
    a library of their own: they are not part of the chunk builder's ABI."""
    OUT.mkdir(exist_ok=True)
    src = CSRC / "bench_probe.cu"
    if force or _stale(PROBE_LIB, [src]):
        cmd = [nvcc(), *ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-cudart", "static",
               str(src), "-o", str(PROBE_LIB)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("build of libuww_bench_probe.so failed")
    return PROBE_LIB


def build_oracle() -> Path:
    """Build the CPU oracle (test infrastructure) with its own Makefile."""
    r = subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], capture_output=True, text=True)
    if r.returncode:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("oracle build failed")
    return ROOT / "oracle" / "_build" / "liboracle.so"


HOST = PKG / "host"
HOST_LIB = OUT / "libuww_host.so"
# the C++ chunk interface over the C ABI; -ffp-contract=off keeps Tri's f32
# arithmetic in the reference's (unfused) order
HOST_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-variable",
              f"-I{ROOT / 'include'}", f"-I{CSRC}", f"-I{HOST}"]


def build_host(force: bool = False) -> Path:
    srcs = [HOST / "uww_chunk.cpp"]
    deps = srcs + [HOST / "uww_chunk.hpp", ROOT / "include" / "uww.h", CSRC / "mc_tables.h", LIB]
    if force or _stale(HOST_LIB, deps):
        cmd = [shutil.which("g++") or "g++", *HOST_FLAGS, "-shared", "-o", str(HOST_LIB), *map(str, srcs),
               f"-L{OUT}", "-luww_gb300", f"-Wl,-rpath,{OUT}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("build of libuww_host.so failed")
    return HOST_LIB


def build_host_program(src: Path, exe: Path) -> Path:
    """Compile a C++ program against the host interface (tests)."""
    build_host()
    cmd = [shutil.which("g++") or "g++", *HOST_FLAGS, "-o", str(exe), str(src), f"-L{OUT}", "-luww_host",
           "-luww_gb300", f"-Wl,-rpath,{OUT}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("compile failed:\n" + r.stdout + r.stderr)
    return exe


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    build_oracle()
    print(LIB)
