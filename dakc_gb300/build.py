"""In-tree build of the engine's native parts (no cmake, no pip install).

* ``_build/libdakc_gb300.so`` -- the engine: sm_103a kernels + C++ host
  pipeline + C ABI (include/dakc_gb300.h), compiled by nvcc for
  ``-gencode arch=compute_103a,code=sm_103a`` only.
* ``_build/dakc-gpu`` -- the command-line counter (host C++ over the C ABI,
  linked against the engine library beside it).
* ``synth/_build/libdk_synth.so`` -- the seeded workload generator (host C++).

Translation units compile in parallel; a rebuild is skipped when the library
is newer than every source.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
ENGINE_SO = os.path.join(BUILD, "libdakc_gb300.so")
CLI = os.path.join(BUILD, "dakc-gpu")
SYNTH_SO = os.path.join(HERE, "synth", "_build", "libdk_synth.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _stale(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_engine(force: bool = False, verbose: bool = False) -> str:
    units = sorted(glob.glob(os.path.join(CSRC, "*.cu")))  # the engine: every .cu file
    deps = units + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.hpp")) + \
        [os.path.join(ROOT, "include", "dakc_gb300.h")]
    if not force and not _stale(ENGINE_SO, deps):
        return ENGINE_SO
    os.makedirs(BUILD, exist_ok=True)
    flags = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
             *ARCH, "-diag-suppress", "550"]
    procs, objs = [], []
    for u in units:
        obj = os.path.join(BUILD, os.path.basename(u) + ".o")
        objs.append(obj)
        cmd = [nvcc(), *flags, "-c", u, "-o", obj]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                                            text=True)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{out}")
        if verbose and out:
            sys.stderr.write(out)
    tmp = ENGINE_SO + ".tmp"
    cmd = [nvcc(), "-shared", *ARCH, "-o", tmp, *objs, "-lcudart"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{p.stdout}{p.stderr}")
    os.replace(tmp, ENGINE_SO)
    return ENGINE_SO


def build_synth(force: bool = False) -> str:
    src = os.path.join(HERE, "synth", "dk_synth.cpp")
    if not force and not _stale(SYNTH_SO, [src]):
        return SYNTH_SO
    os.makedirs(os.path.dirname(SYNTH_SO), exist_ok=True)
    tmp = SYNTH_SO + ".tmp"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-Wall", "-o", tmp,
           src, "-lpthread"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, SYNTH_SO)
    return SYNTH_SO


def build_cli(force: bool = False) -> str:
    """The command-line counter; it finds the engine library beside itself."""
    src = os.path.join(CSRC, "dk_cli.cpp")
    header = os.path.join(ROOT, "include", "dakc_gb300.h")
    if not force and not _stale(CLI, [src, header, ENGINE_SO]):
        return CLI
    tmp = CLI + ".tmp"
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-I", os.path.join(ROOT, "include"), "-o", tmp, src,
           "-L", BUILD, "-ldakc_gb300", "-Wl,-rpath,$ORIGIN"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"g++ failed: {' '.join(cmd)}\n{p.stdout}{p.stderr}")
    os.replace(tmp, CLI)
    return CLI


def build_all(force: bool = False) -> None:
    build_synth(force)
    build_engine(force)
    build_cli(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print(ENGINE_SO)
