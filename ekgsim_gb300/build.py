"""Build the engine in-tree: ``ekgsim_gb300/libekgsim_gb300.so`` (CUDA, sm_103a) and the
command-line front ends in ``ekgsim_gb300/bin/`` (``ekgSim``, ``ekgsim_extern``).

Translation units compile in parallel with nvcc (one -gencode, sm_103a only); the host
programs link against the shared library with an rpath to it.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
MACHINE = platform.machine()
BUILD = os.path.join(PKG, "_build", MACHINE)
LIB = os.path.join(PKG, "libekgsim_gb300.so")
BIN = os.path.join(PKG, "bin")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code keeps the reference's FP64 rounding: no fused multiply-add (gcc fuses by default on aarch64)
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
           "-Xcompiler", "-ffp-contract=off",
           "-diag-suppress", "177,550", "-I", os.path.join(ROOT, "include")]

SOURCES = ["ca.cu", "ecg.cu", "umma.cu", "batch.cu", "setup.cu", "engine.cpp", "host_model.cpp", "server.cpp"]
PROGRAMS = {"ekgSim": ["cli_main.cpp"], "ekgsim_extern": ["extern_main.cpp"]}


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _arch_ok(path):
    stamp = path + ".arch"
    return os.path.exists(path) and os.path.exists(stamp) and open(stamp).read().strip() == MACHINE


def _stamp(path):
    with open(path + ".arch", "w") as f:
        f.write(MACHINE + "\n")


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile what is missing or stale (a library built on another architecture is stale)."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(BIN, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".h")]
    headers.append(os.path.join(ROOT, "include", "ekgsim.h"))
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    objs = []
    jobs = []
    for s in srcs:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmd = [NVCC] + ARCH + NVFLAGS + ["-c", src, "-o", obj]
            if s.endswith(".cpp"):
                cmd = [NVCC] + ARCH + NVFLAGS + ["-x", "cu", "-c", src, "-o", obj]
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for r in ex.map(_run, jobs):
            if verbose and (r.stdout or r.stderr):
                print(r.stdout + r.stderr, file=sys.stderr)
    lib_stale = force or not _arch_ok(LIB) or _stale(LIB, objs)
    if lib_stale:
        tmp = LIB + f".{os.getpid()}.tmp"
        _run([NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcuda"])
        os.replace(tmp, LIB)
        _stamp(LIB)
    for prog, files in PROGRAMS.items():
        srcs_p = [os.path.join(CSRC, f) for f in files if os.path.exists(os.path.join(CSRC, f))]
        if not srcs_p:
            continue
        out = os.path.join(BIN, prog)
        if lib_stale or not _arch_ok(out) or _stale(out, srcs_p + [LIB] + headers):
            tmp = out + f".{os.getpid()}.tmp"
            _run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), "-o", tmp] + srcs_p +
                 ["-L", PKG, "-lekgsim_gb300", "-Wl,-rpath,$ORIGIN/..", "-lpthread"])
            os.replace(tmp, out)
            _stamp(out)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
