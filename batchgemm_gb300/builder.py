"""Builds libbgemm_gb300.so in-tree for sm_103a (nvcc + g++, no cmake).

Translation units compile in parallel into ``batchgemm_gb300/_build`` and are
linked into ``batchgemm_gb300/libbgemm_gb300.so``.  The library links the
shared CUDA runtime (soname libcudart.so.13), so a process that already has
PyTorch's runtime loaded shares it.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INC = os.path.join(ROOT, "include")
# objects per host architecture, so a tree copied between an x86 and an Arm
# machine never links the other machine's objects
BUILD = os.path.join(PKG, "_build", platform.machine())
LIB = os.path.join(PKG, "libbgemm_gb300.so")
CLI_SRC = os.path.join(PKG, "cli", "bgemm_gemm.cpp")
CLI = os.path.join(PKG, "bgemm_gemm")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    hdr = sorted(f for f in os.listdir(CSRC) if f.endswith((".h", ".inc")))
    return cu, cpp, hdr


def _stale(obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, ptxas_verbose: bool = False) -> str:
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    cu, cpp, hdr = _sources()
    headers = [os.path.join(CSRC, h) for h in hdr] + [os.path.join(INC, "bgemm.h")]
    defs = []
    if os.path.exists(os.path.join(CSRC, "tile_table_tuned.inc")):
        defs.append("-DBGEMM_HAVE_TUNED_TABLE")
    jobs = []
    for f in cu:
        obj = os.path.join(BUILD, f + ".o")
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
               "--expt-relaxed-constexpr", "-I", INC, "-I", CSRC, *defs, "-c",
               os.path.join(CSRC, f), "-o", obj]
        if ptxas_verbose:
            cmd.insert(1, "-Xptxas=-v")
        jobs.append((obj, [os.path.join(CSRC, f)] + headers, cmd))
    for f in cpp:
        obj = os.path.join(BUILD, f + ".o")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function",
               "-I", INC, "-I", CSRC, "-I", os.path.join(cuda, "include"), *defs, "-c",
               os.path.join(CSRC, f), "-o", obj]
        jobs.append((obj, [os.path.join(CSRC, f)] + headers, cmd))

    todo = [(o, c) for (o, d, c) in jobs if force or _stale(o, d)]

    def run(job):
        obj, cmd = job
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
        out = (r.stdout + r.stderr).strip()
        return obj, out

    if todo:
        with cf.ThreadPoolExecutor(max_workers=min(len(todo), os.cpu_count() or 4)) as ex:
            for obj, out in ex.map(run, todo):
                if out and (verbose or ptxas_verbose):
                    print(out, flush=True)
    objs = [o for (o, _, _) in jobs]
    stamp = os.path.join(BUILD, "lib.stamp")
    if force or todo or _stale(LIB, objs) or _stale(stamp, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "shared",
               "-Xlinker", "-rpath=" + os.path.join(cuda, "lib64")]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
        os.replace(tmp, LIB)
        with open(stamp, "w") as f:
            f.write(platform.machine() + "\n")
    build_cli(cuda, verbose, force)
    return LIB


def build_cli(cuda: str, verbose: bool = False, force: bool = False) -> str:
    """The reference-compatible command-line benchmark (cli/bgemm_gemm.cpp),
    linked against the library next to it."""
    stamp = os.path.join(BUILD, "cli.stamp")
    deps = [CLI_SRC, LIB, os.path.join(INC, "bgemm.h")]
    if not force and os.path.exists(CLI) and not _stale(stamp, deps):
        return CLI
    tmp = CLI + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-I", INC, "-I", os.path.join(cuda, "include"),
           CLI_SRC, "-o", tmp, "-L", PKG, "-lbgemm_gb300", "-L", os.path.join(cuda, "lib64"),
           "-lcudart", "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + os.path.join(cuda, "lib64")]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("CLI build failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, CLI)
    with open(stamp, "w") as f:
        f.write(platform.machine() + "\n")
    return CLI


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv, ptxas_verbose="--ptxas" in sys.argv)
    print(LIB)
