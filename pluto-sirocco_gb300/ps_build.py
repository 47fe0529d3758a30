"""Build recipe for libps_gb300.so (the C-ABI library) and the CPU oracle.

    python pluto-sirocco_gb300/ps_build.py            # library + oracle
    python pluto-sirocco_gb300/ps_build.py --lib      # library only

CUDA sources are compiled for sm_103a only, in parallel.  Device code
contracts multiplies and adds into FMAs (nvcc's default -fmad=true) and
keeps the IEEE-rounded division and square root that nvcc uses for double;
against the reference's x86-64 build (no FMA) this changes results at the
level of 1e-16 to 1e-13 relative after 100 steps, far inside the 1e-11
tolerance the parity tests hold it to.  Host C sources (grid and initial
conditions, which the parity tests compare exactly) are compiled with gcc
-ffp-contract=off.  The outputs stay in-tree next to the sources.
"""
import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
INC = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libps_gb300.so")
PROBE_SRC = os.path.join(PKG, "probe", "ps_probe.cu")
PROBE = os.path.join(PKG, "libps_probe.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-fmad=true", "-lineinfo", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-ffp-contract=off", "-I" + INC, "-I" + CSRC]
CFLAGS = ["-O3", "-std=c17", "-ffp-contract=off", "-fPIC", "-Wall", "-I" + INC]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _newer(src_list, out):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in src_list)


def build_lib(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    headers.append(os.path.join(INC, "ps_gb300.h"))
    jobs = []
    objs = []
    for f in sorted(os.listdir(CSRC)):
        if f.endswith(".cu"):
            src = os.path.join(CSRC, f)
            obj = os.path.join(BUILD, f[:-3] + ".o")
            objs.append(obj)
            if force or _newer([src] + headers, obj):
                jobs.append([nv] + ARCH + NVFLAGS + ["-c", src, "-o", obj])
    for f in sorted(os.listdir(HOST)):
        if f.endswith(".c"):
            src = os.path.join(HOST, f)
            obj = os.path.join(BUILD, f[:-2] + ".o")
            objs.append(obj)
            if force or _newer([src, os.path.join(INC, "ps_gb300.h")], obj):
                jobs.append(["gcc"] + CFLAGS + ["-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    if force or jobs or not os.path.exists(LIB):
        _run([nv] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    build_probe(force)
    return LIB


def build_probe(force=False):
    """libps_probe.so: measurement helpers for bench.py and the tests (the
    FP64 issue-rate probe, the fast-math check, the integer product's rate
    and check); not part of the C ABI."""
    deps = [PROBE_SRC, os.path.join(CSRC, "ps_fastmath.cuh"),
            os.path.join(CSRC, "ps_fastmath_tables.cuh"), os.path.join(CSRC, "ps_dmul.cuh"),
            os.path.join(CSRC, "ps_tma.cuh")]
    if force or _newer(deps, PROBE):
        _run([nvcc()] + ARCH + NVFLAGS + ["-shared", PROBE_SRC, "-o", PROBE, "-lcudart"])
    return PROBE


def build_oracle():
    _run(["make", "-s", "-C", os.path.join(ROOT, "oracle")])
    return os.path.join(ROOT, "oracle", "liboracle.so")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--lib", action="store_true")
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", action="store_true")
    a = ap.parse_args()
    print(build_lib(force=a.force, verbose=a.v))
    if not a.lib:
        print(build_oracle())


if __name__ == "__main__":
    sys.exit(main())
