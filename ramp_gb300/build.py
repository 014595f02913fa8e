"""Build libramp_cuda.so (sm_103a) in-tree with nvcc.

    python -m ramp_gb300.build [--force]

Translation units are compiled in parallel; the library links the CUDA
runtime statically, so it loads on machines without a GPU (every call then
returns an error).  Device code is compiled with -fmad=false and host code
with -ffp-contract=off: one rounding per floating-point operation, which is
what keeps the GPU results bit-identical to the CPU oracle.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libramp_cuda.so")

CU_SOURCES = ["plain.cu", "fused.cu", "adjoint.cu", "abi.cu"]
# fused_inst.cu once per kernel instantiation: (register cap, keying mode,
# batched one-launch layout, phase, kind set); kind sets: 0 core kinds, 1
# everything (extended kinds and the mesh), 2 core kinds and the mesh.  The
# batched layout runs the extended kinds whole (phase 0 only); phase 4
# (stage B walking a mesh per lane) and phase 5 (finishing the walked
# survivors) exist for kind set 2, phase 3 (stage A
# of a split before component 0: the moderator and the chopper look-ahead)
# for kind set 0
FUSED_INSTANCES = ([(mb, mode, b, ph, ks) for mb in (3, 4) for mode in (0, 1) for b in (0, 1)
                    for ks in (0, 1, 2) for ph in (0, 1, 2) if not (b and ks == 1 and ph)]
                   + [(mb, mode, b, 4, 2) for mb in (3, 4) for mode in (0, 1) for b in (0, 1)]
                   + [(mb, mode, b, 3, 0) for mb in (3, 4) for mode in (0, 1) for b in (0, 1)]
                   + [(mb, mode, b, 5, 2) for mb in (3, 4) for mode in (0, 1) for b in (0, 1)])
CPP_SOURCES = ["bvh.cpp"]
HEADERS = ["device.cuh", "fused_kernel.cuh", "mesh.cuh", "lookahead.h", "plan.h", "launch.h", "rmath.h",
           "rconst.h", "bvh.h",
           os.path.join("..", "..", "include", "ramp.h")]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true",
                     "-prec-sqrt=true", "-ftz=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "-Xptxas", "-warn-spills"]
CXX_FLAGS = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("build failed:\n%s\n%s%s" % (" ".join(cmd), p.stdout, p.stderr))
    return p.stdout + p.stderr


def build(force=False, verbose=False, extra_nvcc=()):
    os.makedirs(OUT, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _stale(o, [s, __file__] + hdrs):
            jobs.append([nvcc()] + NVCC_FLAGS + list(extra_nvcc) + ["-c", s, "-o", o])
    fs = os.path.join(CSRC, "fused_inst.cu")
    # the batched kernels take longest to compile: start them first
    for inst in sorted(FUSED_INSTANCES, key=lambda t: -t[2]):
        o = os.path.join(OUT, "fused_inst_%d%d%d%d%d.o" % inst)
        objs.append(o)
        if force or _stale(o, [fs, __file__] + hdrs):
            defs = ["-DFK_%s=%d" % kv for kv in zip(("MINB", "MODE", "BATCHED", "PHASE", "EXT"), inst)]
            jobs.append([nvcc()] + NVCC_FLAGS + list(extra_nvcc) + defs + ["-c", fs, "-o", o])
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _stale(o, [s, __file__] + hdrs):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", s, "-o", o])
    logs = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 8)) as ex:
            for out in ex.map(_run, jobs):
                logs.append(out)
    if force or jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        _run([nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-Xcompiler", "-fPIC"])
        os.replace(tmp, LIB)
    if verbose:
        for l in logs:
            if l.strip():
                print(l)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True,
                extra_nvcc=["-Xptxas", "-v"] if "-v" in sys.argv else []))
