"""TEST INFRASTRUCTURE ONLY — build recipe for the reference kernels on the
host.

    python -m oracle.refcl.build [--force]

Compiles the reference's own OpenCL C kernels and headers (mcramp/moderator,
geom, scat and include of a RAMP checkout) as host C++ through
oracle/refcl/clshim.h and the sequencing driver oracle/refcl/driver.cpp:

* oracle/_ref/refcl_src/   the kernel sources after the one mechanical
  rewrite C++ needs: OpenCL vector literals "(floatN)(...)" and
  "(floatN){...}" become "floatN(...)" and "floatN{...}" (C++ would parse
  the first as a cast of a comma expression).  Nothing else is changed; the
  vendored Random123 headers are copied as they are.  Like the libraries,
  these generated files are git-ignored; where the checkout is absent (a
  machine the working tree was copied to) the libraries are built from
  them.
* oracle/_ref/librefcl_rmath.so  transcendental built-ins from
  ramp_gb300/csrc/rmath.h (the math library the oracle shares): compared
  with the oracle bit for bit.
* oracle/_ref/librefcl_libm.so   the C library's single-precision
  functions: compared within a relative tolerance.

Both use g++ -fsingle-precision-constant (unsuffixed constants are float, as
on an OpenCL device without cl_khr_fp64) and -ffp-contract=off.  Nothing is
built where neither the checkout nor the generated sources exist (none of
these files is committed), nor on machines other than x86 and powerpc, where
the reference's vendored Random123 headers stop the compilation.
"""
import os
import platform
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
SRC_OUT = os.path.join(OUT, "refcl_src")
LIBS = {"rmath": os.path.join(OUT, "librefcl_rmath.so"),
        "libm": os.path.join(OUT, "librefcl_libm.so")}

# the kernel files the driver includes, and the headers they include
KERNELS = ["moderator/flat_mod.cl", "moderator/cont_mod.cl", "moderator/isis_mod.cl",
           "scat/frametransform.cl", "scat/terminator.cl",
           "geom/plane.cl", "geom/cylinder_ext.cl", "geom/banana.cl", "geom/sphere.cl",
           "geom/sphere_int.cl", "geom/box.cl", "geom/arm.cl", "geom/mesh.cl",
           "scat/arm.cl", "scat/guide.cl", "scat/chopper.cl", "scat/isotropic.cl",
           "scat/powderN.cl", "scat/detector1D.cl", "scat/detector2D.cl", "scat/counter.cl",
           "scat/beamstop.cl", "scat/monochromator.cl", "scat/powder1.cl", "scat/rescal.cl"]
HEADERS = ["include/consts.h", "include/geom.h", "include/rand.h", "include/ref.h"]

_LITERAL = re.compile(r"\(\s*((?:float|real)(?:2|3|4|8|16)(?:_t)?)\s*\)\s*([({])")


def reference_root():
    from oracle import build as ob
    return ob.REFERENCE


def rewrite(text):
    """(floatN)( -> floatN(, (floatN){ -> floatN{ ; nothing else."""
    return _LITERAL.sub(r"\1\2", text)


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def generated_sources_present():
    return all(os.path.exists(os.path.join(SRC_OUT, f)) for f in KERNELS + HEADERS) and \
        os.path.isdir(os.path.join(SRC_OUT, "include", "Random123"))


def _generate(root, force):
    for f in KERNELS + HEADERS:
        dst = os.path.join(SRC_OUT, f)
        src = os.path.join(root, f)
        if force or _stale(dst, [src, __file__]):
            os.makedirs(os.path.dirname(dst), exist_ok=True)
            with open(src) as fh:
                text = fh.read()
            with open(dst + ".tmp", "w") as fh:
                fh.write(rewrite(text))
            os.replace(dst + ".tmp", dst)
    r123 = os.path.join(root, "include", "Random123")
    for d, _, files in os.walk(r123):
        for f in files:
            src = os.path.join(d, f)
            dst = os.path.join(SRC_OUT, "include", "Random123", os.path.relpath(src, r123))
            if force or _stale(dst, [src]):
                os.makedirs(os.path.dirname(dst), exist_ok=True)
                shutil.copyfile(src, dst + ".tmp")
                os.replace(dst + ".tmp", dst)


def supported_here():
    """The reference vendors Random123, whose compiler-feature header stops
    the build on machines other than x86 and powerpc (features/
    gccfeatures.h:37-40): on others (the aarch64 GPU hosts) nothing is
    built and the checker falls back to the oracle alone."""
    return platform.machine().lower() in ("x86_64", "amd64", "i386", "i686", "ppc64le", "ppc64")


UNSUPPORTED_REASON = ("the reference's vendored Random123 refuses to compile on %s "
                      "(Random123/features/gccfeatures.h:37-40: x86 and powerpc only)")


def build(force=False):
    if not supported_here():
        return None
    root = os.path.join(reference_root(), "mcramp")
    if os.path.isdir(root):
        _generate(root, force)
    elif not generated_sources_present():
        return None
    srcs = [os.path.join(SRC_OUT, f) for f in KERNELS + HEADERS]
    driver = os.path.join(HERE, "driver.cpp")
    shim = os.path.join(HERE, "clshim.h")
    rmath = os.path.join(os.path.dirname(ORACLE), "ramp_gb300", "csrc", "rmath.h")
    deps = srcs + [driver, shim, rmath, __file__]
    jobs = []
    for kind, lib in LIBS.items():
        if force or _stale(lib, deps):
            cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared",
                   "-fsingle-precision-constant", "-ffp-contract=off",
                   "-ftrivial-auto-var-init=zero", "-w",
                   "-I", os.path.join(SRC_OUT, "include"), "-I", SRC_OUT]
            if kind == "rmath":
                cmd.append("-DREFCL_RMATH")
            cmd += [driver, "-o", lib + ".tmp"]
            jobs.append((cmd, lib))
    procs = [(subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True),
              lib) for cmd, lib in jobs]
    for p, lib in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("reference kernel build failed:\n" + out[-6000:])
        os.replace(lib + ".tmp", lib)
    return LIBS


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
