"""TEST INFRASTRUCTURE ONLY — build recipes for the CPU oracle and for the
reference pins.

    python -m oracle.build

* oracle/_build/libramp_oracle.so  — the CPU restatement (oracle.cpp), g++
  with OpenMP and -ffp-contract=off.
* oracle/_ref/libref_pins.so       — the reference's own rand.h and ref.h
  compiled from where they lie in the reference checkout (only when that
  checkout is present; RAMP_REFERENCE overrides its location).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
ORACLE_LIB = os.path.join(HERE, "_build", "libramp_oracle.so")
PINS_LIB = os.path.join(HERE, "_ref", "libref_pins.so")
REFERENCE = os.environ.get("RAMP_REFERENCE", "/root/reference")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_oracle(force=False):
    src = os.path.join(HERE, "oracle.cpp")
    deps = [src, os.path.join(REPO, "include", "ramp.h"),
            os.path.join(REPO, "ramp_gb300", "csrc", "rmath.h"),
            os.path.join(REPO, "ramp_gb300", "csrc", "rconst.h")]
    if force or _stale(ORACLE_LIB, deps):
        os.makedirs(os.path.dirname(ORACLE_LIB), exist_ok=True)
        tmp = ORACLE_LIB + ".tmp"
        subprocess.run(["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC",
                        "-shared", src, "-o", tmp], check=True)
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def build_ref_pins(force=False):
    inc = os.path.join(REFERENCE, "mcramp", "include")
    if not os.path.isdir(inc):
        return None
    src = os.path.join(HERE, "ref_pins", "pins.c")
    shim = os.path.join(HERE, "ref_pins", "shim.h")
    if force or _stale(PINS_LIB, [src, shim, os.path.join(inc, "rand.h"),
                                  os.path.join(inc, "ref.h")]):
        os.makedirs(os.path.dirname(PINS_LIB), exist_ok=True)
        tmp = PINS_LIB + ".tmp"
        subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-std=gnu99", "-include", shim,
                        "-ftrivial-auto-var-init=zero", "-I", inc, src,
                        "-o", tmp, "-lm"], check=True)
        os.replace(tmp, PINS_LIB)
    return PINS_LIB


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref_pins(force="--force" in sys.argv))
