"""The C-ABI library: it builds, loads without a GPU and exports every entry
point include/ramp.h declares; the ctypes mirror matches the header."""
import ctypes
import os
import re

import pytest

from ramp_gb300 import _abi, build

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "ramp.h")


def declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^(?:int|int64_t)\s+(ramp_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _abi.load()


def test_every_declared_symbol_is_exported(lib):
    names = declared()
    assert len(names) >= 12
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(_abi.exported_symbols())


def test_version_and_error_string(lib):
    assert lib.ramp_version() == 1
    buf = ctypes.create_string_buffer(64)
    assert lib.ramp_last_error(buf, 64) == 0


def test_struct_sizes_match_header_layout():
    assert ctypes.sizeof(_abi.RampComp) == 464
    assert ctypes.sizeof(_abi.RampSource) == 136
    assert ctypes.sizeof(_abi.RampRng) == 24
    assert ctypes.sizeof(_abi.RampState) == 24


def test_invalid_arguments_are_rejected_without_a_gpu(lib):
    out = ctypes.c_void_p()
    assert lib.ramp_plan_create(None, None, 0, None, 0, ctypes.byref(out)) == -1
    assert "invalid" in _abi.last_error(lib)
    src = _abi.RampSource()
    src.kind = 99
    assert lib.ramp_plan_create(ctypes.byref(src), None, 0, None, 0, ctypes.byref(out)) == -5
    assert lib.ramp_trace_fused(None, 10, 10, 0, None, None, None, None, None) == -1
    assert lib.ramp_plan_destroy(None) == 0


C_CALLER = r"""
#include <stdio.h>
#include <string.h>
#include "ramp.h"
int main(void) {
  RampPlan* plan = NULL;
  RampSource src;
  char msg[256];
  memset(&src, 0, sizeof src);
  if (ramp_version() != 1) return 1;
  /* no components and no GPU: an error code, never a crash */
  int rc = ramp_plan_create(NULL, NULL, 0, NULL, 0, &plan);
  if (rc >= 0) return 2;
  ramp_last_error(msg, sizeof msg);
  printf("%d %zu %zu %s\n", rc, sizeof(RampComp), sizeof(RampSource), msg);
  return 0;
}
"""


def test_header_is_plain_c_and_links(lib, tmp_path):
    """include/ramp.h compiles as C11 (no C++ or torch types) and a C
    program links against libramp_cuda.so and calls it."""
    import subprocess
    src = tmp_path / "caller.c"
    src.write_text(C_CALLER)
    exe = tmp_path / "caller"
    libdir = os.path.dirname(_abi.LIB_PATH)
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-I", os.path.dirname(HEADER),
                    str(src), "-L", libdir, "-lramp_cuda", "-Wl,-rpath," + libdir, "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert int(out[0]) < 0
    assert int(out[1]) == ctypes.sizeof(_abi.RampComp)
    assert int(out[2]) == ctypes.sizeof(_abi.RampSource)
