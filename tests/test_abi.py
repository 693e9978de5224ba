"""The C ABI: every symbol declared in include/*.h is exported by libpfgpu.so
and has a ctypes signature; the ctypes structs have the C layout.  Runs on
the CPU (loading the library needs no GPU; nothing here launches a kernel)."""
import ctypes as C
import glob
import os
import re
import subprocess

import pytest

from pfgpu import abi

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = sorted(glob.glob(os.path.join(REPO, "include", "*.h")))


def declared_functions():
    names = set()
    for h in HEADERS:
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(pf_\w+)\s*\(", txt, flags=re.M):
            names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def lib():
    from pfgpu import build
    build.build()  # incremental: recompiles only changed translation units
    return abi.load()


def test_headers_declare_functions():
    names = declared_functions()
    assert {"pf_network_create", "pf_rstep", "pf_rstep_host", "pf_equilibrate_constraint"} <= names


def test_every_declared_symbol_is_exported(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name
        assert name in abi.SIGNATURES, name


def test_version(lib):
    assert lib.pf_version().startswith(b"pfgpu")


def _structs():
    return [v for v in vars(abi).values()
            if isinstance(v, type) and issubclass(v, C.Structure) and v.__name__.startswith("Pf")]


def _layout_c():
    """A C program printing sizeof and every field offset of each ctypes
    mirror, compiled against the header."""
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "pfgpu.h"', "int main(void) {"]
    for t in _structs():
        lines.append('  printf("%s %%zu\\n", sizeof(%s));' % (t.__name__, t.__name__))
        for f, _ in t._fields_:
            lines.append('  printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (t.__name__, f, t.__name__, f))
    lines += ["  return 0;", "}"]
    return "\n".join(lines) + "\n"


def test_struct_layout_matches_c(tmp_path):
    """Every struct of the ctypes mirror: size and every field offset equal
    the header's (the check a Fortran binding repeats with c_sizeof)."""
    structs = _structs()
    assert {t.__name__ for t in structs} >= {"PfOptions", "PfNetworkDesc", "PfCellState", "PfStepStats",
                                             "PfAdjointArgs", "PfGirtArgs", "PfTransportArgs",
                                             "PfTransportStats", "PfLaunchConfig"}
    src = tmp_path / "layout.c"
    src.write_text(_layout_c())
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-Wall", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    seen = 0
    for line in out:
        if not line.strip():
            continue
        key, val = line.split()
        val = int(val)
        if "." in key:
            t, f = key.split(".")
            assert getattr(getattr(abi, t), f).offset == val, key
        else:
            assert C.sizeof(getattr(abi, key)) == val, key
        seen += 1
    assert seen == sum(1 + len(t._fields_) for t in structs)


def test_invalid_network_rejected_without_gpu(lib):
    """Argument checking happens before any CUDA call."""
    d = abi.PfNetworkDesc()
    d.ncomp = 0
    h = C.c_void_p()
    assert lib.pf_network_create(C.byref(d), C.byref(h)) == abi.PF_ERR_INVALID
    d.ncomp = 99
    assert lib.pf_network_create(C.byref(d), C.byref(h)) == abi.PF_ERR_TOO_LARGE
    assert lib.pf_network_create(None, C.byref(h)) == abi.PF_ERR_INVALID
    assert lib.pf_rstep(None, None, 1.0, 0, None, None) == abi.PF_ERR_INVALID
