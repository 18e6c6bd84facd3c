"""MISA-MD's accelerator plugin (libmisa_arch_cuda.so) without a GPU: it builds, loads, and defines the
hooks under the linker names MISA-MD's own declarations give them; inside a checkout with the MISA-MD
tree, the same source also compiles against the reference's own headers (AtomElement's layout checks
then run against src/atom/atom_element.h) and the golden names are regenerated from them."""
import json
import os
import re
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE_SRC = "/root/reference/src"


def golden():
    with open(os.path.join(HERE, "golden", "reference_hook_symbols.json")) as f:
        return json.load(f)["symbols"]


def defined(path):
    out = subprocess.run(["nm", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    return set(re.findall(r" T (_Z\w+)", out))


def test_plugin_exports_the_reference_hook_names(pkg):
    import ctypes
    pkg.build.build()
    names = golden()
    assert len(names) == 8
    assert set(names) <= defined(pkg.build.PLUGIN_PATH)
    lib = ctypes.CDLL(pkg.build.PLUGIN_PATH)
    for n in names:
        assert hasattr(lib, n), n


@pytest.mark.skipif(not os.path.isdir(REFERENCE_SRC), reason="no MISA-MD tree in this checkout")
def test_plugin_compiles_against_the_reference_headers(pkg, tmp_path):
    obj = str(tmp_path / "cuda_arch.o")
    src = os.path.join(os.path.dirname(pkg.build.__file__), "arch_cuda", "cuda_arch.cpp")
    subprocess.run(["g++", "-std=c++11", "-w", *pkg.build.plugin_include_flags(REFERENCE_SRC), "-c", src, "-o", obj],
                   check=True)
    assert set(golden()) <= defined(obj)
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_hook_symbols
    assert make_hook_symbols.reference_symbols(REFERENCE_SRC) == golden()
