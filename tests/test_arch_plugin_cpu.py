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


def test_plugin_failure_ends_the_process_with_the_message(pkg, tmp_path):
    """The hooks return void and MISA-MD has no error channel for them, so a failed call prints the
    library's message and aborts, as the reference's own failures end the job. Here cuda_domain_init
    gets a domain split over two ranks along x, which the plugin (one box on one GPU) rejects before
    touching a device, so the check runs the same with or without a GPU."""
    import signal
    pkg.build.build()
    names = golden()
    dom = next(n for n, d in names.items() if d.startswith("cuda_domain_init"))
    code = f'''
import ctypes, os, sys
lib = ctypes.CDLL({pkg.build.PLUGIN_PATH!r})
sup = ctypes.CDLL(sys.argv[1])
sup.th_domain_new.restype = ctypes.c_void_p
sup.th_domain_new.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_int32]
import numpy as np
cells = np.array([8, 8, 8], dtype=np.int64)
d = sup.th_domain_new(cells.ctypes.data, 2.855, 5.6 / 2.855, 2)
# a domain split over two ranks along x: the plugin runs one box on one GPU
ctypes.c_int64.from_address(d + 3 * 8).value = 4
getattr(lib, {dom!r}).argtypes = [ctypes.c_void_p]
getattr(lib, {dom!r})(d)
print("returned")
'''
    support = str(tmp_path / "libhooks_support.so")
    subprocess.run(["g++", "-std=c++11", "-O1", "-fPIC", "-shared", "-w", *pkg.build.plugin_include_flags(), "-o", support,
                    os.path.join(HERE, "arch_hooks_support.cpp")], check=True)
    r = subprocess.run([sys.executable, "-c", code, support], capture_output=True, text=True, timeout=120)
    assert r.returncode == -signal.SIGABRT, (r.returncode, r.stdout, r.stderr)
    assert "returned" not in r.stdout
    assert "misa_gb300 cuda_domain_init failed" in r.stderr
