"""Build recipe of libmisa_gb300.so: nvcc for sm_103a, translation units compiled in parallel.

The host translation units (.cpp) go through nvcc to the host compiler with -ffp-contract=off so the
spline coefficients round exactly as written; device code uses explicit rounding intrinsics where
the reference's results must be reproduced bit for bit.
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libmisa_gb300.so")
SOURCES = ["csrc/mg_kernels.cu", "csrc/mg_api.cpp", "csrc/mg_potential.cpp", "csrc/mg_noalloc.cu", "csrc/mg_world.cpp",
           "csrc/mg_dump.cpp", "csrc/mg_probe.cu"]
HEADERS = ["csrc/mg_internal.h", "../include/misa_gb300.h"]
# MISA-MD's accelerator plugin (the cuda_* hooks), built against the layout-compatible declarations in
# arch_cuda/tree and the stand-ins in arch_cuda/config, linked to the library above
PLUGIN_PATH = os.path.join(BUILD_DIR, "libmisa_arch_cuda.so")
PLUGIN_SOURCES = ["arch_cuda/cuda_arch.cpp"]
PLUGIN_HEADERS = ["../include/misa_gb300_arch.h", "arch_cuda/tree/atom/atom_element.h", "arch_cuda/tree/atom/neighbour_index.h",
                  "arch_cuda/tree/arch/arch_imp.h", "arch_cuda/tree/arch/arch_macros.h",
                  "arch_cuda/config/gen/arch_building_config.h", "arch_cuda/config/md_building_config.h",
                  "arch_cuda/config/comm/domain/bcc_domain.h", "arch_cuda/config/comm/domain/domain.h",
                  "arch_cuda/config/comm/domain/region.hpp", "arch_cuda/config/eam.h"]


def plugin_include_flags(tree: str | None = None) -> list:
    """Include directories of the plugin: MISA-MD's own src/ when given (tree), else the declarations in
    arch_cuda/tree; the stand-ins for the fetched packages and CMake-written headers either way."""
    cfg = os.path.join(HERE, "arch_cuda", "config")
    return ["-I", tree or os.path.join(HERE, "arch_cuda", "tree"), "-I", os.path.join(cfg, "gen"), "-I", cfg,
            "-I", os.path.join(HERE, "..", "include")]
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
              "-Xcompiler", "-fPIC,-ffp-contract=off"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmisa_gb300.so")
    return path


def _stale() -> bool:
    if not os.path.exists(LIB_PATH) or not os.path.exists(PLUGIN_PATH):
        return True
    t = min(os.path.getmtime(LIB_PATH), os.path.getmtime(PLUGIN_PATH))
    files = SOURCES + HEADERS + PLUGIN_SOURCES + PLUGIN_HEADERS + [os.path.relpath(__file__, HERE)]
    return any(os.path.getmtime(os.path.join(HERE, f)) > t for f in files)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile the library if a source is newer than it; returns the library path."""
    if not force and not _stale():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    cc = nvcc()
    objs = []
    cmds = []
    for src in SOURCES:
        obj = os.path.join(BUILD_DIR, os.path.splitext(os.path.basename(src))[0] + ".o")
        objs.append(obj)
        cmds.append([cc, *NVCC_FLAGS, "-c", "-o", obj, os.path.join(HERE, src)])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stdout + r.stderr

    with concurrent.futures.ThreadPoolExecutor(len(cmds)) as ex:
        for out in ex.map(run, cmds):
            if verbose and out.strip():
                print(out)
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    run([cc, *NVCC_FLAGS, "-shared", "-o", tmp, *objs, "-lcudart", "-lpthread"])
    os.replace(tmp, LIB_PATH)
    tmp = PLUGIN_PATH + f".tmp{os.getpid()}"
    run([os.environ.get("CXX", "g++"), "-std=c++11", "-O2", "-fPIC", "-shared", "-Wall", "-Wno-non-template-friend",
         *plugin_include_flags(), "-o", tmp, *[os.path.join(HERE, f) for f in PLUGIN_SOURCES],
         "-L" + BUILD_DIR, "-lmisa_gb300", "-Wl,-rpath,$ORIGIN"])
    os.replace(tmp, PLUGIN_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force=True, verbose=True))
