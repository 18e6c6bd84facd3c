"""Writes reference_hook_symbols.json: the linker names of MISA-MD's eight accelerator hooks for
ARCH_NAME = cuda, as the reference's own declarations produce them.

It compiles a probe that takes the address of each hook declared by the reference's
src/arch/arch_imp.h:16-32 (names pasted by src/arch/arch_macros.h:10-11), with the reference tree's
src/ on the include path and the plugin's stand-ins for the headers MISA-MD fetches or generates at
build time (libcomm, pot, md_building_config.h, arch_building_config.h), and lists the undefined
symbols of the object. Run in a checkout that has the MISA-MD tree:
    python tests/golden/make_hook_symbols.py /path/to/MISA-MD
"""
import json
import os
import re
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
HOOKS = ["env_init", "env_clean", "domain_init", "nei_offset_init", "pot_init", "eam_rho_calc", "eam_df_calc",
         "eam_force_calc"]
PROBE = """#include "arch/arch_imp.h"
void (*misa_gb300_probe[])() = {
%s
};
"""


def reference_symbols(reference_src):
    sys.path.insert(0, os.path.join(ROOT, "misa-md_gb300"))
    import build  # the plugin's include layout

    refs = ",\n".join(f"    reinterpret_cast<void (*)()>(&ARCH_PREFIX(ARCH_NAME, {h}))" for h in HOOKS)
    with tempfile.TemporaryDirectory() as tmp:
        src = os.path.join(tmp, "probe.cpp")
        obj = os.path.join(tmp, "probe.o")
        with open(src, "w") as f:
            f.write(PROBE % refs)
        subprocess.run(["g++", "-std=c++11", "-w", *build.plugin_include_flags(reference_src), "-c", src, "-o", obj],
                       check=True)
        nm = subprocess.run(["nm", "-u", obj], capture_output=True, text=True, check=True).stdout
    names = sorted(set(re.findall(r"\b(_Z\d+cuda_\w+)", nm)))
    demangled = subprocess.run(["c++filt", *names], capture_output=True, text=True, check=True).stdout.split("\n")
    return {n: d for n, d in zip(names, demangled)}


if __name__ == "__main__":
    tree = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    syms = reference_symbols(os.path.join(tree, "src"))
    assert len(syms) == len(HOOKS), syms
    with open(os.path.join(HERE, "reference_hook_symbols.json"), "w") as f:
        json.dump({"source": "src/arch/arch_imp.h:16-32 with ARCH_NAME = cuda", "symbols": syms}, f, indent=1)
        f.write("\n")
    print(json.dumps(syms, indent=1))
