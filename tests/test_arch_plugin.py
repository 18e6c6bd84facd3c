"""MISA-MD's accelerator hooks, called by their reference names (GPU).

libmisa_arch_cuda.so exports the eight functions that MISA-MD's src/arch/arch_imp.h:16-32 declares for
ARCH_NAME = cuda, under the linker names the reference's own declarations give them
(tests/golden/reference_hook_symbols.json). This test calls them through ctypes by those names, in the
order MISA-MD's loop does: cuda_env_init, cuda_domain_init, cuda_nei_offset_init, cuda_pot_init, then
per computeEam cuda_eam_rho_calc, the host's rho fold (which adds the zeros left in ghost slots),
cuda_eam_df_calc, the host's forward df exchange, cuda_eam_force_calc; finally cuda_env_clean. The host
slot array is the AoS record array itself, ghost slots filled by the oracle's first exchange. Results
against the oracle's computeEam on the same state: FP64 rho within rel 1e-13 and forces within
1e-9 eV/A; mixed within its error budget.
"""
import ctypes
import json
import os
import subprocess

import numpy as np
import pytest

from test_gpu_parity import A0, RCF, F64_TOL, MIX_RMS, ghosts, local

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def hook_names():
    with open(os.path.join(HERE, "golden", "reference_hook_symbols.json")) as f:
        syms = json.load(f)["symbols"]
    return {d.split("(")[0]: mangled for mangled, d in syms.items()}


@pytest.fixture(scope="module")
def plugin(pkg, gpu_lib, tmp_path_factory):
    lib = ctypes.CDLL(pkg.build.PLUGIN_PATH)
    support = str(tmp_path_factory.mktemp("hooks") / "libhooks_support.so")
    subprocess.run(["g++", "-std=c++11", "-O1", "-fPIC", "-shared", "-w", *pkg.build.plugin_include_flags(),
                    "-o", support, os.path.join(HERE, "arch_hooks_support.cpp")], check=True)
    sup = ctypes.CDLL(support)
    P, I32, I64, D = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double
    sup.th_domain_new.restype = P
    sup.th_domain_new.argtypes = [P, D, D, I32]
    sup.th_domain_free.argtypes = [P]
    sup.th_neighbour_index_new.restype = P
    sup.th_neighbour_index_new.argtypes = [P, P, I32, P, P, I32]
    sup.th_neighbour_index_free.argtypes = [P]
    hooks = {}
    for short, mangled in hook_names().items():
        fn = getattr(lib, mangled)
        fn.restype = None
        if short.startswith("cuda_eam_"):
            fn.argtypes = [P, P, D]
        elif short in ("cuda_env_init", "cuda_env_clean"):
            fn.argtypes = []
        else:
            fn.argtypes = [P]
        hooks[short] = fn
    return hooks, sup


def _owner_map(wl, cells):
    """Owner slot of every slot under the periodic self-exchange (the host's forward df exchange)."""
    Sx, Sy, Sz, gx, gy, gz = wl.grid(cells, RCF)
    s = np.arange(Sx * Sy * Sz)
    X, Y, Z = s % Sx, (s // Sx) % Sy, s // (Sx * Sy)
    bx, by, bz = 2 * cells[0], cells[1], cells[2]
    X = np.where(X < gx, X + bx, np.where(X >= gx + bx, X - bx, X))
    Y = np.where(Y < gy, Y + by, np.where(Y >= gy + by, Y - by, Y))
    Z = np.where(Z < gz, Z + bz, np.where(Z >= gz + bz, Z - bz, Z))
    return (Z * Sy + Y) * Sx + X


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_hooks_by_reference_names(pkg, orc, wl, potentials, plugin, prec, monkeypatch):
    hooks, sup = plugin
    cells = (9, 8, 10)
    pot = potentials["fecuni"]
    atoms = wl.build_state(cells, A0, RCF, temperature=600.0, seed=71, cu_frac=0.05, ni_frac=0.04)
    loc = local(wl, cells)
    atoms["x"][loc] += np.random.default_rng(7).uniform(-0.1, 0.1, size=(loc.size, 3))
    atoms["type"][loc[11::89]] = -1
    ref = orc.OracleSim(cells, A0, RCF, pot)
    ref.set_atoms(atoms)
    ref.exchange_atom_first()
    ref.clear_force()
    host = np.ascontiguousarray(ref.get_atoms())  # the state atom::latRho sees: ghosts filled, rho = f = 0
    ref.compute_eam()
    want = ref.get_atoms()
    ref.close()

    monkeypatch.setenv("MISA_GB300_SETFL", pot)
    monkeypatch.setenv("MISA_GB300_PRECISION", prec)
    monkeypatch.setenv("MISA_GB300_DEVICE", "0")
    Sx, Sy, Sz, _, _, _ = wl.grid(cells, RCF)
    tables = [np.ascontiguousarray(orc.nei_offsets(Sx, Sy, Sz, 2, RCF, w)) for w in range(4)]
    ps = np.asarray(cells, dtype=np.int64)
    dom = sup.th_domain_new(ps.ctypes.data, A0, RCF, 2)
    nei = sup.th_neighbour_index_new(tables[0].ctypes.data, tables[1].ctypes.data, tables[0].size,
                                     tables[2].ctypes.data, tables[3].ctypes.data, tables[2].size)
    hooks["cuda_env_init"]()
    hooks["cuda_domain_init"](dom)
    hooks["cuda_nei_offset_init"](nei)
    hooks["cuda_pot_init"](None)
    rc = A0 * RCF
    ptr = host.ctypes.data
    hooks["cuda_eam_rho_calc"](None, ptr, rc)
    g = ghosts(wl, cells)
    assert (host["rho"][g] == 0).all()       # the reverse rho fold that follows adds nothing
    rtol = 1e-13 if prec == "fp64" else 1e-6
    assert np.allclose(host["rho"][loc], want["rho"][loc], rtol=rtol, atol=0)
    hooks["cuda_eam_df_calc"](None, ptr, rc)
    occ = loc[want["type"][loc] >= 0]
    assert np.allclose(host["df"][occ], want["df"][occ], rtol=1e-12 if prec == "fp64" else 1e-6)
    own = _owner_map(wl, cells)
    host["df"][g] = host["df"][own[g]]       # the host's forward df exchange (DfEmbedPacker)
    hooks["cuda_eam_force_calc"](None, ptr, rc)
    d = host["f"][occ] - want["f"][occ]
    if prec == "fp64":
        assert np.abs(d).max() <= F64_TOL
    else:
        assert np.sqrt((d ** 2).mean()) <= MIX_RMS
    assert (host["f"][loc[want["type"][loc] < 0]] == 0).all()
    hooks["cuda_env_clean"]()
    sup.th_domain_free(dom)
    sup.th_neighbour_index_free(nei)
