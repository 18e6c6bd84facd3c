"""C-ABI library: builds for sm_103a, loads without a GPU, exports every declared entry point."""
import ctypes
import os
import re
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "misa_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mg_[a-z0-9_]+)\s*\(", src)))


def test_library_builds_and_exports(pkg):
    path = pkg.build.build()
    lib = ctypes.CDLL(path)
    names = declared_symbols()
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), n
    nm = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (mg_[a-z0-9_]+)", nm))
    assert set(names) <= exported
    # the Python bindings cover the same set
    assert set(names) == set(pkg.exported_symbols())


def test_library_targets_sm103a(pkg):
    path = pkg.build.build()
    out = subprocess.run(["cuobjdump", "--list-elf", path], capture_output=True, text=True).stdout
    assert "sm_103a" in out


def test_record_layout(pkg):
    dt = pkg.ATOM_DTYPE
    assert dt.itemsize == 104
    assert [dt.fields[k][1] for k in ("id", "type", "x", "v", "f", "rho", "df")] == [0, 8, 16, 40, 64, 88, 96]


def test_workload_generator(wl):
    cells = (6, 7, 8)
    rcf = 5.6 / 2.855
    a = wl.build_state(cells, 2.855, rcf, temperature=600.0, seed=5, cu_frac=0.1, ni_frac=0.05)
    loc = wl.local_slot_indices(cells, rcf)
    n = loc.size
    assert n == 2 * 6 * 7 * 8
    assert np.array_equal(a["id"][loc], np.arange(1, n + 1))
    assert (a["type"][np.setdiff1d(np.arange(a.size), loc)] == -1).all()
    t = a["type"][loc]
    assert (t == 1).sum() == round(0.1 * n) and (t == 2).sum() == round(0.05 * n)
    m = np.asarray(wl.MASS)[t]
    v = a["v"][loc]
    temp = (m * (v * v).sum(axis=1)).sum() * wl.MVV2E / ((3 * n - 3) * wl.BOLTZ)
    assert abs(temp - 600.0) < 1e-9
    assert np.abs((m[:, None] * v).sum(axis=0)).max() < 1e-9
    # WorldBuilder positions (src/world_builder.cpp:120-124)
    i = np.arange(12)
    assert np.array_equal(a["x"][loc[:12], 0], (i * 0.5) * 2.855)


def test_setfl_roundtrip(wl, orc, tmp_path):
    spec = wl.PotentialSpec(n_ele=3, seed=2, nr=200, nrho=200)
    path = wl.write_setfl(str(tmp_path / "p.setfl"), spec)
    F, rho, rphi, drho, dr = wl.potential_tables(spec)
    s = orc.OracleSim((6, 6, 6), 2.855, 5.6 / 2.855, path)
    # the spline passes through the knots exactly (c0 = f)
    assert np.array_equal(s.pot_spline(1, 1)[:, 0], rho[1])
    assert np.array_equal(s.pot_spline(2, 2, 1)[:, 0], rphi[4])
    assert np.array_equal(s.pot_spline(0, 0)[:, 0], F[0])
