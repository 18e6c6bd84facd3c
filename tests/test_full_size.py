"""Size-independent properties at the benchmark's full sizes (GPU).

The oracle finishes only small boxes in seconds, so the full-size workloads are checked through
properties that hold at any size: forces vanish on a perfect lattice, forces sum to zero, identical
inputs give identical bits, the mixed form stays within its error budget against the FP64 form on
the 16M-atom alloy, and a 2M-atom cascade conserves its atoms (ids, Frenkel pairs) and its energy.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

A0 = 2.855
RCF = 5.6 / A0


def _ctx(pkg, cells, prec, pot, atoms, dt=0.001, cap=0):
    c = pkg.Context(cells, A0, RCF, precision=prec, inter_capacity=cap)
    c.pot_init_setfl(pot)
    c.set_timestep(dt)
    c.upload(atoms)
    c.prepare()
    return c


@pytest.fixture(scope="module")
def fe_pot(wl, tmp_path_factory):
    w = wl.WORKLOADS["fe_100c"]
    return wl.workload_potential(w, str(tmp_path_factory.mktemp("fe100")))


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_fe_100c_perfect_lattice_sum_and_determinism(pkg, wl, gpu_lib, fe_pot, prec):
    """2,000,000-atom Fe: perfect-lattice forces vanish; a 600 K state keeps sum f ~ 0 over 20 steps
    and reruns bit for bit."""
    cells = (100, 100, 100)
    loc = wl.local_slot_indices(cells, RCF)
    perfect = wl.build_state(cells, A0, RCF, temperature=0.0, seed=1)
    c = _ctx(pkg, cells, prec, fe_pot, perfect)
    got, _ = c.download()
    assert np.abs(got["f"][loc]).max() < (1e-12 if prec == "fp64" else 1e-5)
    state = wl.workload_state(wl.WORKLOADS["fe_100c"])
    c.upload(state)
    c.prepare()
    c.simulate(20)
    t = c.thermo()
    assert t["device_errors"] == 0
    assert np.abs(t["force_sum"]).max() / loc.size < (1e-13 if prec == "fp64" else 1e-7)
    a1, _ = c.download()
    c.upload(state)
    c.prepare()
    c.simulate(20)
    a2, _ = c.download()
    for f in ("x", "v", "f"):
        assert np.array_equal(a1[f], a2[f]), f
    c.close()


def test_fecuni_200c_mixed_error_budget(pkg, wl, gpu_lib, tmp_path):
    """16,000,000-atom Fe-Cu-Ni (the benchmark workload): mixed forces against FP64 forces on the same
    600 K state, after 10 steps of each: RMS <= 1e-5 eV/A, max <= 1e-4 eV/A."""
    w = wl.WORKLOADS["fecuni_200c"]
    pot = wl.workload_potential(w, str(tmp_path))
    state = wl.workload_state(w)
    loc = wl.local_slot_indices(w.cells, RCF)
    c64 = _ctx(pkg, w.cells, "fp64", pot, state)
    c64.simulate(10)
    s64, _ = c64.download()
    c64.close()
    cm = _ctx(pkg, w.cells, "mixed", pot, s64)   # the FP64 trajectory's state, forces recomputed mixed
    fm, _ = cm.download()
    t = cm.thermo()
    cm.close()
    d = fm["f"][loc] - s64["f"][loc]
    assert np.sqrt((d ** 2).mean()) <= 1e-5
    assert np.abs(d).max() <= 1e-4
    assert np.abs(t["force_sum"]).max() / loc.size < 1e-7


@pytest.mark.parametrize("prec", ["mixed"])
def test_fe_100c_cascade_conserves_atoms_and_energy(pkg, wl, gpu_lib, fe_pot, prec):
    """The 5 keV cascade workload (2,000,000 atoms, 2000 variable-dt steps): every id 1..N appears once
    among lattice slots and the inter-atom list, vacancies equal inter atoms, and the total energy
    stays within 2e-4 eV/atom of its start."""
    w = wl.WORKLOADS["fe_100c_cascade"]
    cells = w.cells
    loc = wl.local_slot_indices(cells, RCF)
    c = _ctx(pkg, cells, prec, fe_pot, wl.workload_state(w), cap=32768)
    c.collision_step([cells[0] // 2, cells[1] // 2, cells[2] // 2, 0], wl.pka_direction(w.seed), w.pka_ev)
    c.set_variable_timestep(wl.CASCADE_DX_MAX, wl.CASCADE_DT_MIN, wl.CASCADE_DT_MAX)
    th0 = c.thermo(with_energy=True)
    e0 = th0["potential_energy"] + th0["kinetic_energy"] * wl.MVV2E
    c.simulate(w.steps)
    th = c.thermo(with_energy=True)
    e1 = th["potential_energy"] + th["kinetic_energy"] * wl.MVV2E
    atoms, inter = c.download()
    c.close()
    lat = atoms[loc]
    ids = np.concatenate([lat["id"][lat["type"] >= 0], inter["id"]])
    assert ids.size == w.n_atoms
    assert np.array_equal(np.sort(ids), np.arange(1, w.n_atoms + 1, dtype=np.uint64))
    assert th["n_vacancy"] == th["n_inter"] == inter.size > 0
    assert th["device_errors"] == 0
    assert abs(e1 - e0) / w.n_atoms < 2e-4
