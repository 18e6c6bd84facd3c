"""Oracle parity at the benchmark workloads' own sizes (GPU).

Two workloads of BCC Fe with the synthetic single-element table, 600 K Maxwell velocities from the
workload seed, dt = 1 fs:
* 20x20x20 cells, 16,000 atoms, 100 steps (the CPU-runnable workload, run whole);
* 100x100x100 cells, 2,000,000 atoms: computeEam after the first ghost exchange, then 5 steps.
The GPU state is compared with the CPU oracle's on the same seeded input:
* indexing: the atom types and ids of every slot, the inter-atom lists and the ghost map (type and
  position of every ghost slot) bit for bit;
* FP64 form: forces within 1e-9 eV/A, rho within rel 1e-13, df within rel 1e-12;
* mixed form: force RMS <= 1e-5 eV/A and max <= 1e-4 eV/A, rho within rel 1e-6.
Trajectories are compared twice: the GPU's after n steps against the oracle's after n steps, and the
oracle restarted from the GPU's state (ghost exchange and computeEam on the GPU's positions), which
separates the code's parity from the growth of rounding differences along a trajectory.
"""
import numpy as np
import pytest

from test_gpu_parity import A0, RCF, F64_TOL, MIX_MAX, MIX_RMS

pytestmark = pytest.mark.gpu

X_TOL = 1e-9       # A, positions after n FP64 steps (summation order only)
V_TOL = 1e-7       # A/ps


def _ghosts(wl, cells):
    Sx, Sy, Sz, _, _, _ = wl.grid(cells, RCF)
    return np.setdiff1d(np.arange(Sx * Sy * Sz), wl.local_slot_indices(cells, RCF))


def _gpu(pkg, cells, prec, pot, atoms):
    c = pkg.Context(cells, A0, RCF, precision=prec)
    c.pot_init_setfl(pot)
    c.set_timestep(0.001)
    c.upload(atoms)
    c.prepare()
    return c


def _check_forces(got, want, occ, prec):
    d = got["f"][occ] - want["f"][occ]
    if prec == "fp64":
        assert np.abs(d).max() <= F64_TOL
        assert np.allclose(got["rho"][occ], want["rho"][occ], rtol=1e-13, atol=0)
        assert np.allclose(got["df"][occ], want["df"][occ], rtol=1e-12, atol=1e-15)
    else:
        assert np.sqrt((d ** 2).mean()) <= MIX_RMS
        assert np.abs(d).max() <= MIX_MAX
        assert np.allclose(got["rho"][occ], want["rho"][occ], rtol=1e-6)


def _check_restart(orc, wl, cells, pot, got, inter, prec):
    """The oracle restarted from the GPU's state: the ghost map of the GPU's positions and computeEam
    on them, against the GPU's ghost slots and forces."""
    ref = orc.OracleSim(cells, A0, RCF, pot, dt=0.001)
    ref.set_atoms(got)
    ref.set_inter(inter)
    ref.exchange_atom_first()
    want = ref.get_atoms()
    g = _ghosts(wl, cells)
    assert np.array_equal(got["type"][g], want["type"][g])
    assert np.array_equal(got["x"][g], want["x"][g])
    ref.clear_force()
    ref.compute_eam()
    want = ref.get_atoms()
    loc = wl.local_slot_indices(cells, RCF)
    _check_forces(got, want, loc[want["type"][loc] >= 0], prec)
    ref.close()


def _check_trajectory(got, inter, want, winter, loc, prec):
    for f in ("id", "type"):
        assert np.array_equal(got[f][loc], want[f][loc]), f
    assert np.array_equal(inter["id"], winter["id"])
    if prec == "fp64":
        assert np.abs(got["x"][loc] - want["x"][loc]).max() <= X_TOL
        assert np.abs(got["v"][loc] - want["v"][loc]).max() <= V_TOL
    _check_forces(got, want, loc[want["type"][loc] >= 0], prec)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_fe_20c_100_steps(pkg, orc, wl, gpu_lib, tmp_path, prec):
    """16,000 atoms, 100 steps of 1 fs, FP64 and mixed, against the oracle's 100 steps."""
    w = wl.WORKLOADS["fe_20c"]
    pot = wl.workload_potential(w, str(tmp_path))
    state = wl.workload_state(w)
    loc = wl.local_slot_indices(w.cells, RCF)
    ref = orc.OracleSim(w.cells, A0, RCF, pot, dt=0.001)
    ref.set_atoms(state)
    ref.prepare()
    c = _gpu(pkg, w.cells, prec, pot, state)
    got0, _ = c.download()
    want0 = ref.get_atoms()
    g = _ghosts(wl, w.cells)
    assert np.array_equal(got0["type"][g], want0["type"][g])
    assert np.array_equal(got0["x"][g], want0["x"][g])
    _check_forces(got0, want0, loc[want0["type"][loc] >= 0], prec)
    c.simulate(w.steps)
    ref.simulate(w.steps)
    got, inter = c.download()
    _check_trajectory(got, inter, ref.get_atoms(), ref.get_inter(), loc, prec)
    t = c.thermo()
    assert t["device_errors"] == 0
    if prec == "fp64":
        assert t["mvv"] == pytest.approx(ref.mvv(), rel=1e-12)
    else:
        assert t["mvv"] == pytest.approx(ref.mvv(), rel=1e-7)
    _check_restart(orc, wl, w.cells, pot, got, inter, prec)
    c.close()
    ref.close()


@pytest.fixture(scope="module")
def fe_100c_oracle(orc, wl, tmp_path_factory):
    """The oracle's 2,000,000-atom Fe state after prepareForStart, and after 5 more steps."""
    w = wl.WORKLOADS["fe_100c"]
    pot = wl.workload_potential(w, str(tmp_path_factory.mktemp("fe100parity")))
    state = wl.workload_state(w)
    ref = orc.OracleSim(w.cells, A0, RCF, pot, dt=0.001)
    ref.set_atoms(state)
    ref.prepare()
    at_prepare = ref.get_atoms()
    ref.simulate(5)
    after5, inter5 = ref.get_atoms(), ref.get_inter()
    ref.close()
    return w, pot, state, at_prepare, after5, inter5


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_fe_100c_prepare_and_5_steps(pkg, orc, wl, gpu_lib, fe_100c_oracle, prec):
    """2,000,000 atoms: rho, df and forces after the first computeEam and the ghost map bit for bit;
    then 5 steps against the oracle's 5 steps, and the oracle restarted from the GPU's state."""
    w, pot, state, at_prepare, after5, inter5 = fe_100c_oracle
    loc = wl.local_slot_indices(w.cells, RCF)
    c = _gpu(pkg, w.cells, prec, pot, state)
    got0, _ = c.download()
    g = _ghosts(wl, w.cells)
    assert np.array_equal(got0["type"], at_prepare["type"])
    assert np.array_equal(got0["id"][loc], at_prepare["id"][loc])
    assert np.array_equal(got0["x"][g], at_prepare["x"][g])
    assert np.array_equal(got0["x"][loc], at_prepare["x"][loc])
    _check_forces(got0, at_prepare, loc[at_prepare["type"][loc] >= 0], prec)
    del got0
    c.simulate(5)
    got, inter = c.download()
    assert c.thermo()["device_errors"] == 0
    c.close()
    _check_trajectory(got, inter, after5, inter5, loc, prec)
    _check_restart(orc, wl, w.cells, pot, got, inter, prec)
