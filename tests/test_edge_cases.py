"""Edge cases of the state: the smallest box the ghost width allows, an empty box, a lone atom and a
dimer, through the C ABI against the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

A0 = 2.855
RCF = 5.6 / A0


def _pair(pkg, orc, pot, cells, atoms, precision):
    ctx = pkg.Context(cells, A0, RCF, precision=precision)
    ctx.pot_init_setfl(pot)
    ctx.set_timestep(0.001)
    ctx.upload(atoms)
    ref = orc.OracleSim(cells, A0, RCF, pot, dt=0.001)
    ref.set_atoms(atoms)
    return ctx, ref


def _emptied(wl, cells, keep=()):
    """A crystal with every local atom removed except the local indices in keep."""
    atoms = wl.build_state(cells, A0, RCF, temperature=0.0, seed=1)
    loc = wl.local_slot_indices(cells, RCF)
    mask = np.ones(loc.size, dtype=bool)
    mask[list(keep)] = False
    atoms["type"][loc[mask]] = -1
    return atoms


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_smallest_box_steps_match_oracle(pkg, orc, wl, potentials, gpu_lib, precision):
    cells = (6, 6, 6)  # twice the ghost width in every dimension
    atoms = wl.build_state(cells, A0, RCF, temperature=600.0, seed=44, cu_frac=0.05, ni_frac=0.05)
    ctx, ref = _pair(pkg, orc, potentials["fecuni"], cells, atoms, precision)
    ctx.prepare()
    ref.prepare()
    ctx.simulate(20, sync=True)
    ref.simulate(20)
    a, inter = ctx.download()
    w = ref.get_atoms()
    loc = wl.local_slot_indices(cells, RCF)
    assert np.array_equal(a["type"][loc], w["type"][loc]) and inter.size == ref.get_inter().size
    tol = 1e-9 if precision == "fp64" else 1e-5
    assert np.abs(a["x"][loc] - w["x"][loc]).max() < tol
    assert np.abs(a["f"][loc] - w["f"][loc]).max() < (1e-8 if precision == "fp64" else 1e-4)
    ctx.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_empty_box(pkg, orc, wl, potentials, gpu_lib, precision):
    cells = (7, 6, 8)
    atoms = _emptied(wl, cells)
    ctx, _ = _pair(pkg, orc, potentials["fe"], cells, atoms, precision)
    ctx.prepare()
    ctx.simulate(5, sync=True)
    th = ctx.thermo(with_energy=True)
    assert th["mvv"] == 0.0 and th["n_inter"] == 0 and th["device_errors"] == 0
    a, inter = ctx.download()
    loc = wl.local_slot_indices(cells, RCF)
    assert np.all(a["type"][loc] == -1) and inter.size == 0
    assert np.all(a["f"][loc] == 0.0)
    host = a.copy()
    n = ctx.step_host(host, np.zeros(4, dtype=pkg.ATOM_DTYPE), 0, 1)  # the pipelined host step as well
    assert n == 0 and np.all(host["type"][loc] == -1)
    ctx.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_lone_atom_and_dimer(pkg, orc, wl, potentials, gpu_lib, precision):
    cells = (8, 8, 8)
    loc_keep = (500,)
    ctx, ref = _pair(pkg, orc, potentials["fe"], cells, _emptied(wl, cells, loc_keep), precision)
    ctx.prepare()
    a, _ = ctx.download()
    loc = wl.local_slot_indices(cells, RCF)
    assert np.all(a["f"][loc[500]] == 0.0) and a["rho"][loc[500]] == 0.0
    ctx.close()
    # a dimer of nearest neighbours (corner site and the body centre next to it)
    atoms = wl.build_state(cells, A0, RCF, temperature=0.0, seed=1)
    d = np.linalg.norm(atoms["x"][loc] - atoms["x"][loc[500]], axis=1)
    nn = int(np.argsort(d)[1])
    ctx, ref = _pair(pkg, orc, potentials["fe"], cells, _emptied(wl, cells, (500, nn)), precision)
    ctx.prepare()
    ref.prepare()
    a, _ = ctx.download()
    w = ref.get_atoms()
    f1, f2 = a["f"][loc[500]], a["f"][loc[nn]]
    assert np.abs(f1 + f2).max() < (1e-12 if precision == "fp64" else 1e-6)      # Newton's third law
    assert np.abs(f1 - w["f"][loc[500]]).max() < (1e-9 if precision == "fp64" else 1e-5)
    assert np.linalg.norm(f1) > 1e-3
    ctx.close()
