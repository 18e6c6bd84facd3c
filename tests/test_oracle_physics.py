"""Physics invariants of the oracle (the checker must itself be right)."""
import numpy as np
import pytest

A0 = 2.855
RCF = 5.6 / A0


def test_force_is_minus_energy_gradient(orc, wl, potentials):
    cells = (6, 6, 6)
    atoms = wl.build_state(cells, A0, RCF, temperature=300.0, seed=4)
    loc = wl.local_slot_indices(cells, RCF)
    s0 = loc[37]
    s = orc.OracleSim(cells, A0, RCF, potentials["fecuni"])
    atoms["type"][loc[::7]] = 1
    atoms["type"][loc[3::11]] = 2
    s.set_atoms(atoms)
    s.prepare()
    f = s.get_atoms()["f"][s0]
    h = 1e-5
    for d in range(3):
        e = []
        for sg in (-1, 1):
            a = atoms.copy()
            a["x"][s0, d] += sg * h
            t = orc.OracleSim(cells, A0, RCF, potentials["fecuni"])
            t.set_atoms(a)
            t.prepare()
            e.append(t.potential_energy()[0])
        assert -(e[1] - e[0]) / (2 * h) == pytest.approx(f[d], abs=2e-7)


def test_sum_of_forces_and_energy_conservation(orc, wl, potentials):
    cells = (8, 8, 8)
    n = 2 * 8 * 8 * 8
    atoms = wl.build_state(cells, A0, RCF, temperature=600.0, seed=9)
    s = orc.OracleSim(cells, A0, RCF, potentials["fe"], dt=0.001)
    s.set_atoms(atoms)
    s.prepare()
    e0 = s.potential_energy()[0] + s.kinetic_energy() * wl.MVV2E
    for _ in range(4):
        s.simulate(25)
        assert np.abs(s.system_force()).max() < 1e-10
        e = s.potential_energy()[0] + s.kinetic_energy() * wl.MVV2E
        assert abs(e - e0) / n < 5e-5
    assert s.get_inter().size == 0


def test_decide_moves_displaced_atom_and_recombines(orc, wl, potentials):
    cells = (6, 6, 6)
    atoms = wl.build_state(cells, A0, RCF, temperature=0.0, seed=1)
    loc = wl.local_slot_indices(cells, RCF)
    s = orc.OracleSim(cells, A0, RCF, potentials["fe"])
    a = atoms.copy()
    a["x"][loc[100], 0] += 0.3 * A0    # beyond 0.2 a0, still in its own WS cell: leaves and returns
    a["x"][loc[200], 1] += 0.55 * A0   # across the WS face at 0.5 a0 into an occupied cell: stays inter
    s.set_atoms(a)
    s.decide()
    inter = s.get_inter()
    got = s.get_atoms()
    assert inter.size == 1 and inter["id"][0] == a["id"][loc[200]]
    assert got["type"][loc[100]] == 0 and got["type"][loc[200]] == -1
    assert (got["v"][loc[200]] == 0).all()
