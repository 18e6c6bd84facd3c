"""Displacement cascades with the variable timestep: the oracle's rule on the CPU, and the GPU against
the oracle through the C ABI.

The timestep rule is an extension (the reference sets dt per stage, frontend/md_simulation.cpp:42-58):
before each step dt = clamp(dx_max / max|v|, dt_min, dt_max), with |v|^2 = (vx^2 + vy^2) + vz^2 over
local lattice and local inter atoms, each operation correctly rounded, so both sides get the same dt
from the same velocities.

Cascade trajectories are chaotic: FP64 forces summed in a different order (1e-15 apart) lead to
different trajectories after a few hundred steps. The long test therefore restarts the oracle from
the GPU's state before every step and compares that one step: dt, the Verlet drift, decide,
exchangeInter and borderInter must then agree bit for bit at every step of the cascade.
"""
import numpy as np
import pytest

A0 = 2.855
RCF = 5.6 / A0
DX_MAX, DT_MIN, DT_MAX = 0.01, 1e-5, 1e-3   # Angstrom, ps: at most 0.01 A per step, 0.01 - 1 fs


def _speed2_max(atoms, loc, inter):
    """max over local lattice and inter atoms of (vx^2 + vy^2) + vz^2 (numpy rounds each operation)."""
    vals = []
    for rec in (atoms[loc], inter):
        rec = rec[rec["type"] >= 0]
        if rec.size:
            v = rec["v"]
            vals.append(((v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + v[:, 2] * v[:, 2]).max())
    return max(vals) if vals else 0.0


def _rule(v2):
    dt = DX_MAX / np.sqrt(v2) if v2 > 0 else DT_MAX
    return min(max(dt, DT_MIN), DT_MAX)


def test_oracle_variable_timestep_rule(orc, wl, potentials):
    """CPU: the oracle's dt of every step follows the rule from the state at the start of that step."""
    cells = (8, 8, 8)
    atoms = wl.build_state(cells, A0, RCF, temperature=300.0, seed=61)
    ref = orc.OracleSim(cells, A0, RCF, potentials["fe"], dt=0.001)
    ref.set_atoms(atoms)
    ref.prepare()
    ref.collision_step([4, 4, 4, 0], wl.pka_direction(61), 200.0)
    ref.set_variable_timestep(DX_MAX, DT_MIN, DT_MAX)
    loc = wl.local_slot_indices(cells, RCF)
    want = []
    for _ in range(12):
        want.append(_rule(_speed2_max(ref.get_atoms(), loc, ref.get_inter())))
        ref.simulate(1)
    got = ref.dt_history()
    assert np.array_equal(got, np.array(want))
    assert got[0] < DT_MAX                      # the PKA's speed sets the first steps
    assert ref.time() == sum(got.tolist())


@pytest.mark.gpu
def test_variable_timestep_clock_and_history(pkg, orc, wl, potentials, gpu_lib):
    cells = (8, 8, 8)
    atoms = wl.build_state(cells, A0, RCF, temperature=600.0, seed=62)
    ctx = pkg.Context(cells, A0, RCF, precision="fp64")
    ctx.pot_init_setfl(potentials["fe"])
    ctx.upload(atoms)
    ctx.prepare()
    ctx.set_timestep(0.0005)
    ctx.simulate(3)
    steps, t, dt = ctx.clock()
    assert steps == 3 and dt == 0.0005 and t == 0.0005 + 0.0005 + 0.0005
    ctx.collision_step([4, 4, 4, 1], wl.pka_direction(62), 300.0)
    ctx.set_variable_timestep(DX_MAX, DT_MIN, DT_MAX)
    loc = wl.local_slot_indices(cells, RCF)
    want = []
    for _ in range(6):
        got_atoms, inter = ctx.download()
        want.append(_rule(_speed2_max(got_atoms, loc, inter)))
        ctx.simulate(1)
    hist = ctx.dt_history()
    assert hist.size == 9
    assert np.array_equal(hist[:3], [0.0005] * 3)
    assert np.array_equal(hist[3:], want)       # device max-reduction + rule, bit for bit
    steps, t, dt = ctx.clock()
    acc = 0.0
    for h in hist:
        acc += h
    assert steps == 9 and t == acc and dt == hist[-1]
    with pytest.raises(pkg.MgError):
        ctx.set_variable_timestep(0.01, 1e-3, 1e-5)   # dt_min > dt_max
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_variable_timestep_after_fixed_steps(pkg, wl, potentials, gpu_lib, prec):
    """Fixed-dt kicks leave the max-|v| words alone; switching the variable rule on (with no other call
    in between) must still give the rule applied to the current velocities, bit for bit. The mixed
    form runs the 20 fixed steps as a fused graph of 16 bodies and 4 single bodies."""
    cells = (8, 8, 8)
    atoms = wl.build_state(cells, A0, RCF, temperature=900.0, seed=63)
    ctx = pkg.Context(cells, A0, RCF, precision=prec)
    ctx.pot_init_setfl(potentials["fe"])
    ctx.upload(atoms)
    ctx.prepare()
    ctx.set_timestep(0.001)
    ctx.simulate(20)
    ctx.set_variable_timestep(DX_MAX, DT_MIN, DT_MAX)
    loc = wl.local_slot_indices(cells, RCF)
    want = []
    for _ in range(4):
        got_atoms, inter = ctx.download()
        want.append(_rule(_speed2_max(got_atoms, loc, inter)))
        ctx.simulate(1)
    hist = ctx.dt_history()
    assert np.array_equal(hist[:20], [0.001] * 20)
    assert np.array_equal(hist[20:], want)
    ctx.close()


def _cascade_pair(pkg, orc, wl, pot, cells, seed, energy, precision):
    atoms = wl.build_state(cells, A0, RCF, temperature=300.0, seed=seed)
    ctx = pkg.Context(cells, A0, RCF, precision=precision, inter_capacity=4096)
    ctx.pot_init_setfl(pot)
    ctx.upload(atoms)
    ctx.prepare()
    lat = [cells[0] // 2, cells[1] // 2, cells[2] // 2, 0]
    ctx.collision_step(lat, wl.pka_direction(seed), energy)
    ctx.set_variable_timestep(DX_MAX, DT_MIN, DT_MAX)
    ref = orc.OracleSim(cells, A0, RCF, pot, dt=0.001)
    ref.set_variable_timestep(DX_MAX, DT_MIN, DT_MAX)
    return ctx, ref


@pytest.mark.gpu
@pytest.mark.parametrize("prec,steps", [("fp64", 2000), ("mixed", 2000)])
def test_cascade_migration_stepwise_bit_exact(pkg, orc, wl, potentials, gpu_lib, prec, steps):
    """A 400 eV cascade in a 12^3-cell box with the variable timestep. Before every step the oracle
    takes the GPU's state; after the step, dt, positions, slot ids and types and the inter-atom list
    (membership, order, positions) must be identical, velocities and forces within the force
    tolerance of the precision."""
    cells = (12, 12, 12)
    ctx, ref = _cascade_pair(pkg, orc, wl, potentials["fe"], cells, seed=71, energy=400.0, precision=prec)
    loc = wl.local_slot_indices(cells, RCF)
    f_abs, f_rel = (1e-9, 1e-12) if prec == "fp64" else (2e-4, 1e-5)
    n_inter_seen, migrations, last_ids = [], 0, None
    state, inter = ctx.download()
    ref.set_atoms(state)
    ref.exchange_atom_first()     # the ghost send/receive lists every later exchangeAtom reuses
    for step in range(steps):
        state, inter = ctx.download()
        ref.set_atoms(state)
        ref.set_inter(inter)
        ctx.simulate(1)
        ref.simulate(1)
        got, gi = ctx.download()
        want, wi = ref.get_atoms(), ref.get_inter()
        assert ctx.clock()[2] == ref.dt_history()[-1], step
        assert np.array_equal(got["id"][loc], want["id"][loc]), step
        assert np.array_equal(got["type"][loc], want["type"][loc]), step
        assert np.array_equal(got["x"][loc], want["x"][loc]), step
        assert np.array_equal(gi["id"], wi["id"]), step
        assert np.array_equal(gi["x"], wi["x"]), step
        for a, b in ((got["f"][loc], want["f"][loc]), (gi["f"], wi["f"])):
            if a.size:
                assert (np.abs(a - b) <= f_abs + f_rel * np.abs(b)).all(), step
        c = 0.5 * ref.dt_history()[-1] * (1.0 / 1.0364269e-4) / 55.845   # dt / (2m), Fe
        dv_tol = 4 * c * (f_abs + f_rel * np.abs(want["f"][loc]).max()) + 1e-12
        assert np.abs(got["v"][loc] - want["v"][loc]).max() <= dv_tol, step
        n_inter_seen.append(gi.size)
        if last_ids is not None and not np.array_equal(last_ids, gi["id"]):
            migrations += 1
        last_ids = gi["id"].copy()
    hist = ctx.dt_history()
    assert hist.size == steps and hist[0] < DT_MAX and hist.min() >= DT_MIN
    assert max(n_inter_seen) >= 5 and migrations >= 10   # the list grew and changed many times
    ctx.close()
