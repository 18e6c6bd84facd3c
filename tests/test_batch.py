"""Batched replicas (mg_batch_*): one CUDA graph advances several independent boxes.

A batch runs exactly the kernels mg_simulate runs for each context, and no kernel's result depends
on the order in which its threads run, so a batched replica is bit-identical to the same context
stepped alone, cascades included; cascades also follow the oracle like a single context does.
"""
import numpy as np
import pytest

from test_gpu_parity import A0, RCF

pytestmark = pytest.mark.gpu

DX_MAX, DT_MIN, DT_MAX = 0.01, 1e-5, 1e-3


def _ctx(pkg, pot, cells, atoms, prec, inter_capacity=0):
    ctx = pkg.Context(cells, A0, RCF, precision=prec, inter_capacity=inter_capacity)
    ctx.pot_init_setfl(pot)
    ctx.upload(atoms)
    ctx.prepare()
    return ctx


def test_batch_bit_identical_to_single_runs(pkg, wl, potentials, gpu_lib):
    specs = [((8, 8, 8), "fp64", 81), ((9, 10, 8), "mixed", 82), ((11, 11, 11), "fp64", 83)]
    batched, alone = [], []
    for cells, prec, seed in specs:
        atoms = wl.build_state(cells, A0, RCF, temperature=600.0, seed=seed)
        batched.append(_ctx(pkg, potentials["fe"], cells, atoms, prec))
        alone.append(_ctx(pkg, potentials["fe"], cells, atoms, prec))
    batch = pkg.Batch(batched, steps_per_launch=3)
    batch.run(7)                       # two launches of 3 steps, one of 1
    for c in alone:
        c.simulate(7)
    assert batch.launches_per_step() == sum(c.launches_per_step() for c in alone)
    for (cells, _, _), a, b in zip(specs, batched, alone):
        ga, ia = a.download()
        gb, ib = b.download()
        assert ia.size == ib.size == 0
        for f in ("id", "type", "x", "v", "f"):
            assert np.array_equal(ga[f], gb[f]), (cells, f)
        assert a.clock() == b.clock()
        assert a.clock()[0] == 7
    # work issued on a member context after the batch sees the batch's result
    batched[0].simulate(2)
    alone[0].simulate(2)
    assert np.array_equal(batched[0].download()[0]["x"], alone[0].download()[0]["x"])
    batch.close()
    for c in batched + alone:
        c.close()


def test_batch_cascades_follow_the_oracle(pkg, orc, wl, potentials, gpu_lib):
    """Two cascades of different box size and PKA energy, each with its own variable timestep."""
    specs = [((10, 10, 10), 500.0, 91), ((12, 11, 10), 800.0, 92)]
    ctxs, refs = [], []
    for cells, energy, seed in specs:
        atoms = wl.build_state(cells, A0, RCF, temperature=300.0, seed=seed)
        ctx = _ctx(pkg, potentials["fe"], cells, atoms, "fp64", inter_capacity=2048)
        ref = orc.OracleSim(cells, A0, RCF, potentials["fe"], dt=0.001)
        ref.set_atoms(atoms)
        ref.prepare()
        lat = [cells[0] // 2, cells[1] // 2, cells[2] // 2, 1]
        ctx.collision_step(lat, wl.pka_direction(seed), energy)
        ref.collision_step(lat, wl.pka_direction(seed), energy)
        ctx.set_variable_timestep(DX_MAX, DT_MIN, DT_MAX)
        ref.set_variable_timestep(DX_MAX, DT_MIN, DT_MAX)
        ctxs.append(ctx)
        refs.append(ref)
    batch = pkg.Batch(ctxs, steps_per_launch=4)
    seen = [0, 0]
    for step in range(400):
        batch.run(1)
        for r, (ctx, ref) in enumerate(zip(ctxs, refs)):
            ref.simulate(1)
            _, inter = ctx.download()
            assert np.array_equal(inter["id"], ref.get_inter()["id"]), (r, step)
            seen[r] = max(seen[r], inter.size)
    for (cells, _, _), ctx, ref in zip(specs, ctxs, refs):
        got, _ = ctx.download()
        want = ref.get_atoms()
        loc = wl.local_slot_indices(cells, RCF)
        assert np.abs(got["x"][loc] - want["x"][loc]).max() < 1e-9
        assert np.allclose(ctx.dt_history(), ref.dt_history(), rtol=1e-12, atol=0)
    assert min(seen) > 0
    # the same cascades stepped alone, one context after the other: the same bits
    for (cells, energy, seed), ctx in zip(specs, ctxs):
        atoms = wl.build_state(cells, A0, RCF, temperature=300.0, seed=seed)
        one = _ctx(pkg, potentials["fe"], cells, atoms, "fp64", inter_capacity=2048)
        one.collision_step([cells[0] // 2, cells[1] // 2, cells[2] // 2, 1], wl.pka_direction(seed), energy)
        one.set_variable_timestep(DX_MAX, DT_MIN, DT_MAX)
        one.simulate(400)
        (ga, ia), (gb, ib) = ctx.download(), one.download()
        assert ga.tobytes() == gb.tobytes() and ia.tobytes() == ib.tobytes()
        assert np.array_equal(ctx.dt_history(), one.dt_history())
        one.close()
    batch.close()
    for c in ctxs:
        c.close()


def test_batch_reports_the_failing_replica(pkg, wl, potentials, gpu_lib):
    cells = (8, 8, 8)
    good = _ctx(pkg, potentials["fe"], cells, wl.build_state(cells, A0, RCF, temperature=300.0, seed=3), "fp64")
    fast = wl.build_state(cells, A0, RCF, temperature=300.0, seed=4)
    loc = wl.local_slot_indices(cells, RCF)
    fast["v"][loc[::97][:10]] = (300.0, 0.0, 0.0)   # 0.3 A per 1 fs step: ten atoms leave their cells
    bad = _ctx(pkg, potentials["fe"], cells, fast, "fp64", inter_capacity=4)
    batch = pkg.Batch([good, bad])
    with pytest.raises(pkg.MgError) as e:
        batch.run(4)
    assert e.value.status == 4 and "replica 1" in str(e.value)
    with pytest.raises(pkg.MgError):
        pkg.Batch([good, good])       # a context may appear once
    batch.close()
    good.close()
    bad.close()
