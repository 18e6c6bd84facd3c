"""The stage machine (mg_run_stages) against the reference's driver logic (MDSimulation::beforeStep /
postStep, frontend/md_simulation.cpp:40-111) restated here on the oracle's step primitives."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

A0 = 2.855
RCF = 5.6 / A0


def run_stages_oracle(ref, stages, steps, default_dt, n_atoms, thermo_interval):
    cur, cur_steps, stage_len, nxt, samples = None, 0, 0, 0, []
    for step in range(steps):
        if cur_steps >= stage_len:
            cur = stages[nxt]
            nxt += 1
            stage_len = cur["steps"]
            cur_steps = 0
            ref.set_timestep(cur.get("step_length", 0.0) or default_dt)
        if "collision_step" in cur and cur_steps + 1 == cur["collision_step"]:
            ref.collision_step(cur["lat"], cur["direction"], cur["energy"])
        if "rescale_t" in cur and cur_steps % cur["rescale_every"] == 0:
            ref.rescale(cur["rescale_t"], n_atoms)
        ref.simulate(1)
        cur_steps += 1
        if thermo_interval and (step + 1) % thermo_interval == 0:
            samples.append((ref.mvv(), ref.time()))
    return samples


def test_stage_machine_matches_the_reference_driver(pkg, orc, wl, potentials, gpu_lib):
    cells = (9, 9, 9)
    n = 2 * 9 * 9 * 9
    atoms = wl.build_state(cells, A0, RCF, temperature=300.0, seed=121)
    stages = [
        {"steps": 20, "step_length": 0.0005, "rescale_t": 600.0, "rescale_every": 5},
        {"steps": 15, "collision_step": 3, "lat": [4, 4, 4, 1], "direction": [1.0, 2.0, 2.5], "energy": 150.0},
        {"steps": 12, "step_length": 0.0002},
        {"steps": 0, "step_length": 0.0003},          # a stage of 0 steps still runs one step
        {"steps": 5},
    ]
    steps = 20 + 15 + 12 + 1 + 5
    ctx = pkg.Context(cells, A0, RCF, precision="fp64")
    ctx.pot_init_setfl(potentials["fe"])
    ctx.upload(atoms)
    ctx.prepare()
    got = ctx.run_stages(stages, steps, default_dt=0.001, n_atoms=n, thermo_interval=4)
    ref = orc.OracleSim(cells, A0, RCF, potentials["fe"], dt=0.001)
    ref.set_atoms(atoms)
    ref.prepare()
    want = run_stages_oracle(ref, stages, steps, 0.001, n, 4)
    assert len(got) == len(want) == steps // 4
    for k, (g, (mvv, t)) in enumerate(zip(got, want)):
        assert g["step"] == 4 * (k + 1)
        assert g["time_ps"] == t                       # the same dt sequence, summed in the same order
        assert g["mvv"] == pytest.approx(mvv, rel=1e-10)
    a, inter = ctx.download()
    loc = wl.local_slot_indices(cells, RCF)
    w = ref.get_atoms()
    assert np.abs(a["x"][loc] - w["x"][loc]).max() < 1e-9
    assert np.array_equal(inter["id"], ref.get_inter()["id"])
    hist = ctx.dt_history()
    assert np.array_equal(hist[:20], [0.0005] * 20) and np.array_equal(hist[35:47], [0.0002] * 12)
    assert hist[47] == 0.0003 and np.array_equal(hist[48:], [0.001] * 5)
    with pytest.raises(pkg.MgError) as e:
        ctx.run_stages([{"steps": 2}], 5, default_dt=0.001, n_atoms=n)   # runs out of stages
    assert e.value.status == 6
    ctx.close()


def test_stage_machine_fused_bodies_are_bit_identical(pkg, wl, potentials, gpu_lib):
    """Mixed form: runs of 16 event-free bodies go through the fused graph (firststep inside the force
    pass); the samples and the final state equal those of one body per launch, bit for bit."""
    cells = (10, 9, 9)
    n = 2 * 10 * 9 * 9
    atoms = wl.build_state(cells, A0, RCF, temperature=300.0, seed=5)
    stages = [
        {"steps": 70, "step_length": 0.0005, "rescale_t": 600.0, "rescale_every": 35},
        {"steps": 60, "collision_step": 27, "lat": [4, 4, 4, 1], "direction": [1.0, 2.0, 2.5], "energy": 150.0},
    ]
    out = []
    for fuse in (16, 0):
        ctx = pkg.Context(cells, A0, RCF, precision="mixed", inter_capacity=1024)
        ctx.pot_init_setfl(potentials["fe"])
        ctx.set_step_fusion(fuse)
        ctx.upload(atoms)
        ctx.prepare()
        got = ctx.run_stages(stages, 130, default_dt=0.001, n_atoms=n, thermo_interval=50)
        a, inter = ctx.download()
        out.append((got, a, inter, ctx.clock()))
        ctx.close()
    (g1, a1, i1, c1), (g0, a0_, i0, c0) = out
    assert [(s["step"], s["time_ps"], s["mvv"]) for s in g1] == [(s["step"], s["time_ps"], s["mvv"]) for s in g0]
    assert a1.tobytes() == a0_.tobytes() and i1.tobytes() == i0.tobytes() and c1 == c0


def test_simulation_run_stages_with_dumps(pkg, wl, potentials, gpu_lib, tmp_path):
    """The Simulation mirror runs a staged schedule with interval frames and an origin dump."""
    sim = pkg.Simulation(precision="mixed")
    sim.create_domain((8, 8, 8), A0, RCF)
    sim.create_atoms(0.001, 300.0, 7)
    sim.prepare_for_start(potentials["fe"])
    stages = [{"steps": 40, "step_length": 0.0005},
              {"steps": 24, "collision_step": 5, "lat": [4, 4, 4, 0], "direction": [1.0, 1.0, 2.0], "energy": 100.0}]
    out = sim.run_stages(stages, 64, 0.001, thermo_interval=16, dump_path=str(tmp_path / "run.out"), dump_interval=32,
                         origin_dump_path=str(tmp_path / "origin.out"))
    assert [s["step"] for s in out] == [16, 32, 48, 64]
    frames = pkg.dumpfile.frames(str(tmp_path / "run.out"))
    assert sorted(frames) == [32, 64] and all(f.size == 2 * 8 ** 3 for f in frames.values())
    origin = pkg.dumpfile.read(str(tmp_path / "origin.out"))
    assert origin.size == 2 * 8 ** 3 and set(origin["step"].tolist()) == {44}
