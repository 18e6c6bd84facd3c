"""Atom dumps (frontend/io/atom_dump.cpp, output_copy.cpp; the layout tools/dump2text/out_convert.cpp
reads): the oracle's record builder and file layout on the CPU, and the device-fed writer through the C
ABI against the oracle on the same states, bit for bit."""
import os

import numpy as np
import pytest

A0 = 2.855
RCF = 5.6 / A0


def _cascade_oracle(orc, wl, pot, cells=(8, 8, 8), steps=60):
    """An oracle state with inter atoms and vacancies: a 300 eV recoil in a small Fe box."""
    atoms = wl.build_state(cells, A0, RCF, temperature=300.0, seed=17)
    ref = orc.OracleSim(cells, A0, RCF, pot, dt=0.0002)
    ref.set_atoms(atoms)
    ref.prepare()
    ref.collision_step([4, 4, 4, 0], [1.0, 0.7, 0.3], 300.0)
    ref.simulate(steps)
    return ref


def _records_py(atoms, inter, cells, step):
    """The dump order written out in Python: inter atoms, then the sub-box in k, j, i order."""
    Sx, Sy, Sz, gx, gy, gz = (int(v) for v in (*_grid(cells),))
    recs = []
    for a in inter:
        recs.append((int(a["id"]), int(a["type"]), tuple(a["x"]), tuple(a["v"])))
    for k in range(gz, gz + cells[2]):
        for j in range(gy, gy + cells[1]):
            for i in range(gx, gx + 2 * cells[0]):
                a = atoms[(k * Sy + j) * Sx + i]
                if a["type"] != -1:
                    recs.append((int(a["id"]), int(a["type"]), tuple(a["x"]), tuple(a["v"])))
    return recs


def _grid(cells):
    g = 3  # ceil(rc / a0) + 1 for rc = 5.6, a0 = 2.855
    return 2 * (cells[0] + 2 * g), cells[1] + 2 * g, cells[2] + 2 * g, 2 * g, g, g


def test_oracle_records_follow_the_reference_order(orc, wl, potentials):
    ref = _cascade_oracle(orc, wl, potentials["fe"])
    inter = ref.get_inter()
    assert inter.size > 0, "the recoil must leave inter atoms"
    got = ref.dump_records(42)
    want = _records_py(ref.get_atoms(), inter, (8, 8, 8), 42)
    assert got.size == len(want) == 2 * 8 ** 3 - np.count_nonzero(ref.get_atoms()["type"][wl.local_slot_indices((8, 8, 8), RCF)] < 0) + inter.size
    for r, (i, t, x, v) in zip(got, want):
        assert (int(r["id"]), int(r["type"]), tuple(r["x"]), tuple(r["v"])) == (i, t, x, v)
    assert np.all(got["step"] == 42) and np.all(got["inter_type"] == 0)


def test_file_layout_round_trip(orc, pkg, tmp_path):
    """The oracle's one-rank file read back by the oracle's dump2text reader and by the package's reader."""
    rng = np.random.default_rng(3)
    recs = np.zeros(2500, dtype=orc.DUMP_DTYPE)      # more than two 1024-record blocks
    recs["id"] = rng.permutation(2500) + 1
    recs["step"] = 7
    recs["type"] = rng.integers(0, 3, 2500)
    recs["x"] = rng.normal(size=(2500, 3))
    recs["v"] = rng.normal(size=(2500, 3))
    p = str(tmp_path / "f.out")
    orc.write_dump_file(p, recs)
    assert os.path.getsize(p) == 256 + 72 * 2500
    (back,) = orc.read_dump_file(p)
    assert back.tobytes() == recs.tobytes()
    assert pkg.dumpfile.read(p).tobytes() == recs.tobytes()
    assert pkg.dumpfile.RECORD_DTYPE == orc.DUMP_DTYPE


def test_dump2text_reader_walks_interleaved_blocks(orc, tmp_path):
    """Two ranks: LocalStorage interleaves their 1024-record blocks; the reader follows rank r's blocks."""
    rng = np.random.default_rng(5)
    n = [1500, 700]
    recs = []
    for r in range(2):
        a = np.zeros(n[r], dtype=orc.DUMP_DTYPE)
        a["id"] = np.arange(n[r]) + 1 + 10000 * r
        a["x"] = rng.normal(size=(n[r], 3))
        recs.append(a)
    blk = orc.DUMP_BLOCK
    body = bytearray(blk * 4)
    for r in range(2):
        raw = recs[r].tobytes()
        for k in range((len(raw) + blk - 1) // blk):
            part = raw[k * blk:(k + 1) * blk]
            at = (2 * k + r) * blk
            body[at:at + len(part)] = part
    head = bytearray(128 + 2 * 128)
    for r in range(2):
        head[128 + 128 * r:128 + 128 * r + 8] = np.uint64(n[r]).tobytes()
    p = tmp_path / "two.out"
    p.write_bytes(bytes(head) + bytes(body))
    back = orc.read_dump_file(str(p), n_ranks=2)
    for r in range(2):
        assert back[r].tobytes() == recs[r].tobytes()


# ---------------------------------------------------------------------------------------------- GPU
def _gpu_cascade(pkg, wl, pot, precision="fp64", cells=(8, 8, 8), steps=60):
    atoms = wl.build_state(cells, A0, RCF, temperature=300.0, seed=17)
    ctx = pkg.Context(cells, A0, RCF, precision=precision, inter_capacity=4096)
    ctx.pot_init_setfl(pot)
    ctx.upload(atoms)
    ctx.set_timestep(0.0002)
    ctx.prepare()
    ctx.collision_step([4, 4, 4, 0], [1.0, 0.7, 0.3], 300.0)
    ctx.simulate(steps, sync=True)
    return ctx


def _oracle_of(orc, ctx, pot, cells):
    a, inter = ctx.download()
    ref = orc.OracleSim(cells, A0, RCF, pot, dt=0.0002)
    ref.set_atoms(a)
    ref.set_inter(inter)
    return ref


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gpu_dump_matches_oracle_records(pkg, orc, wl, potentials, gpu_lib, tmp_path, precision):
    cells = (8, 8, 8)
    ctx = _gpu_cascade(pkg, wl, potentials["fe"], precision)
    p = str(tmp_path / "d.out")
    d = ctx.dump_open(p)
    d.frame(61)
    n = d.close()
    want = _oracle_of(orc, ctx, potentials["fe"], cells).dump_records(61)
    assert ctx.thermo()["n_inter"] > 0
    (got,) = orc.read_dump_file(p)
    assert n == want.size == got.size
    assert got.tobytes() == want.tobytes()
    ctx.close()


@pytest.mark.gpu
def test_gpu_dump_frames_chunked_and_by_frame(pkg, orc, wl, potentials, gpu_lib, tmp_path):
    """Frames appended to one file through chunks smaller than a frame (odd size), and one file per
    frame; every frame equals the oracle's records of the state it was taken from."""
    cells = (8, 8, 8)
    ctx = _gpu_cascade(pkg, wl, potentials["fe"], cells=cells, steps=20)
    single = ctx.dump_open(str(tmp_path / "all.out"), chunk_bytes=72 * 100 + 8)
    per = ctx.dump_open(str(tmp_path / "f_{}.out"), by_frame=True, chunk_bytes=4096)
    want = []
    for k, step in enumerate((100, 200, 300)):
        single.frame(step)
        per.frame(step)
        want.append(_oracle_of(orc, ctx, potentials["fe"], cells).dump_records(step))
        ctx.simulate(25, sync=False)
    n_single = single.close()
    n_per = per.close()
    total = sum(w.size for w in want)
    assert n_single == n_per == total
    (all_recs,) = orc.read_dump_file(str(tmp_path / "all.out"))
    assert all_recs.tobytes() == b"".join(w.tobytes() for w in want)
    for w, step in zip(want, (100, 200, 300)):
        (got,) = orc.read_dump_file(str(tmp_path / f"f_{step}.out"))
        assert got.tobytes() == w.tobytes()
    fr = pkg.dumpfile.frames(str(tmp_path / "all.out"))
    assert sorted(fr) == [100, 200, 300]
    with pytest.raises(pkg.MgError):
        ctx.dump_open(str(tmp_path / "no_placeholder.out"), by_frame=True)
    ctx.close()


@pytest.mark.gpu
def test_gpu_stage_machine_dumps(pkg, orc, wl, potentials, gpu_lib, tmp_path):
    """run_stages writes a frame after every interval-th step and the pre-collision state to the origin
    file (MDSimulation::beforeStep / postStep); the frames follow the oracle's driver to 1e-9."""
    cells = (9, 9, 9)
    n = 2 * 9 * 9 * 9
    atoms = wl.build_state(cells, A0, RCF, temperature=300.0, seed=121)
    stages = [
        {"steps": 10, "step_length": 0.0005},
        {"steps": 14, "collision_step": 4, "lat": [4, 4, 4, 1], "direction": [1.0, 2.0, 2.5], "energy": 150.0},
    ]
    ctx = pkg.Context(cells, A0, RCF, precision="fp64")
    ctx.pot_init_setfl(potentials["fe"])
    ctx.upload(atoms)
    ctx.prepare()
    frames = ctx.dump_open(str(tmp_path / "run.out"))
    origin = str(tmp_path / "origin.out")
    ctx.set_stage_output(frames, 6, origin)
    ctx.run_stages(stages, 24, default_dt=0.001, n_atoms=n)
    frames.close()
    got = pkg.dumpfile.frames(str(tmp_path / "run.out"))
    assert sorted(got) == [6, 12, 18, 24]
    (orig,) = orc.read_dump_file(origin)
    # the second stage starts at step 10; its 4th step (0-based step 13) runs the collision
    assert np.all(orig["step"] == 13)

    # the oracle driving the same schedule and taking the same dumps
    ref = orc.OracleSim(cells, A0, RCF, potentials["fe"], dt=0.001)
    ref.set_atoms(atoms)
    ref.prepare()
    want, want_origin = {}, None
    for step in range(24):
        if step == 0:
            ref.set_timestep(0.0005)
        if step == 10:
            ref.set_timestep(0.001)
        if step == 13:
            want_origin = ref.dump_records(13)
            ref.collision_step([4, 4, 4, 1], [1.0, 2.0, 2.5], 150.0)
        ref.simulate(1)
        if (step + 1) % 6 == 0:
            want[step + 1] = ref.dump_records(step + 1)
    for a, b in [(orig, want_origin)] + [(got[s], want[s]) for s in (6, 12, 18, 24)]:
        assert a.size == b.size
        assert np.array_equal(a["id"], b["id"]) and np.array_equal(a["type"], b["type"])
        assert np.array_equal(a["step"], b["step"])
        assert np.abs(a["x"] - b["x"]).max() < 1e-9 and np.abs(a["v"] - b["v"]).max() < 1e-7
    ctx.set_stage_output()
    ctx.close()


@pytest.mark.gpu
def test_gpu_dump_reports_io_errors(pkg, wl, potentials, gpu_lib, tmp_path):
    """An unwritable single-file path fails at open; an unwritable by-frame path fails in the writer
    thread, and the failure comes back from the next frame or from close."""
    cells = (8, 8, 8)
    ctx = pkg.Context(cells, A0, RCF, precision="fp64")
    ctx.pot_init_setfl(potentials["fe"])
    ctx.upload(wl.build_state(cells, A0, RCF, temperature=300.0, seed=3))
    missing = tmp_path / "no_such_dir"
    with pytest.raises(pkg.MgError):
        ctx.dump_open(str(missing / "d.out"))
    d = ctx.dump_open(str(missing / "f_{}.out"), by_frame=True)
    d.frame(1)
    try:
        d.frame(2)  # fails only if the writer has already met frame 1's error
    except pkg.MgError:
        pass
    with pytest.raises(pkg.MgError, match="cannot write"):
        d.close()
    # the context stays usable
    ok = ctx.dump_open(str(tmp_path / "ok.out"))
    ok.frame(4)
    assert ok.close() == 2 * 8 ** 3
    ctx.close()
