"""mg_step_host: the pipelined path (slot array moved in z-slabs, copies overlapped with firststep and
the force pass) against the unpipelined path (mg_upload + mg_simulate + mg_download), bit for bit, and
against the CPU oracle. Covers both precisions, several chained calls, slab counts that do not divide
the box, and a step whose decide moves an atom off the lattice (the pipeline's fallback download)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

A0 = 2.855
RCF = 5.6 / A0


def _ctx(pkg, cells, pot, precision, chunks):
    c = pkg.Context(cells, A0, RCF, precision=precision, inter_capacity=1024)
    c.pot_init_setfl(pot)
    c.set_timestep(0.001)
    c.set_host_pipeline(chunks)
    return c


def _prepared_state(pkg, wl, cells, pot, precision, alloy=True):
    """A state whose forces come from a computeEam (as the reference host state does after a step)."""
    c = _ctx(pkg, cells, pot, precision, 0)
    c.upload(wl.build_state(cells, A0, RCF, temperature=600.0, seed=9, cu_frac=0.05 if alloy else 0.0,
                            ni_frac=0.03 if alloy else 0.0))
    c.prepare()
    a, inter = c.download()
    c.close()
    return a, inter


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("cells,chunks", [((11, 9, 13), 2), ((11, 9, 13), 5), ((11, 9, 13), 8), ((8, 10, 37), 8),
                                          ((8, 10, 37), 16), ((6, 6, 64), 8)])
def test_pipelined_step_host_is_bit_identical(pkg, wl, potentials, gpu_lib, precision, cells, chunks):
    """(11, 9, 13): 2 slabs (density unsplit) and 3 slabs; (8, 10, 37): 8 and 9 slabs of 4-5 planes;
    (6, 6, 64): thin first slabs and a thin last copy-in chunk."""
    a0, _ = _prepared_state(pkg, wl, cells, potentials["fecuni"], precision)
    got, want = a0.copy(), a0.copy()
    cp = _ctx(pkg, cells, potentials["fecuni"], precision, chunks)
    cu = _ctx(pkg, cells, potentials["fecuni"], precision, 0)
    inter_p = np.zeros(64, dtype=pkg.ATOM_DTYPE)
    inter_u = np.zeros(64, dtype=pkg.ATOM_DTYPE)
    np_, nu = 0, 0
    for _ in range(4):
        np_ = cp.step_host(got, inter_p, np_, 1)
        nu = cu.step_host(want, inter_u, nu, 1)
        assert np_ == nu == 0
        assert got.tobytes() == want.tobytes()
    cp.close()
    cu.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_pipelined_step_host_falls_back_when_decide_moves_atoms(pkg, wl, potentials, gpu_lib, precision):
    """An atom moved 0.3 a0 along (1, 1, 1), so that its nearest site is an occupied neighbour's,
    becomes an inter atom in the step's decide and stays one (an atom nearest its own vacated site
    would recombine into it at once). The pipeline then downloads the whole state again, and the
    result still equals the unpipelined path."""
    cells = (10, 10, 10)
    a0, _ = _prepared_state(pkg, wl, cells, potentials["fecuni"], precision)
    loc = wl.local_slot_indices(cells, RCF)
    a0["x"][loc[1234]] += 0.3 * A0 * np.ones(3)
    got, want = a0.copy(), a0.copy()
    cp = _ctx(pkg, cells, potentials["fecuni"], precision, 8)
    cu = _ctx(pkg, cells, potentials["fecuni"], precision, 0)
    inter_p = np.zeros(64, dtype=pkg.ATOM_DTYPE)
    inter_u = np.zeros(64, dtype=pkg.ATOM_DTYPE)
    np_ = cp.step_host(got, inter_p, 0, 1)
    nu = cu.step_host(want, inter_u, 0, 1)
    assert np_ == nu == 1
    assert got.tobytes() == want.tobytes()
    assert inter_p[:1].tobytes() == inter_u[:1].tobytes()
    assert got["type"][loc[1234]] == -1
    # the next call has an inter atom in, so it takes the unpipelined path on both contexts
    np_ = cp.step_host(got, inter_p, np_, 1)
    nu = cu.step_host(want, inter_u, nu, 1)
    assert np_ == nu and got.tobytes() == want.tobytes()
    cp.close()
    cu.close()


def _push(a, wl, cells, picks, d):
    loc = wl.local_slot_indices(cells, RCF)
    for k in picks:
        a["x"][loc[k]] += A0 * np.asarray(d, dtype=float)


def _plane_picks(cells, planes, per_plane=3):
    """Local indices (k, j, i order) of a few atoms in each of the given local z planes."""
    nxy = 2 * cells[0] * cells[1]
    rng = np.random.default_rng(5)
    return [p * nxy + int(q) for p in planes for q in rng.choice(nxy, size=per_plane, replace=False)]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_overlapped_step_host_with_own_site_displacements(pkg, wl, potentials, gpu_lib, precision):
    """The overlapped path (40 planes, 8 density slabs): atoms pushed 0.26 a0 along x leave their
    sites but stay nearest them, so each step's decide puts them into the list and straight back.
    They sit in the planes at both z seams, at chunk edges and in the middle; four calls against the
    unpipelined path, bit for bit, with no inter atom left."""
    cells = (8, 8, 40)
    a0, _ = _prepared_state(pkg, wl, cells, potentials["fecuni"], precision)
    _push(a0, wl, cells, _plane_picks(cells, (0, 1, 2, 4, 5, 13, 20, 21, 34, 36, 37, 38, 39)), (0.26, 0.0, 0.0))
    got, want = a0.copy(), a0.copy()
    cp = _ctx(pkg, cells, potentials["fecuni"], precision, 8)
    cu = _ctx(pkg, cells, potentials["fecuni"], precision, 0)
    inter_p = np.zeros(64, dtype=pkg.ATOM_DTYPE)
    inter_u = np.zeros(64, dtype=pkg.ATOM_DTYPE)
    np_, nu = 0, 0
    for _ in range(4):
        np_ = cp.step_host(got, inter_p, np_, 1)
        nu = cu.step_host(want, inter_u, nu, 1)
        assert np_ == nu == 0
        assert got.tobytes() == want.tobytes()
    cp.close()
    cu.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("plane", [2, 19, 39])
def test_overlapped_step_host_reruns_when_decide_keeps_an_atom(pkg, wl, potentials, gpu_lib, precision, plane):
    """The overlapped path with one atom pushed 0.3 a0 along (1, 1, 1), nearest an occupied neighbour's
    site, beside own-site displacements: the chunk's decide voids the overlapped step, which runs
    again in full from its input. The result, the inter atom included, equals the unpipelined path."""
    cells = (8, 8, 40)
    a0, _ = _prepared_state(pkg, wl, cells, potentials["fecuni"], precision)
    _push(a0, wl, cells, _plane_picks(cells, (1, 20, 38), per_plane=2), (-0.26, 0.0, 0.0))
    nxy = 2 * cells[0] * cells[1]
    _push(a0, wl, cells, [plane * nxy + 77], (0.3, 0.3, 0.3))
    got, want = a0.copy(), a0.copy()
    cp = _ctx(pkg, cells, potentials["fecuni"], precision, 8)
    cu = _ctx(pkg, cells, potentials["fecuni"], precision, 0)
    inter_p = np.zeros(64, dtype=pkg.ATOM_DTYPE)
    inter_u = np.zeros(64, dtype=pkg.ATOM_DTYPE)
    np_ = cp.step_host(got, inter_p, 0, 1)
    nu = cu.step_host(want, inter_u, 0, 1)
    assert np_ == nu == 1
    assert got.tobytes() == want.tobytes()
    assert inter_p[:1].tobytes() == inter_u[:1].tobytes()
    np_ = cp.step_host(got, inter_p, np_, 1)
    nu = cu.step_host(want, inter_u, nu, 1)
    assert np_ == nu and got.tobytes() == want.tobytes()
    cp.close()
    cu.close()


def test_overlapped_step_host_matches_oracle(pkg, orc, wl, potentials, gpu_lib):
    """Three overlapped FP64 calls (32 planes, 8 density slabs) against three oracle loop bodies."""
    cells = (8, 8, 32)
    a0, _ = _prepared_state(pkg, wl, cells, potentials["fe"], "fp64", alloy=False)
    _push(a0, wl, cells, _plane_picks(cells, (0, 15, 31), per_plane=2), (0.0, 0.26, 0.0))
    got = a0.copy()
    cp = _ctx(pkg, cells, potentials["fe"], "fp64", 8)
    inter = np.zeros(16, dtype=pkg.ATOM_DTYPE)
    n = 0
    for _ in range(3):
        n = cp.step_host(got, inter, n, 1)
    ref = orc.OracleSim(cells, A0, RCF, potentials["fe"], dt=0.001)
    ref.set_atoms(a0)
    ref.exchange_atom_first()
    ref.simulate(3)
    w = ref.get_atoms()
    loc = wl.local_slot_indices(cells, RCF)
    assert n == ref.get_inter().size == 0
    assert np.array_equal(got["type"][loc], w["type"][loc]) and np.array_equal(got["id"][loc], w["id"][loc])
    assert np.abs(got["x"][loc] - w["x"][loc]).max() < 1e-12
    assert np.abs(got["f"][loc] - w["f"][loc]).max() < 1e-9
    cp.close()


def test_pipelined_step_host_matches_oracle(pkg, orc, wl, potentials, gpu_lib):
    """Three pipelined FP64 calls against three oracle loop bodies from the same host state."""
    cells = (9, 9, 9)
    a0, _ = _prepared_state(pkg, wl, cells, potentials["fe"], "fp64", alloy=False)
    got = a0.copy()
    cp = _ctx(pkg, cells, potentials["fe"], "fp64", 4)
    inter = np.zeros(16, dtype=pkg.ATOM_DTYPE)
    n = 0
    for _ in range(3):
        n = cp.step_host(got, inter, n, 1)
    ref = orc.OracleSim(cells, A0, RCF, potentials["fe"], dt=0.001)
    ref.set_atoms(a0)
    ref.exchange_atom_first()
    ref.simulate(3)
    w = ref.get_atoms()
    loc = wl.local_slot_indices(cells, RCF)
    assert np.array_equal(got["type"][loc], w["type"][loc]) and np.array_equal(got["id"][loc], w["id"][loc])
    assert np.abs(got["x"][loc] - w["x"][loc]).max() < 1e-12
    assert np.abs(got["f"][loc] - w["f"][loc]).max() < 1e-9
    cp.close()


@pytest.mark.parametrize("timing", [False, True])
def test_fused_firststep_is_bit_identical(pkg, wl, potentials, gpu_lib, timing):
    """mg_simulate with the next firststep fused into the force pass (blocks of 4 bodies, then single
    bodies) against one body per launch, bit for bit: first a thermal alloy (fusion active), then the
    same state with a few atoms pushed off their sites, so inter atoms appear and the kernels fall
    back to the separate firststep on the device."""
    cells = (10, 9, 11)
    atoms = wl.build_state(cells, A0, RCF, temperature=600.0, seed=31, cu_frac=0.05, ni_frac=0.03)
    loc = wl.local_slot_indices(cells, RCF)
    out = []
    for fuse in (4, 0):
        c = pkg.Context(cells, A0, RCF, precision="mixed", inter_capacity=256)
        c.pot_init_setfl(potentials["fecuni"])
        c.set_timestep(0.001)
        c.set_step_fusion(fuse)
        c.upload(atoms)
        c.prepare()
        c.enable_timing(timing)
        c.simulate(11, sync=True)    # two fused blocks of 4, then 3 single bodies
        mid, _ = c.download()
        assert c.thermo()["n_inter"] == 0
        pushed = mid.copy()
        for k in (17, 400, 901):  # to an octahedral interstice: inter atoms for the rest of the run
            pushed["x"][loc[k]] += A0 * np.array([0.5, 0.5, 0.0])
        c.upload(pushed)
        c.prepare()
        c.simulate(9, sync=True)
        a, inter = c.download()
        out.append((mid, a, inter, c.thermo()["n_inter"]))
        c.close()
    (m1, a1, i1, n1), (m0, a0_, i0, n0) = out
    assert m1.tobytes() == m0.tobytes()
    assert n1 == n0 and n1 > 0
    assert a1.tobytes() == a0_.tobytes() and i1.tobytes() == i0.tobytes()
