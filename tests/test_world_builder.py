"""Creation mode (WorldBuilder::build, src/world_builder.cpp:64-199) on the host: the library's
mg_world_build against the oracle, which restates the same steps with the platform's own rand() and
<random> engines, and the properties the reference's own test checks
(tests/unit/world_builder_test.cpp:13-43)."""
import numpy as np
import pytest

A0 = 2.855
RCF = 5.6 / A0


@pytest.mark.parametrize("rng,cells,ratio,seed,t_set", [
    ("mt", (6, 7, 8), (1, 0, 0), 1234, 600.0),
    ("mt", (8, 6, 6), (97, 3, 1), 1024, 300.0),
    ("lcg", (6, 6, 6), (985, 15, 10), 7, 600.0),
    ("stc", (7, 6, 6), (2, 1, 1), 99, 0.0),
    ("legacy", (6, 6, 7), (1, 1, 0), 466953, 600.0),
])
def test_world_build_matches_oracle(pkg, orc, potentials, rng, cells, ratio, seed, t_set):
    got = pkg.world_build(cells, A0, RCF, t_set, seed, ratio, rng)
    ref = orc.OracleSim(cells, A0, RCF, potentials["fe"])
    ref.world_build(t_set, seed, ratio, pkg.RNG[rng])
    want = ref.get_atoms()
    for f in ("id", "type", "x", "v", "f", "rho", "df"):
        assert np.array_equal(got[f], want[f]), f


def test_world_build_reference_properties(pkg, wl):
    """The reference's zero_momentum_test: 50 x 60 x 72 cells, a0 0.86, ratio 97:3:1, seed 1024,
    T 600: temperature 600 (float equality) and every momentum component within 1e-8."""
    cells, a0, rcf = (50, 60, 72), 0.86, 1.1421
    atoms = pkg.world_build(cells, a0, rcf, 600.0, 1024, (97, 3, 1), "mt")
    loc = wl.local_slot_indices(cells, rcf)
    a = atoms[loc]
    assert np.array_equal(a["id"], np.arange(1, loc.size + 1, dtype=np.uint64))
    m = np.asarray(wl.MASS)[a["type"]]
    mvv = float(((a["v"] ** 2).sum(axis=1) * m).sum())
    n = 2 * cells[0] * cells[1] * cells[2]
    t = mvv * wl.MVV2E / ((3 * n - 3) * wl.BOLTZ)
    assert np.float32(t) == np.float32(600.0) or abs(t - 600.0) <= 4 * np.spacing(np.float32(600.0))
    p = (a["v"] * m[:, None]).sum(axis=0)
    assert np.abs(p).max() < 1e-8
    frac = np.bincount(a["type"], minlength=3) / a.size
    assert abs(frac[1] - 3 / 101) < 0.003 and abs(frac[2] - 1 / 101) < 0.002
    ghosts = np.setdiff1d(np.arange(atoms.size), loc)
    assert (atoms["type"][ghosts] == -1).all()


def test_world_build_rejects_bad_input(pkg, wl):
    with pytest.raises(pkg.MgError):
        pkg.world_build((6, 6, 6), A0, RCF, 600.0, 1, (0, 0, 0))        # no atom type selected
    lib = pkg.load_library()
    Sx, Sy, Sz, _, _, _ = wl.grid((6, 6, 6), RCF)
    atoms = np.zeros(Sx * Sy * Sz, dtype=pkg.ATOM_DTYPE)
    ps = np.array([6, 6, 6], dtype=np.int64)
    ratio = np.array([1, 0, 0], dtype=np.int32)
    ptr = lambda a: a.ctypes.data_as(__import__("ctypes").c_void_p)
    assert lib.mg_world_build(ptr(ps), A0, RCF, 600.0, 1, ptr(ratio), 9, ptr(atoms), atoms.size) == 1   # engine
    assert lib.mg_world_build(ptr(ps), A0, RCF, 600.0, 1, ptr(ratio), 0, ptr(atoms), atoms.size - 1) == 1  # size
