"""The mixed form's Verlet skin on the group candidate lists: results are bit-identical for every skin.

The density pass visits only the candidates a group had within rc + skin at the last rebuild, and
rebuilds when twice the summed per-step maximum displacement reaches the skin, or when a displacement
record changed outside firststep (an upload, a recombination). Every pair inside the cutoff is still
visited, in the same order, so each run here is compared byte for byte with the same run at skin 0,
where every pass visits all pruned candidates. That holds with inter atoms too: the lattice owners
sum the inter atoms' shares in a fixed order, so a cascade run at two skins gives the same bits.
"""
import numpy as np
import pytest

from test_gpu_parity import A0, RCF, assert_records_equal, displaced_state, local

pytestmark = pytest.mark.gpu

FIELDS = ("id", "type", "x", "v", "f", "rho", "df")


def assert_same_run(run, ref):
    (a, ia), (b, ib) = run, ref
    assert_records_equal(a, b, FIELDS)
    assert_records_equal(ia, ib, FIELDS)


def mixed_ctx(pkg, cells, pot, atoms, skin, dt=0.001, inter_capacity=0):
    ctx = pkg.Context(cells, A0, RCF, precision="mixed", inter_capacity=inter_capacity)
    ctx.pot_init_setfl(pot)
    ctx.set_timestep(dt)
    ctx.set_tuning(1, 256, 1, 256)  # warp-interleaved parities: group lists for any box size
    ctx.set_neighbour_skin(skin)
    ctx.upload(atoms)
    ctx.prepare()
    return ctx


@pytest.mark.parametrize("temperature,dt", [(600.0, 0.001), (3000.0, 0.002)])
def test_skin_runs_are_bit_identical(pkg, wl, potentials, gpu_lib, temperature, dt):
    cells = (14, 12, 13)
    atoms = wl.build_state(cells, A0, RCF, temperature=temperature, seed=101, cu_frac=0.02, ni_frac=0.01)
    runs, stats = {}, {}
    for skin in (0.0, 0.3, 0.12, 0.8):
        ctx = mixed_ctx(pkg, cells, potentials["fecuni"], atoms, skin, dt=dt)
        ctx.simulate(40)  # two fused 16-body graphs and 8 single bodies
        runs[skin] = ctx.download()
        stats[skin] = ctx.skin_stats()
        ctx.close()
    for skin in (0.3, 0.12, 0.8):
        assert_same_run(runs[skin], runs[0.0])
    if temperature == 600.0:
        assert runs[0.0][1].size == 0  # the bit-exact case
    passes, rebuilds = stats[0.0]
    assert passes == 41 and rebuilds == passes  # prepare's pass and one per step; skin 0 always rebuilds
    if temperature == 600.0:
        # at 600 K and 1 fs the lists of a 0.3 A skin last several steps
        assert stats[0.3][1] <= stats[0.3][0] // 3
        assert stats[0.8][1] < stats[0.3][1] <= stats[0.12][1]


def test_skin_with_inter_atoms_and_recombination(pkg, wl, potentials, gpu_lib):
    """Displaced atoms leave their sites, travel as inter atoms and recombine into vacancies (records
    written outside firststep); the lists must be rebuilt each time."""
    cells = (8, 8, 8)
    atoms = displaced_state(wl, cells, seed=23, n_move=50)
    runs, stats = {}, {}
    for skin in (0.0, 0.3):
        ctx = mixed_ctx(pkg, cells, potentials["fe"], atoms, skin)
        for _ in range(12):
            ctx.simulate(1)
        runs[skin] = ctx.download()
        stats[skin] = ctx.skin_stats()
        ctx.close()
    assert_same_run(runs[0.3], runs[0.0])
    assert runs[0.0][1].size > 0
    assert stats[0.3][1] < stats[0.3][0]  # the lists outlived some steps


def test_skin_through_a_cascade(pkg, wl, potentials, gpu_lib):
    """A 1 keV PKA with the variable timestep: fast atoms, many inter atoms, recombinations."""
    cells = (12, 12, 12)
    atoms = wl.build_state(cells, A0, RCF, temperature=300.0, seed=7)
    runs, stats = {}, {}
    for skin in (0.0, 0.3):
        ctx = mixed_ctx(pkg, cells, potentials["fe"], atoms, skin, inter_capacity=4096)
        ctx.set_variable_timestep(0.01, 1e-5, 0.001)
        ctx.collision_step((6, 6, 6, 0), (1.0, 0.8, 0.6), 1000.0)
        ctx.simulate(300)
        runs[skin] = ctx.download()
        stats[skin] = ctx.skin_stats()
        ctx.close()
    assert_same_run(runs[0.3], runs[0.0])
    assert runs[0.0][1].size > 0


def test_upload_between_runs_rebuilds(pkg, wl, potentials, gpu_lib):
    """An upload that moves atoms by more than the skin, between two runs on one context."""
    cells = (10, 10, 10)
    atoms = wl.build_state(cells, A0, RCF, temperature=600.0, seed=5)
    loc = local(wl, cells)
    runs = {}
    for skin in (0.0, 0.3):
        ctx = mixed_ctx(pkg, cells, potentials["fe"], atoms, skin)
        ctx.simulate(10)
        mid, inter = ctx.download()
        rng = np.random.default_rng(3)
        pick = rng.choice(loc.size, size=200, replace=False)
        mid["x"][loc[pick]] += rng.uniform(-0.12, 0.12, size=(200, 3)) * A0  # inside the WS cell
        ctx.upload(mid, inter)
        ctx.prepare()
        ctx.simulate(10)
        runs[skin] = ctx.download()
        ctx.close()
    assert_same_run(runs[0.3], runs[0.0])


def test_skin_changes_on_a_live_context(pkg, wl, potentials, gpu_lib):
    """Changing the skin between runs rebuilds the captured graphs; the trajectory does not change."""
    cells = (10, 10, 10)
    atoms = wl.build_state(cells, A0, RCF, temperature=600.0, seed=9)
    ref = mixed_ctx(pkg, cells, potentials["fe"], atoms, 0.0)
    ref.simulate(60)
    want = ref.download()
    ref.close()
    ctx = mixed_ctx(pkg, cells, potentials["fe"], atoms, 0.3)
    for skin in (0.3, 0.0, 0.5, 0.2):
        ctx.set_neighbour_skin(skin)
        ctx.simulate(15)
    assert_same_run(ctx.download(), want)
    ctx.close()


def test_skin_argument_checks(pkg, wl, potentials, gpu_lib):
    ctx = pkg.Context((6, 6, 6), A0, RCF, precision="mixed")
    for bad in (-0.1, float("nan"), 2 * A0):
        with pytest.raises(pkg.MgError):
            ctx.set_neighbour_skin(bad)
    ctx.set_neighbour_skin(0.0)
    ctx.set_neighbour_skin(A0)
    ctx.close()
