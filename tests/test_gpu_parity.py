"""GPU parity against the CPU oracle, through the C ABI (libmisa_gb300.so).

Tiers: integer/index work (Wigner-Seitz mapping, offset tables, ghost map, decide/exchange/border,
inter-atom list order and contents) is compared bit for bit; FP64 forces within 1e-9 eV/A; the mixed
form within its error budget (force RMS <= 1e-5 eV/A).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

A0 = 2.855
RCF = 5.6 / A0
F64_TOL = 1e-9     # eV/A, FP64 build
MIX_RMS = 1e-5     # eV/A, mixed form
MIX_MAX = 1e-4


def make_pair(pkg, orc, wl, pot, cells, atoms, precision="fp64", dt=0.001, inter_capacity=0):
    ctx = pkg.Context(cells, A0, RCF, precision=precision, inter_capacity=inter_capacity)
    ctx.pot_init_setfl(pot)
    ctx.set_timestep(dt)
    ctx.upload(atoms)
    ref = orc.OracleSim(cells, A0, RCF, pot, dt=dt)
    ref.set_atoms(atoms)
    return ctx, ref


def local(wl, cells):
    return wl.local_slot_indices(cells, RCF)


def ghosts(wl, cells):
    Sx, Sy, Sz, gx, gy, gz = wl.grid(cells, RCF)
    allidx = np.arange(Sx * Sy * Sz)
    return np.setdiff1d(allidx, local(wl, cells))


def assert_records_equal(a, b, fields=("id", "type", "x", "v", "f", "rho", "df")):
    for f in fields:
        assert np.array_equal(a[f], b[f]), f


def displaced_state(wl, cells, seed, n_move=40, temperature=300.0):
    """A crystal with atoms pushed off their sites: some inside their WS cell, some into neighbouring
    cells, some through the box faces."""
    atoms = wl.build_state(cells, A0, RCF, temperature=temperature, seed=seed)
    loc = local(wl, cells)
    rng = np.random.default_rng(seed)
    pick = rng.choice(loc.size, size=n_move, replace=False)
    for q, k in enumerate(pick):
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        atoms["x"][loc[k]] += d * A0 * (0.22 + 0.3 * (q % 4) / 3)
    # atoms on the low and high faces pushed outward
    Sx, Sy, Sz, gx, gy, gz = wl.grid(cells, RCF)
    for s, dvec in ((loc[0], (-0.6, 0.0, 0.0)), (loc[-1], (0.0, 0.0, 0.6)), (loc[2 * cells[0] * 3], (0.0, -0.6, 0.1))):
        atoms["x"][s] += np.asarray(dvec) * A0
    return atoms


# ------------------------------------------------------------------------------------------------
# indexing tier
# ------------------------------------------------------------------------------------------------
def test_ws_map_matches_oracle(pkg, orc, wl, potentials, gpu_lib):
    cells = (25, 25, 25)
    a = 2.85532
    rcf = 1.96125
    ctx = pkg.Context(cells, a, rcf)
    desc = orc.domain_desc(cells, a, rcf)
    rng = np.random.default_rng(3)
    L = np.asarray(cells) * a
    pts = [rng.uniform(-2 * a, L + 2 * a, size=(20000, 3))]
    # lattice sites, half-way points and exact bisector-plane points
    s = rng.integers(-2, 27, size=(4000, 3)).astype(float) * a
    pts += [s, s + 0.5 * a, s + 0.25 * a, s + np.array([0.25, 0.25, 0.25]) * a, s - 0.5 * a]
    # the neighbourhoods of those decision boundaries (nearest integer, sign of the offset, bisector
    # plane), from one ulp to past the margin within which the search re-divides exactly
    edge = np.concatenate([s, s + 0.5 * a, s + np.array([0.25, 0.25, 0.25]) * a, s + np.array([0.5, 0.25, 0.0]) * a])
    pts += [np.nextafter(edge, np.inf), np.nextafter(edge, -np.inf)]
    for eps in (1e-15, 1e-12, 1e-10, 5e-10, 1e-9, 2e-9, 1e-8):
        pts.append(edge + eps * a * rng.choice([-1.0, 0.0, 1.0], size=edge.shape))
    # coordinates beyond 2^20 lattice constants
    pts.append(rng.uniform(-3e6, 3e6, size=(500, 3)) * a)
    xyz = np.concatenate(pts)
    coords, flags, index = ctx.ws_map(xyz)
    ext, _, oflags, oindex = orc.ws_batch(desc, xyz)
    assert np.array_equal(coords, ext)
    assert np.array_equal(flags, oflags)
    assert np.array_equal(index, oindex)
    ctx.close()


def test_offset_tables_match_oracle(pkg, orc, wl, gpu_lib):
    cells = (10, 11, 12)
    ctx = pkg.Context(cells, A0, RCF)
    Sx, Sy, Sz, gx, gy, gz = ctx.grid
    t = [orc.nei_offsets(Sx, Sy, Sz, 2, RCF, w) for w in range(4)]
    for w in range(4):
        assert np.array_equal(ctx.nei_offsets(w), t[w])
    ctx.nei_offset_init(*t)
    with pytest.raises(pkg.MgError):
        bad = [x.copy() for x in t]
        bad[0][3] += 1
        ctx.nei_offset_init(*bad)
    # the pruned gather tables are the full entries within rc + 0.4 a0, in reference order
    for p in (0, 1):
        pruned = ctx.nei_offsets(4 + p)
        assert pruned.size == 112 // 2 * 2 and set(pruned) <= set(t[p])
    ctx.close()


def test_spline_coefficients_identical(pkg, orc, wl, potentials, gpu_lib):
    cells = (6, 6, 6)
    ctx = pkg.Context(cells, A0, RCF)
    ctx.pot_init_setfl(potentials["fecuni"])
    ref = orc.OracleSim(cells, A0, RCF, potentials["fecuni"])
    for kind, e1, e2 in [(0, 0, 0), (0, 2, 0), (1, 1, 0), (2, 0, 0), (2, 2, 1), (2, 1, 2)]:
        assert np.array_equal(ctx.pot_spline(kind, e1, e2), ref.pot_spline(kind, e1, e2)), (kind, e1, e2)
    ctx.close()


def test_ghost_map_bit_exact(pkg, orc, wl, potentials, gpu_lib):
    cells = (7, 8, 9)
    atoms = wl.build_state(cells, A0, RCF, temperature=900.0, seed=21)
    loc = local(wl, cells)
    atoms["x"][loc] += np.random.default_rng(1).uniform(-0.1, 0.1, size=(loc.size, 3))
    atoms["type"][loc[::13]] = -1
    ctx, ref = make_pair(pkg, orc, wl, potentials["fe"], cells, atoms)
    ctx.phase(4)  # exchangeAtom
    ref.exchange_atom_first()
    got, _ = ctx.download()
    want = ref.get_atoms()
    g = ghosts(wl, cells)
    assert np.array_equal(got["type"][g], want["type"][g])
    assert np.array_equal(got["x"][g], want["x"][g])
    ctx.close()


# ------------------------------------------------------------------------------------------------
# EAM arithmetic
# ------------------------------------------------------------------------------------------------
@pytest.mark.parametrize("pot_name,prec", [("fe", "fp64"), ("fecuni", "fp64"), ("fe", "mixed"), ("fecuni", "mixed")])
def test_compute_eam_parity(pkg, orc, wl, potentials, gpu_lib, pot_name, prec):
    cells = (9, 8, 10)
    alloy = pot_name == "fecuni"
    atoms = wl.build_state(cells, A0, RCF, temperature=600.0, seed=5, cu_frac=0.1 if alloy else 0.0,
                           ni_frac=0.08 if alloy else 0.0)
    loc = local(wl, cells)
    atoms["x"][loc] += np.random.default_rng(2).uniform(-0.12, 0.12, size=(loc.size, 3))
    atoms["type"][loc[5::97]] = -1  # vacancies
    ctx, ref = make_pair(pkg, orc, wl, potentials[pot_name], cells, atoms, precision=prec)
    ctx.prepare()
    ref.prepare()
    got, _ = ctx.download()
    want = ref.get_atoms()
    occ = loc[want["type"][loc] >= 0]
    df = got["f"][occ] - want["f"][occ]
    if prec == "fp64":
        assert np.abs(df).max() <= F64_TOL
        assert np.allclose(got["rho"][occ], want["rho"][occ], rtol=1e-13, atol=0)
        assert np.allclose(got["df"][occ], want["df"][occ], rtol=1e-12, atol=1e-15)
    else:
        assert np.sqrt((df ** 2).mean()) <= MIX_RMS
        assert np.abs(df).max() <= MIX_MAX
        assert np.allclose(got["rho"][occ], want["rho"][occ], rtol=1e-6)
    vac = loc[want["type"][loc] < 0]
    assert (got["f"][vac] == 0).all() and (got["rho"][vac] == 0).all()
    ctx.close()


def test_steps_parity_fp64(pkg, orc, wl, potentials, gpu_lib):
    cells = (8, 8, 8)
    atoms = wl.build_state(cells, A0, RCF, temperature=600.0, seed=8)
    ctx, ref = make_pair(pkg, orc, wl, potentials["fe"], cells, atoms)
    ctx.prepare()
    ref.prepare()
    ctx.simulate(20)
    ref.simulate(20)
    got, _ = ctx.download()
    want = ref.get_atoms()
    loc = local(wl, cells)
    assert np.abs(got["x"][loc] - want["x"][loc]).max() < 1e-10
    assert np.abs(got["v"][loc] - want["v"][loc]).max() < 1e-8
    assert np.abs(got["f"][loc] - want["f"][loc]).max() < F64_TOL
    t = ctx.thermo()
    assert t["mvv"] == pytest.approx(ref.mvv(), rel=1e-12)
    assert np.allclose(t["force_sum"], ref.system_force(), atol=1e-9)
    ctx.close()


def test_mixed_error_budget_and_energy(pkg, orc, wl, potentials, gpu_lib):
    cells = (10, 10, 10)
    atoms = wl.build_state(cells, A0, RCF, temperature=600.0, seed=12, cu_frac=0.015, ni_frac=0.01)
    ctx, ref = make_pair(pkg, orc, wl, potentials["fecuni"], cells, atoms, precision="mixed")
    ctx.prepare()
    ref.prepare()
    got, _ = ctx.download()
    want = ref.get_atoms()
    loc = local(wl, cells)
    d = got["f"][loc] - want["f"][loc]
    assert np.sqrt((d ** 2).mean()) <= MIX_RMS
    pe_ref, e_ref, _ = ref.potential_energy(per_slot=True)
    t = ctx.thermo(with_energy=True)
    assert t["potential_energy"] == pytest.approx(pe_ref, rel=1e-7)
    e_got, _ = ctx.energies()
    assert np.abs(e_got[loc] - e_ref[loc]).max() < 1e-6
    ctx.close()


def test_energy_parity_fp64(pkg, orc, wl, potentials, gpu_lib):
    cells = (8, 9, 8)
    atoms = displaced_state(wl, cells, seed=31)
    ctx, ref = make_pair(pkg, orc, wl, potentials["fecuni"], cells, atoms)
    # one step so that inter atoms exist, then energies on the post-step state
    ctx.prepare(); ref.prepare()
    ctx.simulate(1); ref.simulate(1)
    ref.clear_force(); ref.compute_eam()
    pe_ref, e_ref, e_inter = ref.potential_energy(per_slot=True, inter_cap=1000)
    t = ctx.thermo(with_energy=True)
    assert t["n_inter"] == ref.get_inter().size > 0
    assert t["potential_energy"] == pytest.approx(pe_ref, rel=1e-12)
    e_got, ei_got = ctx.energies(inter_cap=t["n_inter"])
    loc = local(wl, cells)
    assert np.abs(e_got[loc] - e_ref[loc]).max() < 1e-10
    assert np.abs(ei_got - e_inter[:t["n_inter"]]).max() < 1e-10
    ctx.close()


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_inter_atom_runs_are_reproducible(pkg, wl, potentials, gpu_lib, prec):
    """Two runs of the same cascade give the same bits: the lattice atoms' shares of the inter-atom
    pairs are summed by their owners in a fixed order, so no result depends on thread timing. After
    the PKA and 150 steps about a dozen inter atoms remain, most of them sharing lattice neighbours;
    dozens passed through the list on the way."""
    cells = (10, 10, 10)
    atoms = displaced_state(wl, cells, seed=41, n_move=80)
    out = []
    for _ in range(2):
        ctx = pkg.Context(cells, A0, RCF, precision=prec, inter_capacity=4096)
        ctx.pot_init_setfl(potentials["fecuni"] if prec == "mixed" else potentials["fe"])
        ctx.upload(atoms)
        ctx.prepare()
        ctx.collision_step((5, 5, 5, 1), (0.3, 1.0, 0.2), 600.0)
        ctx.set_variable_timestep(0.01, 1e-5, 1e-3)
        ctx.simulate(150)
        a, inter = ctx.download()
        t = ctx.thermo(with_energy=True)
        e, ei = ctx.energies(inter_cap=inter.size)
        out.append((a.tobytes(), inter.tobytes(), e.tobytes(), ei.tobytes(), t["potential_energy"], inter.size))
        ctx.close()
    assert out[0] == out[1]
    assert out[0][5] >= 8


# ------------------------------------------------------------------------------------------------
# migration tier: decide, exchangeInter, borderInter bit for bit
# ------------------------------------------------------------------------------------------------
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("cells,n_move", [((8, 9, 10), 60), ((20, 20, 20), 8000)])
def test_decide_exchange_border_bit_exact(pkg, orc, wl, potentials, gpu_lib, prec, cells, n_move):
    """The list phases one at a time against the oracle's. The 20^3 box moves 8,000 of its 16,000
    atoms: about 1,400 stay inter atoms, with about 1,700 ghost images, so the list and the entries of
    every border pass span more than one chunk of the list manager's block (1,024 threads)."""
    atoms = displaced_state(wl, cells, seed=17, n_move=n_move)
    ctx, ref = make_pair(pkg, orc, wl, potentials["fe"], cells, atoms, precision=prec)
    for phase, fn in ((1, ref.decide), (2, ref.exchange_inter), (3, ref.border_inter)):
        ctx.phase(phase)
        fn()
        got, inter = ctx.download()
        want = ref.get_atoms()
        loc = local(wl, cells)
        fields = ("id", "type", "x", "v", "f", "rho") if prec == "mixed" else ("id", "type", "x", "v", "f", "rho", "df")
        assert_records_equal(got[loc], want[loc], fields)
        assert_records_equal(inter, ref.get_inter(), fields)
    gi = ctx.download_ghost_inter()
    wi = ref.get_ghost_inter()
    assert gi.size == wi.size > 0
    assert np.array_equal(gi["type"], wi["type"]) and np.array_equal(gi["x"], wi["x"])
    ctx.close()


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_steps_with_inter_atoms(pkg, orc, wl, potentials, gpu_lib, prec):
    cells = (8, 8, 8)
    atoms = displaced_state(wl, cells, seed=23, n_move=50)
    ctx, ref = make_pair(pkg, orc, wl, potentials["fe"], cells, atoms, precision=prec)
    ctx.prepare()
    ref.prepare()
    loc = local(wl, cells)
    tol = F64_TOL if prec == "fp64" else MIX_MAX * 50
    for step in range(8):
        ctx.simulate(1)
        ref.simulate(1)
        got, inter = ctx.download()
        want = ref.get_atoms()
        winter = ref.get_inter()
        # membership and order of the inter-atom list, and the vacancy pattern, are exact
        assert np.array_equal(inter["id"], winter["id"]), step
        assert np.array_equal(got["type"][loc], want["type"][loc]), step
        assert np.abs(got["f"][loc] - want["f"][loc]).max() < tol, step
        if inter.size:
            assert np.abs(inter["f"] - winter["f"]).max() < tol, step
            assert np.allclose(inter["rho"], winter["rho"], rtol=1e-6 if prec == "mixed" else 1e-12)
    assert winter.size > 0
    ctx.close()


def test_collision_step_parity(pkg, orc, wl, potentials, gpu_lib):
    cells = (10, 10, 10)
    atoms = wl.build_state(cells, A0, RCF, temperature=300.0, seed=41)
    ctx, ref = make_pair(pkg, orc, wl, potentials["fe"], cells, atoms, dt=0.0001)
    ctx.prepare()
    ref.prepare()
    lat, direction, energy = [5, 5, 5, 1], [1.0, 3.0, 5.0], 5000.0
    ctx.collision_step(lat, direction, energy)
    ref.collision_step(lat, direction, energy)
    got, _ = ctx.download()
    want = ref.get_atoms()
    loc = local(wl, cells)
    assert np.array_equal(got["v"][loc], want["v"][loc])  # setv arithmetic is exact
    assert np.abs(got["f"][loc] - want["f"][loc]).max() < F64_TOL
    for step in range(30):
        ctx.simulate(1)
        ref.simulate(1)
        _, inter = ctx.download()
        assert np.array_equal(inter["id"], ref.get_inter()["id"]), step
    ctx.close()


# ------------------------------------------------------------------------------------------------
# the reference's per-phase hooks on host AoS arrays
# ------------------------------------------------------------------------------------------------
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_hooks_parity(pkg, orc, wl, potentials, gpu_lib, prec):
    cells = (8, 8, 9)
    atoms = wl.build_state(cells, A0, RCF, temperature=600.0, seed=51)
    loc = local(wl, cells)
    atoms["x"][loc] += np.random.default_rng(5).uniform(-0.1, 0.1, size=(loc.size, 3))
    ctx = pkg.Context(cells, A0, RCF, precision=prec)
    ctx.pot_init_setfl(potentials["fe"])
    ref = orc.OracleSim(cells, A0, RCF, potentials["fe"])
    ref.set_atoms(atoms)
    ref.exchange_atom_first()
    ref.clear_force()
    host = ref.get_atoms()  # ghosts filled, rho = f = 0 (the state latRho sees)
    ref.compute_eam()
    want = ref.get_atoms()
    ctx.eam_rho_calc(host)
    rtol = 1e-13 if prec == "fp64" else 1e-6
    assert np.allclose(host["rho"][loc], want["rho"][loc], rtol=rtol, atol=0)
    ctx.eam_df_calc(host)
    assert np.allclose(host["df"][loc], want["df"][loc], rtol=1e-12 if prec == "fp64" else 1e-6)
    g = ghosts(wl, cells)
    host["df"][g] = want["df"][g]  # the host's forward df exchange
    ctx.eam_force_calc(host)
    d = host["f"][loc] - want["f"][loc]
    if prec == "fp64":
        assert np.abs(d).max() <= F64_TOL
    else:
        assert np.sqrt((d ** 2).mean()) <= MIX_RMS
    ctx.close()


# ------------------------------------------------------------------------------------------------
# size-independent properties at larger sizes, determinism, error paths
# ------------------------------------------------------------------------------------------------
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_large_box_invariants(pkg, wl, potentials, gpu_lib, prec):
    cells = (48, 40, 44)
    atoms = wl.build_state(cells, A0, RCF, temperature=0.0, seed=61)
    ctx = pkg.Context(cells, A0, RCF, precision=prec)
    ctx.pot_init_setfl(potentials["fe"])
    ctx.upload(atoms)
    ctx.prepare()
    got, _ = ctx.download()
    loc = local(wl, cells)
    # perfect lattice: every force vanishes by symmetry
    assert np.abs(got["f"][loc]).max() < (1e-12 if prec == "fp64" else 1e-5)
    atoms = wl.build_state(cells, A0, RCF, temperature=600.0, seed=61)
    ctx.upload(atoms)
    ctx.prepare()
    ctx.simulate(10)
    t = ctx.thermo()
    n = loc.size
    assert np.abs(t["force_sum"]).max() / n < (1e-13 if prec == "fp64" else 1e-7)
    got1, _ = ctx.download()
    # determinism: the same input gives the same bits
    ctx.upload(atoms)
    ctx.prepare()
    ctx.simulate(10)
    got2, _ = ctx.download()
    assert np.array_equal(got1["x"], got2["x"]) and np.array_equal(got1["v"], got2["v"])
    ctx.close()


def test_capacity_overflow_is_reported(pkg, wl, potentials, gpu_lib):
    cells = (8, 8, 8)
    atoms = displaced_state(wl, cells, seed=71, n_move=60)
    ctx = pkg.Context(cells, A0, RCF, inter_capacity=4)
    ctx.pot_init_setfl(potentials["fe"])
    ctx.upload(atoms)
    with pytest.raises(pkg.MgError) as e:
        ctx.phase(1)
    assert e.value.status == 4
    ctx.close()


def test_bad_inputs_are_rejected(pkg, wl, potentials, gpu_lib, tmp_path):
    cells = (6, 6, 6)
    ctx = pkg.Context(cells, A0, RCF)
    bad = tmp_path / "bad.setfl"
    bad.write_text("a\nb\nc\n1 Fe\n5000 0.04 5000 0.001 5.6\n26 55.8 2.855 bcc\n1.0 2.0\n")
    with pytest.raises(pkg.MgError) as e:
        ctx.pot_init_setfl(str(bad))
    assert e.value.status == 3
    with pytest.raises(pkg.MgError):
        ctx.prepare()  # no potential yet
    ctx.pot_init_setfl(potentials["fe"])
    atoms = wl.build_state(cells, A0, RCF, temperature=300.0, seed=1)
    atoms["type"][wl.local_slot_indices(cells, RCF)[3]] = 1  # Cu with a Fe-only table
    ctx.upload(atoms)
    with pytest.raises(pkg.MgError):
        ctx.prepare()
    with pytest.raises(pkg.MgError):
        pkg.Context((4, 6, 6), A0, RCF)  # narrower than 2 ghost widths
    with pytest.raises(pkg.MgError):
        pkg.Context((1300, 1300, 1300), A0, RCF)  # more slots than 32-bit indices address
    with pytest.raises(pkg.MgError):
        pkg.Context((6, 6, 1 << 40), A0, RCF)
    ctx.close()


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_autotune_keeps_results_bit_identical(pkg, wl, potentials, gpu_lib, prec):
    cells = (14, 12, 13)
    atoms = wl.build_state(cells, A0, RCF, temperature=600.0, seed=81, cu_frac=0.02, ni_frac=0.01)
    runs = []
    for tune in (None, (1, 128, 1, 512), (0, 256, 1, 128, 2, 4), "auto"):
        ctx = pkg.Context(cells, A0, RCF, precision=prec)
        ctx.pot_init_setfl(potentials["fecuni"])
        ctx.upload(atoms)
        ctx.prepare()
        if tune == "auto":
            t = ctx.autotune(reps=2)
            assert t["rho_order"] in (0, 1) and t["force_block"] in (128, 256, 512) and t["force_apt"] in (1, 2, 4)
        elif tune is not None:
            ctx.set_tuning(*tune)
        ctx.simulate(20)  # mixed: a fused 16-body graph; (1, 128, 1, 512) walks the group candidate lists
        got, _ = ctx.download()
        runs.append(got)
        ctx.close()
    for r in runs[1:]:
        assert np.array_equal(r["x"], runs[0]["x"]) and np.array_equal(r["f"], runs[0]["f"])


def test_contexts_with_different_boxes_coexist(pkg, orc, wl, potentials, gpu_lib):
    """Each context carries its own offset tables: interleaved steps of two differently sized boxes
    must each match their own oracle."""
    pairs = []
    for cells, seed in (((8, 8, 8), 91), ((11, 9, 10), 92)):
        atoms = wl.build_state(cells, A0, RCF, temperature=600.0, seed=seed)
        ctx, ref = make_pair(pkg, orc, wl, potentials["fe"], cells, atoms)
        ctx.prepare()
        ref.prepare()
        pairs.append((cells, ctx, ref))
    for _ in range(3):
        for cells, ctx, ref in pairs:
            ctx.simulate(2)
            ref.simulate(2)
    for cells, ctx, ref in pairs:
        got, _ = ctx.download()
        want = ref.get_atoms()
        loc = local(wl, cells)
        assert np.abs(got["f"][loc] - want["f"][loc]).max() < F64_TOL
        ctx.close()


def test_fma_probe_orders_the_pipes(pkg, gpu_lib):
    """mg_probe_fma: FP64, FP32 and packed FP32x2 FMA throughput of this GPU, in FLOP/s. On GB300 the
    FP64 pipe is tens of times slower than FP32, and the packed form is at least as fast as scalar FP32."""
    f64, f32, f32x2 = (pkg.probe_fma(k) for k in range(3))
    assert 0.1e12 < f64 < 10e12
    assert f32 > 20 * f64
    assert f32x2 > 0.9 * f32
    with pytest.raises(pkg.MgError):
        pkg.probe_fma(3)
