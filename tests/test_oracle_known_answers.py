"""The oracle against the known answers of the reference's own unit tests (indexing tier)."""
import json
import math
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
KA = json.load(open(os.path.join(HERE, "golden", "reference_known_answers.json")))


def _desc(orc, c):
    space = [c["local_space"][i] * c["grid_size"][i] for i in range(3)]
    return orc.domain_desc(space, c["lattice_const"], c["cutoff_radius_factor"], c["grid_size"], c["grid_coord"])


def _val(v, a):
    return float(eval(v, {"a": a, "sqrt": math.sqrt})) if isinstance(v, str) else float(v)


def test_ws_identity_and_perturbed(orc):
    c = KA["ws_identity"]
    d = _desc(orc, c)
    a = c["lattice_const"]
    nx, ny, nz = 2 * c["local_space"][0], c["local_space"][1], c["local_space"][2]
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    x = x.reshape(-1); y = y.reshape(-1); z = z.reshape(-1)
    pos = np.empty((x.size, 3))
    pos[:, 0] = x * (a / 2)
    odd = x % 2 == 1
    pos[:, 1] = np.where(odd, a * y + a / 2, a * y)
    pos[:, 2] = np.where(odd, a * z + a / 2, a * z)
    want = np.stack([x, y, z], axis=1)
    _, sub, _, _ = orc.ws_batch(d, pos)
    assert np.array_equal(sub, want)
    p = c["perturbation"]
    pos2 = pos.copy()
    pos2[:, 0] = pos[:, 0] + p[0] * a
    pos2[:, 1] = pos[:, 1] - (-p[1]) * a
    pos2[:, 2] = pos[:, 2] + p[2] * a
    _, sub2, _, _ = orc.ws_batch(d, pos2)
    assert np.array_equal(sub2, want)


@pytest.mark.parametrize("name", ["ws_minus_z_even", "ws_minus_z_odd", "ws_minus_x"])
def test_ws_negative_rounding(orc, name):
    c = KA[name]
    d = _desc(orc, c)
    a = c["lattice_const"]
    for p in c["points"]:
        x = [_val(v, a) for v in p["x"]]
        got = orc.ws_near_lat_sub_box_coord(d, x)
        assert got[p["axis"]] == p["expect"], (p, got)


@pytest.mark.parametrize("name", ["is_out_box_litter", "is_out_box_big"])
def test_is_out_box(orc, name):
    c = KA[name]
    d = _desc(orc, c)
    a = c["lattice_const"]
    for p in c["points"]:
        x = [_val(v, a) for v in p["x"]]
        assert orc.ws_is_out_box(d, x) == p["expect"], p


def test_is_positive_index(orc):
    for p in KA["is_positive_index"]["points"]:
        assert orc.is_positive_index(*p["x"]) == p["expect"]


def test_offset_table_lengths(orc):
    c = KA["offset_lengths"]
    e = c["ext"]
    t = [orc.nei_offsets(2 * e, e, e, c["cut_lattice"], c["cutoff_radius_factor"], w) for w in range(4)]
    assert t[1].size == 2 * t[3].size
    assert t[0].size == 2 * t[2].size
    assert t[1].size == t[0].size


def test_offset_first_neighbours(orc):
    c = KA["offset_1nn"]
    e = c["ext"]
    Sx, Sy = 2 * e, e
    rcf = _val(c["cutoff_radius_factor"], 0)
    lim = (rcf + 1.0) ** 2
    # independent count of BCC lattice vectors (corner or body centre) inside the search radius
    r = np.arange(-6, 7)
    X, Y, Z = np.meshgrid(r, r, r, indexing="ij")
    n_corner = int(((X**2 + Y**2 + Z**2 > 0) & (X**2 + Y**2 + Z**2 < lim)).sum())
    n_body = int((((X + 0.5)**2 + (Y + 0.5)**2 + (Z + 0.5)**2) < lim).sum())
    for w, first in ((0, [(-1, -1, -1), (1, -1, -1), (-1, 0, -1), (1, 0, -1), (-1, -1, 0), (1, -1, 0), (-1, 0, 0), (1, 0, 0)]),
                     (1, [(-1, 0, 0), (1, 0, 0), (-1, 1, 0), (1, 1, 0), (-1, 0, 1), (1, 0, 1), (-1, 1, 1), (1, 1, 1)])):
        t = orc.nei_offsets(Sx, Sy, e, c["cut_lattice"], rcf, w)
        assert t.size == n_corner + n_body
        for (dx, dy, dz) in first:
            assert (dz * Sy + dy) * Sx + dx in set(t.tolist())
        assert len(first) == c["first_shell"]


def test_offset_case(orc):
    c = KA["offset_case"]
    e = c["ext"]
    Sx, Sy = 2 * e, e
    half_even = orc.nei_offsets(Sx, Sy, e, c["cut_lattice"], c["cutoff_radius_factor"], 2)
    sx, sy, sz = c["source_site"]
    nx, ny, nz = c["neighbour"]
    src = (sz * Sy + sy) * Sx + sx
    dst = (nz * Sy + ny) * Sx + nx
    assert ((src + half_even) == dst).any() == c["expect"]


def _legacy_offsets(Sx, Sy, cut, rcf):
    """The legacy CrystalMD derivation the reference compares against (neighbour_index_test.cpp:29-107)."""
    lim = rcf + 0.5 + 0.5
    idx = lambda x, y, z: (z * Sy + y) * Sx + x
    fe, fo, he, ho = [], [], [], []
    rng = range(-cut - 1, cut + 2)

    def pos(x, y, z):
        if z > 0:
            return True
        if z == 0:
            return y > 0 or (y == 0 and x > 0)
        return False

    for z in rng:
        for y in rng:
            for x in rng:
                r = x * x + y * y + z * z
                if 0 < r < lim * lim:
                    fe.append(idx(2 * x, y, z))
                    if pos(x, y, z):
                        he.append(idx(2 * x, y, z))
                r = (x + 0.5) ** 2 + (y + 0.5) ** 2 + (z + 0.5) ** 2
                if 0 < r < lim * lim:
                    fe.append(idx(2 * x + 1, y, z))
                    if pos(x + 0.5, y + 0.5, z + 0.5):
                        he.append(idx(2 * x + 1, y, z))
    for z in rng:
        for y in rng:
            for x in rng:
                r = x * x + y * y + z * z
                if 0 < r < lim * lim:
                    fo.append(idx(2 * x, y, z))
                    if pos(x, y, z):
                        ho.append(idx(2 * x, y, z))
                r = (x - 0.5) ** 2 + (y - 0.5) ** 2 + (z - 0.5) ** 2
                if 0 < r < lim * lim:
                    fo.append(idx(2 * x - 1, y, z))
                    if pos(x - 0.5, y - 0.5, z - 0.6):
                        ho.append(idx(2 * x - 1, y, z))
    return [np.sort(np.array(v)) for v in (fe, fo, he, ho)]


def test_offsets_equal_legacy_derivation(orc):
    c = KA["offset_legacy"]
    ext = c["box"] + 2 * c["cut_lattice"]
    Sx, Sy = 2 * ext, ext
    legacy = _legacy_offsets(Sx, Sy, c["cut_lattice"], c["cutoff_radius_factor"])
    for w in range(4):
        got = np.sort(orc.nei_offsets(Sx, Sy, ext, c["cut_lattice"], c["cutoff_radius_factor"], w))
        assert np.array_equal(got, legacy[w]), w


def test_offsets_cover_random_pairs(orc):
    c = KA["offset_random_pairs"]
    d = _desc(orc, c)
    a, rcf = c["lattice_const"], c["cutoff_radius_factor"]
    rc = rcf * a
    g = math.ceil(rcf) + 1
    ext = [c["local_space"][i] + 2 * g for i in range(3)]
    Sx, Sy = 2 * ext[0], ext[1]
    tabs = {p: set(orc.nei_offsets(Sx, Sy, ext[2], math.ceil(rcf), rcf, p).tolist()) for p in (0, 1)}
    rng = np.random.default_rng(c["seed"])
    lo, hi = c["coord_range"]
    checked = 0
    for _ in range(40):
        p1 = rng.integers(lo, hi + 1, size=(2000, 3)) / c["scale"]
        p2 = rng.integers(lo, hi + 1, size=(2000, 3)) / c["scale"]
        near = ((p1 - p2) ** 2).sum(axis=1) < rc * rc
        if not near.any():
            continue
        _, c1, _, _ = orc.ws_batch(d, p1[near])
        _, c2, _, _ = orc.ws_batch(d, p2[near])
        diff = (c2[:, 2] - c1[:, 2]) * Sy * Sx + (c2[:, 1] - c1[:, 1]) * Sx + (c2[:, 0] - c1[:, 0])
        same = (c1 == c2).all(axis=1)
        for k in np.nonzero(~same)[0]:
            assert int(diff[k]) in tabs[int(c1[k, 0] % 2)], (p1[near][k], p2[near][k])
            checked += 1
    assert checked > 100


def test_setv_golden(orc, wl, potentials):
    c = KA["setv"]
    cells = (8, 8, 8)
    a0 = 2.855
    rcf = 5.6 / a0
    for case in c["cases"]:
        atoms = wl.build_state(cells, a0, rcf, temperature=0.0, seed=1)
        s = orc.OracleSim(cells, a0, rcf, potentials["fe"])
        s.set_atoms(atoms)
        lat = [4, 4, 4, 0]
        before = s.get_atoms()
        s.setv(lat, case["direction"], case["energy"])
        after = s.get_atoms()
        Sx, Sy, Sz, gx, gy, gz = wl.grid(cells, rcf)
        kk = ((lat[2] + gz) * Sy + (lat[1] + gy)) * Sx + (2 * lat[0] + gx) + lat[3]
        dv = after["v"][kk] - before["v"][kk]
        assert np.allclose(dv, case["expect_dv"], rtol=4 * 2.0**-23, atol=0), dv  # EXPECT_FLOAT_EQ


def test_rescale_temperature(orc, wl, potentials):
    c = KA["rescale_temperature"]
    cells = (8, 8, 8)
    a0 = 2.855
    rcf = 5.6 / a0
    atoms = wl.build_state(cells, a0, rcf, temperature=437.0, seed=3)
    s = orc.OracleSim(cells, a0, rcf, potentials["fe"])
    s.set_atoms(atoms)
    n = 2 * 8 * 8 * 8
    s.rescale(c["t_set"], n)
    assert s.temperature(n) == pytest.approx(c["t_set"], rel=4 * 2.0**-23)
    local = wl.local_slot_indices(cells, rcf)
    a = s.get_atoms()[local]
    p = (a["v"] * np.asarray(wl.MASS)[a["type"]][:, None]).sum(axis=0)
    assert np.abs(p).max() < c["momentum_tol"] * n
