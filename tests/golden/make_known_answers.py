"""Writes reference_known_answers.json: the known-answer cases of the reference's unit tests that pin
the indexing tier (Wigner-Seitz mapping, out-of-box flags, offset tables, PKA velocity, temperature).

Each case copies the inputs and expected values of one EXPECT_* in the named reference test file.
The reference's tests are gtest C++ that cannot be built here (no MPI, libcomm, kiwi or gtest), so
the values are transcribed; run this script to regenerate the JSON.
"""
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))

cases = {
    # tests/unit/lattice/ws_utils_test.cpp:13-51 -- every site of a 2x2x2-rank sub-domain maps to
    # itself, also after a (+0.1, -0.2, +0.15) a0 perturbation.
    "ws_identity": {
        "source": "tests/unit/lattice/ws_utils_test.cpp:13-51",
        "grid_size": [2, 2, 2], "grid_coord": [0, 0, 0], "local_space": [50, 60, 72],
        "lattice_const": 0.86, "cutoff_radius_factor": 1.1421,
        "perturbation": [0.1, -0.2, 0.15],
    },
    # tests/unit/lattice/ws_utils_test.cpp:54-102, x even, z negative
    "ws_minus_z_even": {
        "source": "tests/unit/lattice/ws_utils_test.cpp:54-102",
        "grid_size": [2, 2, 2], "grid_coord": [0, 0, 0], "local_space": [25, 25, 25],
        "lattice_const": 2.85532, "cutoff_radius_factor": 1.96125,
        "points": [
            {"x": [0.0, 0.0, "-0.01"], "axis": 2, "expect": 0},
            {"x": [0.0, 0.0, "a*(-2)-0.01"], "axis": 2, "expect": -2},
            {"x": [0.0, 0.0, "a*(-2.44)"], "axis": 2, "expect": -2},
            {"x": [0.0, 0.0, "a*(-2.66)"], "axis": 2, "expect": -3},
        ],
    },
    # tests/unit/lattice/ws_utils_test.cpp:104-156, x odd, z negative
    "ws_minus_z_odd": {
        "source": "tests/unit/lattice/ws_utils_test.cpp:104-156",
        "grid_size": [2, 2, 2], "grid_coord": [0, 0, 0], "local_space": [25, 25, 25],
        "lattice_const": 2.85532, "cutoff_radius_factor": 1.96125,
        "points": [
            {"x": ["3.5*a", "0.5*a", "-0.01"], "axis": 2, "expect": -1},
            {"x": ["3.5*a", "0.5*a", "a*(-2)+0.01"], "axis": 2, "expect": -2},
            {"x": ["3.5*a", "0.5*a", "a*(-2)-0.01"], "axis": 2, "expect": -3},
            {"x": ["3.5*a", "0.5*a", "a*(-2.44)"], "axis": 2, "expect": -3},
            {"x": ["3.5*a", "0.5*a", "a*(-2.66)"], "axis": 2, "expect": -3},
        ],
    },
    # tests/unit/lattice/ws_utils_test.cpp:158-209, x negative (doubled coordinate expected)
    "ws_minus_x": {
        "source": "tests/unit/lattice/ws_utils_test.cpp:158-209",
        "grid_size": [2, 2, 2], "grid_coord": [0, 0, 0], "local_space": [25, 25, 25],
        "lattice_const": 2.85532, "cutoff_radius_factor": 1.96125,
        "points": [
            {"x": ["-0.01", 0.0, 0.0], "axis": 0, "expect": 0},
            {"x": ["a*(-2)-0.01", 0.0, 0.0], "axis": 0, "expect": -4},
            {"x": ["a*(-2-0.1)", 0.0, 0.0], "axis": 0, "expect": -4},
            {"x": ["a*(-2+0.1)", 0.0, 0.0], "axis": 0, "expect": -4},
            {"x": ["a*(-2.25-0.1)", 0.0, 0.0], "axis": 0, "expect": -4},
            {"x": ["a*(-2.75+0.1)", 0.0, 0.0], "axis": 0, "expect": -6},
            {"x": ["a*(-2.75-0.1)", 0.0, 0.0], "axis": 0, "expect": -6},
        ],
    },
    # tests/unit/inter_atom_test.cpp:26-62 -- isOutBox flags (1 x-low, 4 y-low, 16 z-low)
    "is_out_box_litter": {
        "source": "tests/unit/inter_atom_test.cpp:26-62",
        "grid_size": [2, 2, 2], "grid_coord": [0, 0, 0], "local_space": [50, 60, 72],
        "lattice_const": 0.86, "cutoff_radius_factor": 1.1421,
        "points": [
            {"x": ["10*a", "10*a", "10*a"], "expect": 0},
            {"x": ["-10*a", "10*a", "10*a"], "expect": 1},
            {"x": ["-0.01", "10*a", "10*a"], "expect": 0},
            {"x": ["-a/2-0.01", "-a/2-0.01", "-a/2-0.01"], "expect": 21},
        ],
    },
    # tests/unit/inter_atom_test.cpp:65-79 -- periodic boundary rank (1,1,0) of a 2x2x1 grid
    "is_out_box_big": {
        "source": "tests/unit/inter_atom_test.cpp:65-79",
        "grid_size": [2, 2, 1], "grid_coord": [1, 1, 0], "local_space": [25, 25, 50],
        "lattice_const": 2.85532, "cutoff_radius_factor": 1.96125,
        "points": [{"x": [71.3905, 71.3921, 74.234], "expect": 0}],
    },
    # tests/unit/neighbour_index_test.cpp:110-114
    "is_positive_index": {
        "source": "tests/unit/neighbour_index_test.cpp:110-114",
        "points": [{"x": [-3, -2, 0], "expect": False}, {"x": [-3, -2, -1], "expect": False},
                   {"x": [-3, 1, 0], "expect": True}],
    },
    # tests/unit/neighbour_index_test.cpp:117-130: ext 8, box 6, ghost 2, make(ghost, ghost - 0.1)
    "offset_lengths": {
        "source": "tests/unit/neighbour_index_test.cpp:117-130",
        "ext": 8, "cut_lattice": 2, "cutoff_radius_factor": 1.9,
    },
    # tests/unit/neighbour_index_test.cpp:132-145: make(2, 0.51*sqrt(3)) expects 8 entries, but
    # make() searches rcf + 2 * LAT_CUTOFF (src/atom/neighbour_index.inl:18, LAT_CUTOFF 0.5), which
    # gives 58: the reference's own test fails against its code, like the 2nn case at :147-161.
    # Ported as: the 8 first neighbours are in the table and the length equals the BCC vector count
    # inside rcf + 1.
    "offset_1nn": {
        "source": "tests/unit/neighbour_index_test.cpp:132-145",
        "ext": 8, "cut_lattice": 2, "cutoff_radius_factor": "0.51*sqrt(3)", "first_shell": 8,
        "reference_expect_full": 8, "reference_test_fails_on_its_code": True,
    },
    # tests/unit/neighbour_index_test.cpp:163-185: ext 9 grid, make(3, 1.96125); (23,17,4) is a
    # half-list neighbour of (24,16,3)
    "offset_case": {
        "source": "tests/unit/neighbour_index_test.cpp:163-185",
        "ext": 9, "cut_lattice": 3, "cutoff_radius_factor": 1.96125,
        "source_site": [24, 16, 3], "neighbour": [23, 17, 4], "expect": True,
    },
    # tests/unit/neighbour_index_test.cpp:188-243: tables equal the legacy CrystalMD derivation
    "offset_legacy": {
        "source": "tests/unit/neighbour_index_test.cpp:188-243",
        "box": 6, "cut_lattice": 2, "cutoff_radius_factor": 1.96125,
    },
    # tests/unit/atom/nei_index_test.cpp:71-173 (random seed fixed here instead of time(NULL))
    "offset_random_pairs": {
        "source": "tests/unit/atom/nei_index_test.cpp:71-173",
        "grid_size": [2, 2, 2], "grid_coord": [0, 0, 0], "local_space": [25, 25, 25],
        "lattice_const": 2.85532, "cutoff_radius_factor": 1.96125, "coord_range": [-5000, 5000],
        "scale": 1000.0, "seed": 20240611,
    },
    # tests/unit/atom_test.cpp:11-54: PKA velocity increments (EXPECT_FLOAT_EQ)
    "setv": {
        "source": "tests/unit/atom_test.cpp:11-54",
        "cases": [
            {"energy": 5000.0, "direction": [1.0, 3.0, 5.0], "type": 0,
             "expect_dv": [222.17975, 666.53928, 1110.89879]},
            {"energy": 20000.0, "direction": [1.0, 2.0, 2.0], "type": 0,
             "expect_dv": [876.28882, 1752.5776, 1752.5776]},
        ],
    },
    # tests/unit/configuration_test.cpp:12-42 and world_builder_test.cpp:13-42: T after rescale(600)
    "rescale_temperature": {
        "source": "tests/unit/configuration_test.cpp:12-42; tests/unit/world_builder_test.cpp:13-42",
        "t_set": 600.0, "momentum_tol": 1e-8,
    },
}

if __name__ == "__main__":
    with open(os.path.join(HERE, "reference_known_answers.json"), "w") as fh:
        json.dump(cases, fh, indent=1)
