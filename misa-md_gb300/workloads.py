"""Synthetic inputs for the EAM step: setfl potential tables and BCC initial states.

The reference has no bundled potential or test lattice (its Fe-Cu-Ni setfl file is downloaded at
run time), so the workloads are generated from a seed:

* potential: setfl text with nr = nrho = 5000 knots and a 5.6 A cutoff. Pair term Morse
  D[exp(-2a(r-r0)) - 2 exp(-a(r-r0))] (D = 0.4 eV, a = 1.4 /A, r0 = 2.5 A), density
  A exp(-b(r-r0)) (A = 1, b = 1.5 /A), embedding -sqrt(rho). With b = 3.0 /A the BCC lattice at
  a0 = 2.855 A is mechanically unstable (a displaced atom feels an outward force: Einstein constant
  -2.5 eV/A^2, and a 600 K crystal heats past 6000 K within 200 fs as it collapses); b = 1.5 /A gives
  +3.2 eV/A^2 and a stable crystal. ``EamParams(beta=3.0)`` still builds the unstable table. Pair and
  density are multiplied by a C2 quintic switch 1 - 10t^3 + 15t^4 - 6t^5, t = (r - 5.0)/(5.6 - 5.0),
  so both vanish smoothly at the cutoff. The three-element table perturbs each species' Morse and
  density parameters by a uniform factor in [0.9, 1.1] from the seed; cross pairs use geometric means.
* state: the reference's WorldBuilder lattice (src/world_builder.cpp:105-131: positions, ids 1..N
  in k, j, i scan order), random substitutional Cu/Ni from the seed, Maxwell velocities at T,
  momentum removed as WorldBuilder::zeroMomentum does (src/world_builder.cpp:143-156), then scaled
  exactly to T as configuration::rescale does (src/system_configuration.cpp:86-111).

Records use the reference's AtomElement layout (src/atom/atom_element.h:18-41).
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

ATOM_DTYPE = np.dtype(
    [("id", "<u8"), ("type", "<i4"), ("pad_", "<i4"), ("x", "<f8", (3,)), ("v", "<f8", (3,)),
     ("f", "<f8", (3,)), ("rho", "<f8"), ("df", "<f8")],
    align=True,
)
assert ATOM_DTYPE.itemsize == 104

BOLTZ = 8.617343e-5  # src/types/pre_define.h:11
MVV2E = 1.0364269e-4  # src/types/pre_define.h:18
MASS = (55.845, 63.546, 58.6934)  # Fe, Cu, Ni (src/types/atom_types.h:17-19)
ATOMIC_NUMBER = (26, 29, 28)  # src/types/atom_types.h:61-73
SYMBOL = ("Fe", "Cu", "Ni")

INVALID = -1


@dataclass
class EamParams:
    D: float = 0.4
    alpha: float = 1.4
    r0: float = 2.5
    A: float = 1.0
    beta: float = 1.5


# Morse minimum and density reference distance of the single-element table. The listed 2.5 A gives a
# BCC crystal at a0 = 2.855 A that is unstable along the Bain path (its energy falls toward c/a < 1),
# and a 600 K box transforms after ~0.4 ps (inter atoms grow to a quarter of all atoms by 1 ps).
# With 2.65 A the BCC site is a minimum along the Bain path, the Einstein constant rises from 3.2 to
# 6.5 eV/A^2, and 64k- and 2M-atom boxes at 300 K and 600 K stay on their lattice through 3000 steps.
# The multi-element tables keep the listed 2.5 A as the centre of their per-species perturbations:
# the dilute Fe-Cu-Ni alloy built from it is stable as listed.
SINGLE_ELEMENT_R0 = 2.65


@dataclass
class PotentialSpec:
    n_ele: int = 1
    seed: int = 0
    nr: int = 5000
    nrho: int = 5000
    cutoff: float = 5.6
    r_on: float = 5.0
    rho_max: float = 200.0
    lattice_const: float = 2.855
    core: bool = True       # screened-Coulomb core below core_r2, joined to the Morse term on [core_r1, core_r2]
    core_r1: float = 1.0
    core_r2: float = 2.0
    params: list = field(default_factory=list)

    def __post_init__(self):
        if not self.params:
            base = EamParams()
            if self.n_ele == 1:
                self.params = [EamParams(r0=SINGLE_ELEMENT_R0)]
            else:
                rng = np.random.default_rng(self.seed)
                self.params = []
                for _ in range(self.n_ele):
                    f = rng.uniform(0.9, 1.1, size=5)
                    self.params.append(EamParams(base.D * f[0], base.alpha * f[1], base.r0 * f[2],
                                                 base.A * f[3], base.beta * f[4]))


def _switch(r, r_on, rc):
    t = np.clip((r - r_on) / (rc - r_on), 0.0, 1.0)
    return 1.0 - 10.0 * t**3 + 15.0 * t**4 - 6.0 * t**5


# Universal screening function of Ziegler, Biersack and Littmark (The Stopping and Range of Ions in
# Solids, 1985): phi(r) = Zi Zj e^2 / (4 pi eps0 r) * sum_k c_k exp(-d_k r / a),
# a = 0.8854 a_Bohr / (Zi^0.23 + Zj^0.23).
ZBL_C = (0.18175, 0.50986, 0.28022, 0.02817)
ZBL_D = (3.19980, 0.94229, 0.40290, 0.20162)
COULOMB_EV_A = 14.399645   # e^2 / (4 pi eps0) in eV * Angstrom


def zbl_rphi(r, zi, zj):
    """r * phi_ZBL(r) in eV * Angstrom (finite at r = 0)."""
    a = 0.46850 / (zi ** 0.23 + zj ** 0.23)
    return COULOMB_EV_A * zi * zj * sum(c * np.exp(-d * r / a) for c, d in zip(ZBL_C, ZBL_D))


def _smoothstep(r, r1, r2):
    t = np.clip((r - r1) / (r2 - r1), 0.0, 1.0)
    return 10.0 * t**3 - 15.0 * t**4 + 6.0 * t**5


def potential_tables(spec: PotentialSpec):
    """Return (F[e][nrho], rho[e][nr], rphi[pair][nr], drho, dr) for the setfl body."""
    dr = spec.cutoff / (spec.nr - 1)
    drho = spec.rho_max / (spec.nrho - 1)
    r = np.arange(spec.nr) * dr
    rho_grid = np.arange(spec.nrho) * drho
    sw = _switch(r, spec.r_on, spec.cutoff)
    F = np.stack([-np.sqrt(rho_grid) for _ in range(spec.n_ele)])
    rho = np.stack([p.A * np.exp(-p.beta * (r - p.r0)) * sw for p in spec.params])
    pairs = []
    for i in range(spec.n_ele):
        for j in range(i + 1):
            pi, pj = spec.params[i], spec.params[j]
            D = math.sqrt(pi.D * pj.D)
            a = math.sqrt(pi.alpha * pj.alpha)
            r0 = math.sqrt(pi.r0 * pj.r0)
            phi = D * (np.exp(-2.0 * a * (r - r0)) - 2.0 * np.exp(-a * (r - r0))) * sw
            rphi = r * phi
            if spec.core:
                # displacement cascades bring atoms to a fraction of an Angstrom: a Morse term alone
                # peaks near 0.4 keV at r = 0 and lets keV recoils pass through atoms
                s = _smoothstep(r, spec.core_r1, spec.core_r2)
                rphi = (1.0 - s) * zbl_rphi(r, ATOMIC_NUMBER[i], ATOMIC_NUMBER[j]) + s * rphi
            pairs.append(rphi)
    return F, rho, np.stack(pairs), drho, dr


def write_setfl(path: str, spec: PotentialSpec) -> str:
    F, rho, rphi, drho, dr = potential_tables(spec)
    lines = [
        "synthetic EAM: Morse pair, exponential density, -sqrt(rho) embedding" +
        (f", ZBL core joined on [{spec.core_r1}, {spec.core_r2}] A" if spec.core else ""),
        f"seed {spec.seed}; quintic switch on [{spec.r_on}, {spec.cutoff}] A",
        "generated by misa-md_gb300/workloads.py",
        f"{spec.n_ele} " + " ".join(SYMBOL[:spec.n_ele]),
        f"{spec.nrho} {drho:.16e} {spec.nr} {dr:.16e} {spec.cutoff:.16e}",
    ]

    def block(a):
        out = []
        for k in range(0, len(a), 5):
            out.append(" ".join(f"{v:.16e}" for v in a[k:k + 5]))
        return out

    for e in range(spec.n_ele):
        lines.append(f"{ATOMIC_NUMBER[e]} {MASS[e]} {spec.lattice_const} bcc")
        lines += block(F[e])
        lines += block(rho[e])
    for q in range(rphi.shape[0]):
        lines += block(rphi[q])
    tmp = path + f".tmp{os.getpid()}"
    with open(tmp, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    os.replace(tmp, path)
    return path


# ----------------------------------------------------------------------------------------------
# slot grid
# ----------------------------------------------------------------------------------------------
def ghost_size(cutoff_radius_factor: float) -> int:
    """src/simulation.cpp:46: ceil(cutoff_radius_factor) + 1 unit cells."""
    return int(math.ceil(cutoff_radius_factor)) + 1


def grid(cells, cutoff_radius_factor):
    """(Sx, Sy, Sz, gx, gy, gz): ghost-extended slot grid with doubled x (src/atom/atom_set.cpp:18-26)."""
    g = ghost_size(cutoff_radius_factor)
    n = [int(c) for c in cells]
    return (2 * (n[0] + 2 * g), n[1] + 2 * g, n[2] + 2 * g, 2 * g, g, g)


def local_slot_indices(cells, cutoff_radius_factor) -> np.ndarray:
    """Linear slot indices of the local sites in k, j, i scan order."""
    Sx, Sy, Sz, gx, gy, gz = grid(cells, cutoff_radius_factor)
    bx, by, bz = 2 * int(cells[0]), int(cells[1]), int(cells[2])
    k, j, i = np.meshgrid(np.arange(bz), np.arange(by), np.arange(bx), indexing="ij")
    return (((k + gz) * Sy + (j + gy)) * Sx + (i + gx)).reshape(-1)


@dataclass
class Workload:
    name: str
    cells: tuple
    lattice_const: float = 2.855
    cutoff: float = 5.6
    n_ele: int = 1
    cu_frac: float = 0.0
    ni_frac: float = 0.0
    temperature: float = 600.0
    dt: float = 0.001
    steps: int = 100
    seed: int = 1234
    pka_ev: float = 0.0          # cascades: PKA energy at the central site, direction from the seed

    @property
    def cutoff_radius_factor(self) -> float:
        return self.cutoff / self.lattice_const

    @property
    def n_atoms(self) -> int:
        return 2 * self.cells[0] * self.cells[1] * self.cells[2]


# Variable timestep of the cascade workloads: at most 0.01 A per step, 0.01 - 1 fs (Angstrom, ps).
CASCADE_DX_MAX, CASCADE_DT_MIN, CASCADE_DT_MAX = 0.01, 1e-5, 1e-3

# The single-box workloads of the benchmark set (sizes, compositions, temperatures, steps).
WORKLOADS = {
    "fe_20c": Workload("fe_20c", (20, 20, 20), temperature=600.0, steps=100),
    "fe_100c": Workload("fe_100c", (100, 100, 100), temperature=600.0, steps=1000),
    "fecuni_200c": Workload("fecuni_200c", (200, 200, 200), n_ele=3, cu_frac=0.015, ni_frac=0.010,
                            temperature=600.0, steps=500),
    "fe_100c_cascade": Workload("fe_100c_cascade", (100, 100, 100), temperature=300.0, steps=2000,
                                pka_ev=5000.0),
}


@dataclass
class CascadeSet:
    """Independent cascade replicas: cubic boxes with edges drawn uniformly from [cells_lo, cells_hi]
    unit cells, the Fe-Cu-Ni composition, PKA energies uniform in [energy_lo, energy_hi] eV with
    random directions, each replica on its own variable timestep."""
    name: str = "fecuni_cascades_64"
    replicas: int = 64
    cells_lo: int = 40
    cells_hi: int = 80
    energy_lo: float = 1000.0
    energy_hi: float = 10000.0
    temperature: float = 300.0
    steps: int = 1500
    n_ele: int = 3
    cu_frac: float = 0.015
    ni_frac: float = 0.010
    lattice_const: float = 2.855
    cutoff: float = 5.6
    seed: int = 4321

    @property
    def cutoff_radius_factor(self) -> float:
        return self.cutoff / self.lattice_const

    def replica_specs(self):
        """Per replica: cells, PKA lattice site [x, y, z, basis], direction, energy (eV), state seed."""
        rng = np.random.default_rng(self.seed)
        out = []
        for r in range(self.replicas):
            n = int(rng.integers(self.cells_lo, self.cells_hi + 1))
            e = float(rng.uniform(self.energy_lo, self.energy_hi))
            d = rng.standard_normal(3)
            out.append({"cells": (n, n, n), "lat": [n // 2, n // 2, n // 2, 0], "dir": d / np.linalg.norm(d),
                        "energy": e, "seed": self.seed + 1 + r})
        return out

    def potential_workload(self) -> "Workload":
        return Workload(self.name, (self.cells_lo,) * 3, lattice_const=self.lattice_const, cutoff=self.cutoff,
                        n_ele=self.n_ele, cu_frac=self.cu_frac, ni_frac=self.ni_frac,
                        temperature=self.temperature, seed=1234)


CASCADE_SETS = {"fecuni_cascades_64": CascadeSet()}


def build_state(cells, lattice_const, cutoff_radius_factor, *, temperature=600.0, seed=1234,
                cu_frac=0.0, ni_frac=0.0) -> np.ndarray:
    """Slot array (ghost-extended grid, reference index order) of a perfect BCC crystal at temperature."""
    Sx, Sy, Sz, gx, gy, gz = grid(cells, cutoff_radius_factor)
    atoms = np.zeros(Sx * Sy * Sz, dtype=ATOM_DTYPE)
    atoms["type"] = INVALID
    bx, by, bz = 2 * int(cells[0]), int(cells[1]), int(cells[2])
    n = bx * by * bz
    k, j, i = np.meshgrid(np.arange(bz, dtype=np.int64), np.arange(by, dtype=np.int64),
                          np.arange(bx, dtype=np.int64), indexing="ij")
    k = k.reshape(-1); j = j.reshape(-1); i = i.reshape(-1)
    slots = ((k + gz) * Sy + (j + gy)) * Sx + (i + gx)
    a0 = float(lattice_const)
    half = (i % 2) * (a0 / 2)
    pos = np.empty((n, 3))
    pos[:, 0] = (i * 0.5) * a0           # (x_low + i) * 0.5 * a0, x_low = 0 on one rank
    pos[:, 1] = j * a0 + half            # (y_low + j) * a0 + (i % 2) * (a0 / 2)
    pos[:, 2] = k * a0 + half
    rng = np.random.default_rng(seed)
    types = np.zeros(n, dtype=np.int32)
    n_cu = int(round(cu_frac * n))
    n_ni = int(round(ni_frac * n))
    if n_cu or n_ni:
        perm = rng.permutation(n)
        types[perm[:n_cu]] = 1
        types[perm[n_cu:n_cu + n_ni]] = 2
    mass = np.asarray(MASS)[types]
    sigma = np.sqrt(BOLTZ * temperature / (mass * MVV2E)) if temperature > 0 else np.zeros(n)
    vel = rng.standard_normal((n, 3)) * sigma[:, None]
    # WorldBuilder::zeroMomentum: v_i -= (sum m v / N) / m_i
    vcm = (vel * mass[:, None]).sum(axis=0) / n
    vel -= vcm[None, :] / mass[:, None]
    if temperature > 0:
        mvv = float((mass * (vel * vel).sum(axis=1)).sum())
        t_now = mvv * MVV2E / ((3 * n - 3) * BOLTZ)
        vel *= math.sqrt(temperature / t_now)
    atoms["id"][slots] = np.arange(1, n + 1, dtype=np.uint64)
    atoms["type"][slots] = types
    atoms["x"][slots] = pos
    atoms["v"][slots] = vel
    return atoms


def workload_state(w: Workload, seed=None) -> np.ndarray:
    return build_state(w.cells, w.lattice_const, w.cutoff_radius_factor, temperature=w.temperature,
                       seed=w.seed if seed is None else seed, cu_frac=w.cu_frac, ni_frac=w.ni_frac)


def workload_potential(w: Workload, directory: str) -> str:
    spec = PotentialSpec(n_ele=w.n_ele, seed=w.seed, cutoff=w.cutoff, lattice_const=w.lattice_const)
    path = os.path.join(directory, f"synthetic_{w.n_ele}ele_seed{w.seed}.setfl")
    if not os.path.exists(path):
        write_setfl(path, spec)
    return path


def pka_direction(seed: int) -> np.ndarray:
    """Random unit direction from the seed (cascade workloads)."""
    rng = np.random.default_rng(seed + 7919)
    d = rng.standard_normal(3)
    return d / np.linalg.norm(d)
