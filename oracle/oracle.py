"""TEST INFRASTRUCTURE - NOT PART OF THE PRODUCT.

ctypes binding of the CPU oracle (oracle/misa_oracle.cpp), the single-rank restatement of MISA-MD's
EAM hot path. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, as the
checker or the timed CPU baseline; the product never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
# the same source built with the compiler's default FP contraction, for the timed CPU baseline only
TIMED_LIB_PATH = os.path.join(HERE, "_build", "liboracle_timed.so")

ATOM_DTYPE = np.dtype(
    [("id", "<u8"), ("type", "<i4"), ("pad_", "<i4"), ("x", "<f8", (3,)), ("v", "<f8", (3,)),
     ("f", "<f8", (3,)), ("rho", "<f8"), ("df", "<f8")],
    align=True,
)


# AtomInfoDump / the record tools/dump2text/out_convert.cpp:18-25 reads: 72 bytes on LP64
DUMP_DTYPE = np.dtype(
    [("id", "<u8"), ("step", "<u8"), ("type", "<i4"), ("inter_type", "<i2"), ("pad_", "<i2"),
     ("x", "<f8", (3,)), ("v", "<f8", (3,))],
    align=True,
)
DUMP_HEADER = 128        # HEADER_SIZE (out_convert.cpp:5)
DUMP_RANK_HEADER = 128   # _LOCAL_HEADER_SIZE (out_convert.cpp:6)
DUMP_BLOCK = 1024 * 72   # BLOCK_SIZE (out_convert.cpp:30): LocalStorage's block, 1024 records


def write_dump_file(path, records):
    """The copy-mode file of one rank (AtomDump::dump + writeDumpHeader, frontend/io/atom_dump.cpp:38-82,
    through kiwi::LocalStorage): file header, rank header {size_t atoms_count}, then the records. With
    one rank LocalStorage's blocks are consecutive, so the records are contiguous. The file header is
    kiwi's and unread by any reader; it is written as zeros."""
    records = np.ascontiguousarray(records, dtype=DUMP_DTYPE)
    head = np.zeros(DUMP_HEADER + DUMP_RANK_HEADER, dtype=np.uint8)
    head[DUMP_HEADER:DUMP_HEADER + 8] = np.frombuffer(np.uint64(records.size).tobytes(), dtype=np.uint8)
    with open(path, "wb") as f:
        f.write(head.tobytes())
        f.write(records.tobytes())


def read_dump_file(path, n_ranks=1):
    """dump2text's reader (tools/dump2text/out_convert.cpp:66-98, readBytes :129-163) restated: for each
    rank, its count from the rank header, then its records from its blocks, which LocalStorage
    interleaves round-robin over the ranks. Returns one record array per rank."""
    data = np.fromfile(path, dtype=np.uint8)
    h = DUMP_HEADER + DUMP_RANK_HEADER * n_ranks
    out = []
    for rank in range(n_ranks):
        at = DUMP_HEADER + DUMP_RANK_HEADER * rank
        count = int(np.frombuffer(data[at:at + 8].tobytes(), dtype=np.uint64)[0])
        want = count * DUMP_DTYPE.itemsize
        parts, k = [], 0
        while want > 0:  # block k of this rank starts at h + (n_ranks * k + rank) * BLOCK
            lo = h + (n_ranks * k + rank) * DUMP_BLOCK
            take = min(DUMP_BLOCK, want)
            parts.append(data[lo:lo + take])
            want -= take
            k += 1
        raw = np.concatenate(parts) if parts else np.zeros(0, dtype=np.uint8)
        if raw.size != count * DUMP_DTYPE.itemsize:
            raise ValueError(f"{path}: truncated (rank {rank}: {raw.size} bytes for {count} records)")
        out.append(np.frombuffer(raw.tobytes(), dtype=DUMP_DTYPE))
    return out


class DomainDesc(ctypes.Structure):
    _fields_ = [("phase_space", ctypes.c_int64 * 3), ("lattice_const", ctypes.c_double),
                ("cutoff_radius_factor", ctypes.c_double), ("grid_size", ctypes.c_int32 * 3),
                ("grid_coord", ctypes.c_int32 * 3), ("ghost_size", ctypes.c_int32)]


def build(force=False, timed=False):
    path = TIMED_LIB_PATH if timed else LIB_PATH
    src = os.path.join(HERE, "misa_oracle.cpp")
    if force or not os.path.exists(path) or os.path.getmtime(src) > os.path.getmtime(path) or \
            os.path.getmtime(os.path.join(HERE, "misa_oracle.h")) > os.path.getmtime(path):
        target = os.path.relpath(path, HERE)
        subprocess.run(["make", "-s", "-C", HERE] + (["-B"] if force else []) + [target], check=True)
    return path


def use_timed_build():
    """Make this process load the timed build (the CPU baseline's workers call it before lib())."""
    global LIB_PATH
    if _LIB is not None:
        raise RuntimeError("the oracle library is already loaded")
    LIB_PATH = TIMED_LIB_PATH


_LIB = None
_P, _I32, _I64, _U64, _D = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_uint64, ctypes.c_double
_PROTOS = {
    "orc_ws_near_lat_sub_box_coord": (None, [_P, _P, _P]),
    "orc_ws_near_lat_coord": (None, [_P, _P, _P]),
    "orc_ws_is_out_box": (ctypes.c_uint32, [_P, _P]),
    "orc_ws_find_near_lat_index_in_sub_box": (_I64, [_P, _P]),
    "orc_ws_batch": (None, [_P, _P, _I64, _P, _P, _P, _P]),
    "orc_nei_offsets": (_I32, [_I64, _I64, _I64, _I32, _D, _I32, _P, _I32]),
    "orc_is_positive_index": (_I32, [_D, _D, _D]),
    "orc_create": (_P, [_P, _D, _D, ctypes.c_char_p, _D]),
    "orc_destroy": (None, [_P]),
    "orc_last_error": (ctypes.c_char_p, []),
    "orc_grid": (None, [_P, _P]),
    "orc_n_slots": (_I64, [_P]),
    "orc_set_atoms": (None, [_P, _P, _I64]),
    "orc_get_atoms": (None, [_P, _P, _I64]),
    "orc_get_inter": (_I64, [_P, _P, _I64]),
    "orc_get_ghost_inter": (_I64, [_P, _P, _I64]),
    "orc_set_inter": (None, [_P, _P, _I64]),
    "orc_set_timestep": (None, [_P, _D]),
    "orc_set_variable_timestep": (None, [_P, _D, _D, _D]),
    "orc_max_speed2": (_D, [_P]),
    "orc_dt_history": (_I64, [_P, _P, _I64]),
    "orc_time": (_D, [_P]),
    "orc_firststep": (None, [_P]),
    "orc_decide": (_I32, [_P]),
    "orc_exchange_inter": (None, [_P]),
    "orc_border_inter": (None, [_P]),
    "orc_exchange_atom_first": (None, [_P]),
    "orc_exchange_atom": (None, [_P]),
    "orc_clear_force": (None, [_P]),
    "orc_compute_eam": (None, [_P]),
    "orc_secondstep": (None, [_P]),
    "orc_prepare": (None, [_P]),
    "orc_simulate": (None, [_P, _I64]),
    "orc_collision_step": (None, [_P, _P, _P, _D]),
    "orc_setv": (None, [_P, _P, _P, _D]),
    "orc_world_build": (_I32, [_P, _D, ctypes.c_uint32, _P, _I32]),
    "orc_dump_records": (_I64, [_P, _U64, _P, _I64]),
    "orc_mvv": (_D, [_P]),
    "orc_kinetic_energy": (_D, [_P]),
    "orc_temperature": (_D, [_P, _U64]),
    "orc_rescale": (None, [_P, _D, _U64]),
    "orc_system_force": (None, [_P, _P]),
    "orc_potential_energy": (_D, [_P, _P, _P, _I64]),
    "orc_pot_charge_density": (_D, [_P, _I32, _D]),
    "orc_pot_d_embed": (_D, [_P, _I32, _D]),
    "orc_pot_embed": (_D, [_P, _I32, _D]),
    "orc_pot_to_force": (_D, [_P, _I32, _I32, _D, _D, _D]),
    "orc_pot_pair": (_D, [_P, _I32, _I32, _D]),
    "orc_pot_spline": (_I32, [_P, _I32, _I32, _I32, _P, _I32]),
    "orc_time_simulate": (_D, [_P, _I64]),
}


def lib():
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _PROTOS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _LIB = L
    return _LIB


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def domain_desc(phase_space, lattice_const, cutoff_radius_factor, grid_size=(1, 1, 1), grid_coord=(0, 0, 0),
                ghost_size=0):
    d = DomainDesc()
    for i in range(3):
        d.phase_space[i] = int(phase_space[i])
        d.grid_size[i] = int(grid_size[i])
        d.grid_coord[i] = int(grid_coord[i])
    d.lattice_const = float(lattice_const)
    d.cutoff_radius_factor = float(cutoff_radius_factor)
    d.ghost_size = int(ghost_size)
    return d


def ws_near_lat_sub_box_coord(desc, x):
    out = np.zeros(3, dtype=np.int64)
    xx = np.asarray(x, dtype=np.float64)
    lib().orc_ws_near_lat_sub_box_coord(ctypes.byref(desc), _ptr(xx), _ptr(out))
    return out


def ws_near_lat_coord(desc, x):
    out = np.zeros(3, dtype=np.int64)
    xx = np.asarray(x, dtype=np.float64)
    lib().orc_ws_near_lat_coord(ctypes.byref(desc), _ptr(xx), _ptr(out))
    return out


def ws_is_out_box(desc, x):
    xx = np.asarray(x, dtype=np.float64)
    return int(lib().orc_ws_is_out_box(ctypes.byref(desc), _ptr(xx)))


def ws_find_near_lat_index_in_sub_box(desc, x):
    xx = np.asarray(x, dtype=np.float64)
    return int(lib().orc_ws_find_near_lat_index_in_sub_box(ctypes.byref(desc), _ptr(xx)))


def ws_batch(desc, xyz):
    """Vectorised Wigner-Seitz mapping: (ext_coords, sub_coords, flags, index)."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    n = xyz.shape[0]
    ext = np.zeros((n, 3), dtype=np.int64)
    sub = np.zeros((n, 3), dtype=np.int64)
    flags = np.zeros(n, dtype=np.uint32)
    index = np.zeros(n, dtype=np.int64)
    lib().orc_ws_batch(ctypes.byref(desc), _ptr(xyz), n, _ptr(ext), _ptr(sub), _ptr(flags), _ptr(index))
    return ext, sub, flags, index


def nei_offsets(size_x, size_y, size_z, cut_lattice, cutoff_radius_factor, which):
    n = lib().orc_nei_offsets(size_x, size_y, size_z, cut_lattice, cutoff_radius_factor, which, None, 0)
    out = np.zeros(n, dtype=np.int64)
    lib().orc_nei_offsets(size_x, size_y, size_z, cut_lattice, cutoff_radius_factor, which, _ptr(out), n)
    return out


def is_positive_index(x, y, z):
    return bool(lib().orc_is_positive_index(x, y, z))


class OracleSim:
    """Single-rank CPU restatement of the reference's simulation state."""

    def __init__(self, cells, lattice_const, cutoff_radius_factor, setfl_path, dt=0.001):
        L = lib()
        ps = np.asarray(cells, dtype=np.int64)
        self.h = L.orc_create(_ptr(ps), float(lattice_const), float(cutoff_radius_factor),
                              os.fsencode(setfl_path), float(dt))
        if not self.h:
            raise RuntimeError("oracle: " + L.orc_last_error().decode())
        g = np.zeros(6, dtype=np.int64)
        L.orc_grid(self.h, _ptr(g))
        self.grid = tuple(int(v) for v in g)
        self.n_slots = int(L.orc_n_slots(self.h))
        self.L = L

    def close(self):
        if self.h:
            self.L.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_atoms(self, atoms):
        atoms = np.ascontiguousarray(atoms, dtype=ATOM_DTYPE)
        assert atoms.size == self.n_slots
        self.L.orc_set_atoms(self.h, _ptr(atoms), atoms.size)

    def get_atoms(self):
        out = np.zeros(self.n_slots, dtype=ATOM_DTYPE)
        self.L.orc_get_atoms(self.h, _ptr(out), out.size)
        return out

    def get_inter(self):
        n = self.L.orc_get_inter(self.h, None, 0)
        out = np.zeros(n, dtype=ATOM_DTYPE)
        if n:
            self.L.orc_get_inter(self.h, _ptr(out), n)
        return out

    def get_ghost_inter(self):
        n = self.L.orc_get_ghost_inter(self.h, None, 0)
        out = np.zeros(n, dtype=ATOM_DTYPE)
        if n:
            self.L.orc_get_ghost_inter(self.h, _ptr(out), n)
        return out

    def set_inter(self, inter):
        inter = np.ascontiguousarray(inter, dtype=ATOM_DTYPE)
        self.L.orc_set_inter(self.h, _ptr(inter) if inter.size else None, inter.size)

    def set_timestep(self, dt):
        self.L.orc_set_timestep(self.h, float(dt))

    def set_variable_timestep(self, dx_max, dt_min, dt_max):
        self.L.orc_set_variable_timestep(self.h, float(dx_max), float(dt_min), float(dt_max))

    def dt_history(self):
        n = self.L.orc_dt_history(self.h, None, 0)
        out = np.zeros(n)
        if n:
            self.L.orc_dt_history(self.h, _ptr(out), n)
        return out

    def __getattr__(self, name):
        # thin pass-through for the step pieces: firststep, decide, exchange_inter, ...
        fn = getattr(lib(), "orc_" + name, None)
        if fn is None or name.startswith("_"):
            raise AttributeError(name)
        return lambda *a: fn(self.h, *a)

    def collision_step(self, lat, direction, energy):
        lat = np.asarray(lat, dtype=np.int32)
        d = np.asarray(direction, dtype=np.float64)
        self.L.orc_collision_step(self.h, _ptr(lat), _ptr(d), float(energy))

    def setv(self, lat, direction, energy):
        lat = np.asarray(lat, dtype=np.int32)
        d = np.asarray(direction, dtype=np.float64)
        self.L.orc_setv(self.h, _ptr(lat), _ptr(d), float(energy))

    def world_build(self, t_set, seed, ratio=(1, 0, 0), rng=0):
        r = np.asarray(ratio, dtype=np.int32)
        if self.L.orc_world_build(self.h, float(t_set), int(seed), _ptr(r), int(rng)) != 0:
            raise ValueError("unknown random engine")

    def dump_records(self, time_step):
        n = self.L.orc_dump_records(self.h, int(time_step), None, 0)
        out = np.zeros(n, dtype=DUMP_DTYPE)
        if n:
            self.L.orc_dump_records(self.h, int(time_step), _ptr(out), n)
        return out

    def system_force(self):
        out = np.zeros(3)
        self.L.orc_system_force(self.h, _ptr(out))
        return out

    def potential_energy(self, per_slot=False, inter_cap=0):
        e = np.zeros(self.n_slots) if per_slot else None
        ei = np.zeros(inter_cap) if inter_cap else None
        total = self.L.orc_potential_energy(self.h, _ptr(e), _ptr(ei), inter_cap)
        return total, e, ei

    def pot_spline(self, kind, e1, e2=0):
        n = self.L.orc_pot_spline(self.h, kind, e1, e2, None, 0)
        out = np.zeros(7 * n)
        self.L.orc_pot_spline(self.h, kind, e1, e2, _ptr(out), out.size)
        return out.reshape(n, 7)
