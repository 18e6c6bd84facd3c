"""misa_md_gb300: GB300-native EAM step for MISA-MD's lattice-indexed atom store.

Python plumbing over the C ABI of libmisa_gb300.so (include/misa_gb300.h): ctypes bindings, a
``Context`` per GPU state, and ``Simulation``, which mirrors the reference's ``simulation`` class
(src/simulation.h: createDomain, createAtoms, prepareForStart, simulate, collisionStep) so callers of
the reference's API find the same call order. All compute runs in the CUDA library; there is no CPU
fallback: loading fails loudly when the library is missing.
"""
from __future__ import annotations

import ctypes
import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _load_sibling(name):
    mod_name = f"misa_md_gb300.{name}"
    if mod_name in sys.modules:
        return sys.modules[mod_name]
    spec = importlib.util.spec_from_file_location(mod_name, os.path.join(HERE, f"{name}.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules[mod_name] = mod
    spec.loader.exec_module(mod)
    return mod


workloads = _load_sibling("workloads")
build = _load_sibling("build")
dumpfile = _load_sibling("dumpfile")
ATOM_DTYPE = workloads.ATOM_DTYPE

PREC = {"fp64": 0, "mixed": 1}
STATUS = {0: "MG_OK", 1: "MG_ERR_ARG", 2: "MG_ERR_CUDA", 3: "MG_ERR_POTENTIAL", 4: "MG_ERR_CAPACITY",
          5: "MG_ERR_OUT_OF_GRID", 6: "MG_ERR_STATE"}


class MgError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class ThermoOut(ctypes.Structure):
    _fields_ = [("mvv", ctypes.c_double), ("kinetic_energy", ctypes.c_double),
                ("potential_energy", ctypes.c_double), ("force_sum", ctypes.c_double * 3),
                ("n_inter", ctypes.c_int64), ("n_ghost_inter", ctypes.c_int64), ("n_vacancy", ctypes.c_int64),
                ("device_errors", ctypes.c_uint32), ("pad_", ctypes.c_uint32)]


class StageIn(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int64), ("step_length", ctypes.c_double), ("collision_set", ctypes.c_int32),
                ("rescales_set", ctypes.c_int32), ("collision_step", ctypes.c_int64),
                ("collision_lat", ctypes.c_int32 * 4), ("direction", ctypes.c_double * 3),
                ("pka_energy", ctypes.c_double), ("rescale_t", ctypes.c_double), ("rescale_every", ctypes.c_int64)]


class ThermoSample(ctypes.Structure):
    _fields_ = [("step", ctypes.c_int64), ("time_ps", ctypes.c_double), ("mvv", ctypes.c_double),
                ("temperature", ctypes.c_double)]


_LIB = None
_P = ctypes.c_void_p
_I32, _I64, _U64, _D = ctypes.c_int32, ctypes.c_int64, ctypes.c_uint64, ctypes.c_double

_PROTOS = {
    "mg_env_init": (_I32, [_I32]),
    "mg_env_clean": (_I32, []),
    "mg_create": (_I32, [_P, _D, _D, _I32, _I64, _P]),
    "mg_destroy": (_I32, [_P]),
    "mg_last_error": (ctypes.c_char_p, [_P]),
    "mg_grid": (_I32, [_P, _P]),
    "mg_set_precision": (_I32, [_P, _I32]),
    "mg_nei_offset_init": (_I32, [_P, _P, _P, _I32, _P, _P, _I32]),
    "mg_nei_offsets": (_I32, [_P, _I32, _P, _I32, _P]),
    "mg_pot_init_setfl": (_I32, [_P, ctypes.c_char_p]),
    "mg_pot_init_tables": (_I32, [_P, _I32, _P, _I32, _D, _I32, _D, _D, _P, _P, _P]),
    "mg_pot_spline": (_I32, [_P, _I32, _I32, _I32, _P, _I32, _P]),
    "mg_eam_rho_calc": (_I32, [_P, _P, _D]),
    "mg_eam_df_calc": (_I32, [_P, _P, _D]),
    "mg_eam_force_calc": (_I32, [_P, _P, _D]),
    "mg_upload": (_I32, [_P, _P, _I64, _P, _I64]),
    "mg_download": (_I32, [_P, _P, _I64, _P, _I64, _P]),
    "mg_download_ghost_inter": (_I32, [_P, _P, _I64, _P]),
    "mg_set_timestep": (_I32, [_P, _D]),
    "mg_set_variable_timestep": (_I32, [_P, _D, _D, _D]),
    "mg_clock": (_I32, [_P, _P, _P, _P]),
    "mg_dt_history": (_I32, [_P, _P, _I64, _P]),
    "mg_prepare": (_I32, [_P]),
    "mg_simulate": (_I32, [_P, _I64, _I32]),
    "mg_phase": (_I32, [_P, _I32]),
    "mg_collision_step": (_I32, [_P, _P, _P, _D]),
    "mg_rescale": (_I32, [_P, _D, _U64]),
    "mg_thermo": (_I32, [_P, _I32, _P]),
    "mg_download_energies": (_I32, [_P, _P, _I64, _P, _I64]),
    "mg_clear_errors": (_I32, [_P]),
    "mg_step_host": (_I32, [_P, _P, _I64, _P, _I64, _P, _I64]),
    "mg_ws_map": (_I32, [_P, _P, _I64, _P, _P, _P]),
    "mg_enable_timing": (_I32, [_P, _I32]),
    "mg_kernel_times": (_I32, [_P, _P, _I32, _P, _P]),
    "mg_launches_per_step": (_I32, [_P, _P]),
    "mg_stream": (_P, [_P]),
    "mg_world_build": (_I32, [_P, _D, _D, _D, ctypes.c_uint32, _P, _I32, _P, _I64]),
    "mg_run_stages": (_I32, [_P, _P, _I32, _I64, _D, _I64, _I32, _P, _I64, _P]),
    "mg_batch_create": (_I32, [_P, _I32, _I32, _P]),
    "mg_batch_run": (_I32, [_P, _I64, _I32]),
    "mg_batch_launches_per_step": (_I32, [_P, _P]),
    "mg_batch_stream": (_P, [_P]),
    "mg_batch_last_error": (ctypes.c_char_p, [_P]),
    "mg_batch_destroy": (_I32, [_P]),
    "mg_host_register": (_I32, [_P, _U64]),
    "mg_host_unregister": (_I32, [_P]),
    "mg_mvv_noalloc": (_I32, [_P, _P, _P, _P, _I64, _P, _P]),
    "mg_probe_fma": (_I32, [_I32, _P]),
    "mg_autotune": (_I32, [_P, _I32, _P]),
    "mg_set_tuning": (_I32, [_P, _P]),
    "mg_dump_open": (_I32, [_P, ctypes.c_char_p, _I32, _I64, _P]),
    "mg_dump_frame": (_I32, [_P, _U64]),
    "mg_dump_close": (_I32, [_P, _P]),
    "mg_dump_last_error": (ctypes.c_char_p, [_P]),
    "mg_set_stage_output": (_I32, [_P, _P, _U64, ctypes.c_char_p]),
    "mg_set_host_pipeline": (_I32, [_P, _I32]),
    "mg_set_step_fusion": (_I32, [_P, _I32]),
    "mg_set_neighbour_skin": (_I32, [_P, ctypes.c_double]),
    "mg_skin_stats": (_I32, [_P, _P, _P]),
}


def library_path() -> str:
    return build.LIB_PATH


def load_library(build_if_missing: bool = False) -> ctypes.CDLL:
    """Load libmisa_gb300.so; raises if it is not built (no fallback path exists)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = build.LIB_PATH
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"libmisa_gb300.so is not built ({path}); run __graft_entry__.build()")
        build.build()
    lib = ctypes.CDLL(path)
    for name, (res, args) in _PROTOS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def exported_symbols():
    return list(_PROTOS)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


RNG = {"mt": 0, "lcg": 1, "stc": 2, "legacy": 3}


def world_build(cells, lattice_const, cutoff_radius_factor, t_set, seed, alloy_ratio=(1, 0, 0), rng="mt"):
    """The reference's creation mode (WorldBuilder::build): returns the host slot array of the
    ghost-extended grid, equal to the reference's for the same seed, alloy ratio and MD_RAND engine."""
    lib = load_library()
    Sx, Sy, Sz, _, _, _ = workloads.grid(cells, cutoff_radius_factor)
    atoms = np.zeros(Sx * Sy * Sz, dtype=ATOM_DTYPE)
    ps = np.asarray(cells, dtype=np.int64)
    ratio = np.asarray(alloy_ratio, dtype=np.int32)
    st = lib.mg_world_build(_ptr(ps), float(lattice_const), float(cutoff_radius_factor), float(t_set), int(seed),
                            _ptr(ratio), RNG[rng], _ptr(atoms), atoms.size)
    if st != 0:
        raise MgError(st, (lib.mg_last_error(None) or b"").decode())
    return atoms


def probe_fma(kind):
    """FMA throughput of the current device in FLOP/s: kind 0 FP64, 1 FP32, 2 packed FP32x2 (mg_probe_fma)."""
    lib = load_library()
    out = ctypes.c_double()
    st = lib.mg_probe_fma(int(kind), ctypes.byref(out))
    if st != 0:
        raise MgError(st, (lib.mg_last_error(None) or b"").decode())
    return out.value


def host_register(array):
    """Page-lock a numpy array's memory for DMA copies (mg_host_register)."""
    lib = load_library()
    st = lib.mg_host_register(array.ctypes.data_as(ctypes.c_void_p), array.nbytes)
    if st != 0:
        raise MgError(st, (lib.mg_last_error(None) or b"").decode())


def host_unregister(array):
    lib = load_library()
    st = lib.mg_host_unregister(array.ctypes.data_as(ctypes.c_void_p))
    if st != 0:
        raise MgError(st, (lib.mg_last_error(None) or b"").decode())


class Context:
    """One GPU state (mg_context): the ghost-extended slot grid of a periodic BCC box."""

    def __init__(self, cells, lattice_const, cutoff_radius_factor, precision="fp64", inter_capacity=0,
                 device=0):
        self.lib = load_library()
        self.cells = tuple(int(c) for c in cells)
        self.lattice_const = float(lattice_const)
        self.cutoff_radius_factor = float(cutoff_radius_factor)
        self.precision = precision
        self._check(self.lib.mg_env_init(device), None)
        h = ctypes.c_void_p()
        ps = np.asarray(self.cells, dtype=np.int64)
        st = self.lib.mg_create(_ptr(ps), self.lattice_const, self.cutoff_radius_factor, PREC[precision],
                                int(inter_capacity), ctypes.byref(h))
        self._check(st, None)
        self.h = h
        g = np.zeros(6, dtype=np.int64)
        self._check(self.lib.mg_grid(self.h, _ptr(g)))
        self.grid = tuple(int(v) for v in g)
        self.n_slots = int(g[0] * g[1] * g[2])

    # ---- plumbing ----
    def _check(self, status, h="self"):
        if status != 0:
            handle = self.h if h == "self" else None
            msg = self.lib.mg_last_error(handle)
            raise MgError(status, msg.decode() if msg else "")

    def close(self):
        if getattr(self, "h", None):
            self.lib.mg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def cutoff_radius(self):
        return self.lattice_const * self.cutoff_radius_factor

    # ---- setup ----
    def pot_init_setfl(self, path):
        self._check(self.lib.mg_pot_init_setfl(self.h, os.fsencode(path)))

    def pot_spline(self, kind, e1, e2=0):
        n = ctypes.c_int32()
        self._check(self.lib.mg_pot_spline(self.h, kind, e1, e2, None, 0, ctypes.byref(n)))
        out = np.zeros(7 * n.value)
        self._check(self.lib.mg_pot_spline(self.h, kind, e1, e2, _ptr(out), out.size, ctypes.byref(n)))
        return out.reshape(n.value, 7)

    def nei_offsets(self, which):
        n = ctypes.c_int32()
        self._check(self.lib.mg_nei_offsets(self.h, which, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value, dtype=np.int64)
        self._check(self.lib.mg_nei_offsets(self.h, which, _ptr(out), out.size, ctypes.byref(n)))
        return out

    def nei_offset_init(self, full_even, full_odd, half_even, half_odd):
        a = [np.ascontiguousarray(x, dtype=np.int64) for x in (full_even, full_odd, half_even, half_odd)]
        self._check(self.lib.mg_nei_offset_init(self.h, _ptr(a[0]), _ptr(a[1]), len(a[0]), _ptr(a[2]),
                                                _ptr(a[3]), len(a[2])))

    def set_timestep(self, dt):
        self._check(self.lib.mg_set_timestep(self.h, float(dt)))

    def set_variable_timestep(self, dx_max, dt_min, dt_max):
        """dt = clamp(dx_max / max|v|, dt_min, dt_max) before every step (Angstrom, ps)."""
        self._check(self.lib.mg_set_variable_timestep(self.h, float(dx_max), float(dt_min), float(dt_max)))

    def dump_open(self, path, by_frame=False, chunk_bytes=0):
        """An atom dump of this context in the reference's copy-mode layout (mg_dump_open)."""
        return Dump(self, path, by_frame, chunk_bytes)

    def set_stage_output(self, dump=None, interval=0, origin_path=None):
        """Dumps taken by run_stages: a frame into `dump` after every interval-th step, and the state
        before each collision into origin_path (mg_set_stage_output)."""
        self._check(self.lib.mg_set_stage_output(self.h, dump.h if dump is not None else None, int(interval),
                                                 os.fsencode(origin_path) if origin_path else None))

    def run_stages(self, stages, steps, default_dt, n_atoms, thermo_interval=0):
        """The reference's stage driver (MDSimulation::beforeStep / postStep) on the device. stages: dicts
        with steps, step_length, and optionally collision_step + lat + direction + energy and
        rescale_t + rescale_every. Returns the thermo samples as dicts. Dumps as set_stage_output set."""
        arr = (StageIn * max(1, len(stages)))()
        for k, st in enumerate(stages):
            a = arr[k]
            a.steps = int(st["steps"])
            a.step_length = float(st.get("step_length", 0.0))
            if "collision_step" in st:
                a.collision_set = 1
                a.collision_step = int(st["collision_step"])
                for i in range(4):
                    a.collision_lat[i] = int(st["lat"][i])
                for i in range(3):
                    a.direction[i] = float(st["direction"][i])
                a.pka_energy = float(st["energy"])
            if "rescale_t" in st:
                a.rescales_set = 1
                a.rescale_t = float(st["rescale_t"])
                a.rescale_every = int(st["rescale_every"])
        cap = steps // thermo_interval if thermo_interval else 0
        out = (ThermoSample * max(1, cap))()
        n = ctypes.c_int64(0)
        self._check(self.lib.mg_run_stages(self.h, arr, len(stages), int(steps), float(default_dt), int(n_atoms),
                                           int(thermo_interval), out, cap, ctypes.byref(n)))
        return [{"step": out[k].step, "time_ps": out[k].time_ps, "mvv": out[k].mvv,
                 "temperature": out[k].temperature} for k in range(n.value)]

    def clock(self):
        """(steps taken, simulated time in ps, dt of the last step)."""
        n = ctypes.c_int64(0)
        t = ctypes.c_double(0)
        d = ctypes.c_double(0)
        self._check(self.lib.mg_clock(self.h, ctypes.byref(n), ctypes.byref(t), ctypes.byref(d)))
        return n.value, t.value, d.value

    def dt_history(self, cap=65536):
        out = np.zeros(cap)
        n = ctypes.c_int64(0)
        self._check(self.lib.mg_dt_history(self.h, out.ctypes.data_as(ctypes.c_void_p), cap, ctypes.byref(n)))
        return out[: n.value].copy()

    def set_precision(self, precision):
        self._check(self.lib.mg_set_precision(self.h, PREC[precision]))
        self.precision = precision

    # ---- state ----
    def upload(self, atoms, inter=None):
        atoms = np.ascontiguousarray(atoms, dtype=ATOM_DTYPE)
        if atoms.size != self.n_slots:
            raise ValueError(f"slot array has {atoms.size} records, grid has {self.n_slots}")
        inter = np.zeros(0, dtype=ATOM_DTYPE) if inter is None else np.ascontiguousarray(inter, dtype=ATOM_DTYPE)
        self._check(self.lib.mg_upload(self.h, _ptr(atoms), atoms.size, _ptr(inter) if inter.size else None,
                                       inter.size))

    def download(self, inter_cap=None):
        atoms = np.zeros(self.n_slots, dtype=ATOM_DTYPE)
        n = ctypes.c_int64()
        self._check(self.lib.mg_download(self.h, _ptr(atoms), atoms.size, None, 0, ctypes.byref(n)))
        cap = n.value if inter_cap is None else inter_cap
        inter = np.zeros(cap, dtype=ATOM_DTYPE)
        if cap:
            self._check(self.lib.mg_download(self.h, _ptr(atoms), atoms.size, _ptr(inter), cap, ctypes.byref(n)))
        return atoms, inter[:min(cap, n.value)]

    def download_ghost_inter(self):
        n = ctypes.c_int64()
        self._check(self.lib.mg_download_ghost_inter(self.h, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value, dtype=ATOM_DTYPE)
        if n.value:
            self._check(self.lib.mg_download_ghost_inter(self.h, _ptr(out), n.value, ctypes.byref(n)))
        return out

    # ---- steps ----
    def prepare(self):
        self._check(self.lib.mg_prepare(self.h))

    def simulate(self, steps, sync=True):
        self._check(self.lib.mg_simulate(self.h, int(steps), 1 if sync else 0))

    def phase(self, k):
        self._check(self.lib.mg_phase(self.h, int(k)))

    def collision_step(self, lat, direction, energy):
        lat = np.asarray(lat, dtype=np.int32)
        d = np.asarray(direction, dtype=np.float64)
        self._check(self.lib.mg_collision_step(self.h, _ptr(lat), _ptr(d), float(energy)))

    def rescale(self, t_set, n_atoms):
        self._check(self.lib.mg_rescale(self.h, float(t_set), int(n_atoms)))

    def thermo(self, with_energy=False):
        out = ThermoOut()
        self._check(self.lib.mg_thermo(self.h, 1 if with_energy else 0, ctypes.byref(out)))
        return {"mvv": out.mvv, "kinetic_energy": out.kinetic_energy, "potential_energy": out.potential_energy,
                "force_sum": tuple(out.force_sum), "n_inter": out.n_inter, "n_ghost_inter": out.n_ghost_inter,
                "n_vacancy": out.n_vacancy, "device_errors": out.device_errors}

    def energies(self, inter_cap=0):
        per_slot = np.zeros(self.n_slots)
        per_inter = np.zeros(inter_cap)
        self._check(self.lib.mg_download_energies(self.h, _ptr(per_slot), per_slot.size,
                                                  _ptr(per_inter) if inter_cap else None, inter_cap))
        return per_slot, per_inter

    # ---- reference hooks ----
    def eam_rho_calc(self, atoms):
        self._check(self.lib.mg_eam_rho_calc(self.h, _ptr(atoms), self.cutoff_radius))

    def eam_df_calc(self, atoms):
        self._check(self.lib.mg_eam_df_calc(self.h, _ptr(atoms), self.cutoff_radius))

    def eam_force_calc(self, atoms):
        self._check(self.lib.mg_eam_force_calc(self.h, _ptr(atoms), self.cutoff_radius))

    def set_step_fusion(self, steps_per_graph):
        """Loop bodies per graph launch of simulate in the mixed form (fused firststep; 0 or 1: off)."""
        self._check(self.lib.mg_set_step_fusion(self.h, int(steps_per_graph)))

    def set_neighbour_skin(self, skin):
        """Verlet skin (Angstrom) of the mixed form's candidate lists (0: off); results do not depend on it."""
        self._check(self.lib.mg_set_neighbour_skin(self.h, float(skin)))

    def skin_stats(self):
        """(density passes that used the candidate lists, passes that rebuilt them)."""
        p, r = ctypes.c_int64(0), ctypes.c_int64(0)
        self._check(self.lib.mg_skin_stats(self.h, ctypes.byref(p), ctypes.byref(r)))
        return p.value, r.value

    def set_host_pipeline(self, chunks):
        """z-slabs of step_host's copy/compute pipeline (0 or 1: off)."""
        self._check(self.lib.mg_set_host_pipeline(self.h, int(chunks)))

    def step_host(self, atoms, inter, n_inter, nsteps):
        n = ctypes.c_int64(n_inter)
        self._check(self.lib.mg_step_host(self.h, _ptr(atoms), atoms.size, _ptr(inter), inter.size,
                                          ctypes.byref(n), int(nsteps)))
        return n.value

    # ---- utilities ----
    def ws_map(self, xyz):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        n = xyz.shape[0]
        coords = np.zeros((n, 3), dtype=np.int64)
        flags = np.zeros(n, dtype=np.uint32)
        index = np.zeros(n, dtype=np.int64)
        self._check(self.lib.mg_ws_map(self.h, _ptr(xyz), n, _ptr(coords), _ptr(flags), _ptr(index)))
        return coords, flags, index

    def autotune(self, reps=3):
        out = np.zeros(6, dtype=np.int32)
        self._check(self.lib.mg_autotune(self.h, int(reps), _ptr(out)))
        return {"rho_order": int(out[0]), "rho_block": int(out[1]), "rho_apt": int(out[2]),
                "force_order": int(out[3]), "force_block": int(out[4]), "force_apt": int(out[5])}

    def set_tuning(self, rho_order, rho_block, force_order, force_block, rho_apt=1, force_apt=1):
        t = np.asarray([rho_order, rho_block, rho_apt, force_order, force_block, force_apt], dtype=np.int32)
        self._check(self.lib.mg_set_tuning(self.h, _ptr(t)))

    def enable_timing(self, on=True):
        self._check(self.lib.mg_enable_timing(self.h, 1 if on else 0))

    def kernel_times(self):
        n = ctypes.c_int32()
        ms = np.zeros(32)
        names = (ctypes.c_char_p * 32)()
        self._check(self.lib.mg_kernel_times(self.h, _ptr(ms), 32, ctypes.byref(n), names))
        return {names[k].decode(): float(ms[k]) for k in range(n.value)}

    def launches_per_step(self):
        n = ctypes.c_int32()
        self._check(self.lib.mg_launches_per_step(self.h, ctypes.byref(n)))
        return n.value

    def stream(self):
        return self.lib.mg_stream(self.h)


class Dump:
    """Binary atom dump fed from the device (mg_dump_*): frames are packed on the GPU and written by a
    background thread. by_frame: path holds "{}" for the time step, one file per frame."""

    def __init__(self, ctx, path, by_frame=False, chunk_bytes=0):
        self.lib = ctx.lib
        self.ctx = ctx
        h = ctypes.c_void_p()
        st = self.lib.mg_dump_open(ctx.h, os.fsencode(path), 1 if by_frame else 0, int(chunk_bytes), ctypes.byref(h))
        if st != 0:
            raise MgError(st, f"cannot open dump {path}")
        self.h = h

    def frame(self, time_step):
        st = self.lib.mg_dump_frame(self.h, int(time_step))
        if st != 0:
            raise MgError(st, (self.lib.mg_dump_last_error(self.h) or b"").decode())

    def close(self):
        """Waits for every frame and writes the header; returns the records written."""
        if not getattr(self, "h", None):
            return None
        n = ctypes.c_uint64(0)
        h, self.h = self.h, None
        st = self.lib.mg_dump_close(h, ctypes.byref(n))
        if st != 0:
            raise MgError(st, (self.lib.mg_last_error(self.ctx.h) or b"").decode())
        return n.value

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Independent replicas advanced together by one CUDA graph (mg_batch_*). The contexts must be
    prepared and stay open while the batch exists."""

    def __init__(self, contexts, steps_per_launch=1):
        self.lib = load_library()
        self.contexts = list(contexts)
        arr = (ctypes.c_void_p * len(self.contexts))(*[c.h.value for c in self.contexts])
        h = ctypes.c_void_p()
        st = self.lib.mg_batch_create(arr, len(self.contexts), int(steps_per_launch), ctypes.byref(h))
        if st != 0:
            raise MgError(st, (self.lib.mg_batch_last_error(None) or b"").decode())
        self.h = h

    def run(self, steps, sync=True):
        st = self.lib.mg_batch_run(self.h, int(steps), 1 if sync else 0)
        if st != 0:
            raise MgError(st, (self.lib.mg_batch_last_error(self.h) or b"").decode())

    def launches_per_step(self):
        n = ctypes.c_int32()
        self.lib.mg_batch_launches_per_step(self.h, ctypes.byref(n))
        return n.value

    def stream(self):
        return self.lib.mg_batch_stream(self.h)

    def close(self):
        if getattr(self, "h", None):
            self.lib.mg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Simulation:
    """Mirror of the reference's simulation class (src/simulation.h), one GPU owning the whole box.

    createDomain -> create_domain, createAtoms -> create_atoms, prepareForStart -> prepare_for_start,
    simulate -> simulate, collisionStep -> collision_step. Errors raise MgError instead of MPI_Abort.
    """

    def __init__(self, precision="fp64", inter_capacity=0):
        self.precision = precision
        self.inter_capacity = inter_capacity
        self.ctx = None
        self.phase_space = None

    def create_domain(self, phase_space, lattice_const, cutoff_radius_factor):
        self.phase_space = tuple(int(v) for v in phase_space)
        self.lattice_const = float(lattice_const)
        self.cutoff_radius_factor = float(cutoff_radius_factor)
        self.ctx = Context(self.phase_space, lattice_const, cutoff_radius_factor, self.precision,
                           self.inter_capacity)

    def create_atoms(self, init_step_len, t_set, create_seed, alloy_ratio=(1.0, 0.0, 0.0), atoms=None,
                     builder="maxwell", rng="mt"):
        """Create-mode state unless a slot array is given. builder "worldbuilder" reproduces the
        reference's WorldBuilder::build bit for bit (integer alloy ratios, rng = the MD_RAND engine);
        "maxwell" draws Maxwell velocities and exact alloy counts from the seed."""
        if atoms is None and builder == "worldbuilder":
            atoms = world_build(self.phase_space, self.lattice_const, self.cutoff_radius_factor, t_set, create_seed,
                                tuple(int(r) for r in alloy_ratio), rng)
        if atoms is None:
            total = float(sum(alloy_ratio))
            atoms = workloads.build_state(self.phase_space, self.lattice_const, self.cutoff_radius_factor,
                                          temperature=t_set, seed=create_seed,
                                          cu_frac=alloy_ratio[1] / total, ni_frac=alloy_ratio[2] / total)
        self._atoms = atoms
        self.ctx.set_timestep(init_step_len)

    def prepare_for_start(self, pot_file_path):
        self.ctx.pot_init_setfl(pot_file_path)
        self.ctx.upload(self._atoms)
        self._atoms = None
        self.ctx.prepare()

    def simulate(self, steps):
        self.ctx.simulate(steps, sync=True)

    def run_stages(self, stages, steps, default_dt, thermo_interval=0, dump_path=None, dump_interval=0,
                   by_frame=False, origin_dump_path=None):
        """MDSimulation's run (frontend/md_simulation.cpp:24-111): the stage list on the device, atom
        frames every dump_interval steps into dump_path (OutputCopy; by_frame: one file per frame,
        "{}" in the path), the state before each PKA into origin_dump_path, and the dump header written
        at the end (onSimulationDone -> onAllOut). Returns the thermo samples."""
        n = 2 * self.phase_space[0] * self.phase_space[1] * self.phase_space[2]
        dump = self.ctx.dump_open(dump_path, by_frame=by_frame) if dump_path and dump_interval else None
        try:
            self.ctx.set_stage_output(dump, dump_interval if dump else 0, origin_dump_path)
            return self.ctx.run_stages(stages, steps, default_dt, n, thermo_interval)
        finally:
            self.ctx.set_stage_output()
            if dump is not None:
                dump.close()

    def collision_step(self, coll_lat, coll_dir, pka_energy):
        self.ctx.collision_step(coll_lat, coll_dir, pka_energy)

    def set_timestep_length(self, dt):
        self.ctx.set_timestep(dt)

    def kinetic_energy(self):
        return self.ctx.thermo()["kinetic_energy"]

    def temperature(self):
        n = 2 * self.phase_space[0] * self.phase_space[1] * self.phase_space[2]
        return self.ctx.thermo()["mvv"] * workloads.MVV2E / ((3 * n - 3) * workloads.BOLTZ)
