"""Python side of the GB300 kinetics module: ctypes bindings to
``libsimstack_gpu.so`` (the C ABI declared in ``include/simstack_gpu.h``) and a
host mirror of the reference's zone-block layout.

The compute path is the CUDA library; nothing here integrates anything on the
CPU. If the library is missing, :func:`lib` raises -- there is no fallback.

Reference interfaces mirrored here:
  - the GPU module's C ABI           src/gpu/gpu_api.h:30-115
  - the zone SoA block               src/sim/dbd.cpp:35-83 (DbdZones, dbd_zones_alloc)
  - the GPU advance call site        src/sim/dbd.cpp:272-295 (dbd_advance_gpu)
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libsimstack_gpu.so")

N_AVOGADRO_CM3 = 6.02214076e20      # mol/L -> molecules/cm^3
ATOL_1E12_MOLAR = 1e-12 * N_AVOGADRO_CM3
METHODS = {"ros2": 0, "ros3": 1, "rodas3": 2}
PRECISION = {"f64": 0, "f32": 1, "mixed": 2}

# --------------------------------------------------------------------------
# ABI records (layouts of include/simstack_gpu.h = the reference's).

KIN_MAX_SPECIES, KIN_MAX_REACTIONS, KIN_MAX_NNZ, KIN_MAX_LU_DIV, KIN_MAX_LU_SUB = 32, 96, 512, 512, 4096


class KinReaction(C.Structure):
    _fields_ = [("reactant", C.c_uint8 * 3), ("reactant_count", C.c_uint8), ("net_count", C.c_uint8),
                ("net_species", C.c_uint8 * 6), ("net_coef", C.c_int8 * 6), ("jac_index", (C.c_uint16 * 6) * 3)]


class KinLuDiv(C.Structure):
    _fields_ = [("ik", C.c_uint16), ("kk", C.c_uint16), ("sub_begin", C.c_uint16), ("sub_end", C.c_uint16)]


class KinLuSub(C.Structure):
    _fields_ = [("ij", C.c_uint16), ("kj", C.c_uint16)]


class KinRowEntry(C.Structure):
    _fields_ = [("index", C.c_uint16), ("col", C.c_uint8), ("pad", C.c_uint8)]


class KinMech(C.Structure):
    _fields_ = [("species_count", C.c_uint32), ("reaction_count", C.c_uint32),
                ("reactions", KinReaction * KIN_MAX_REACTIONS), ("nnz", C.c_uint32),
                ("diag", C.c_uint16 * KIN_MAX_SPECIES), ("lu_div_count", C.c_uint32), ("lu_sub_count", C.c_uint32),
                ("div_begin", C.c_uint16 * (KIN_MAX_SPECIES + 1)), ("lu_div", KinLuDiv * KIN_MAX_LU_DIV),
                ("lu_sub", KinLuSub * KIN_MAX_LU_SUB), ("lower_begin", C.c_uint16 * (KIN_MAX_SPECIES + 1)),
                ("upper_begin", C.c_uint16 * (KIN_MAX_SPECIES + 1)), ("lower", KinRowEntry * KIN_MAX_NNZ),
                ("upper", KinRowEntry * KIN_MAX_NNZ)]


class KinMethod(C.Structure):
    _fields_ = [("stages", C.c_uint32), ("order", C.c_uint32), ("a", C.c_double * 6), ("c", C.c_double * 6),
                ("m", C.c_double * 4), ("e", C.c_double * 4), ("gamma0", C.c_double), ("new_f", C.c_int32 * 4),
                ("name", C.c_char_p)]


class KinControl(C.Structure):
    _fields_ = [("rtol", C.c_double), ("atol", C.c_double), ("h_min", C.c_double), ("h_max", C.c_double),
                ("h_start", C.c_double), ("max_steps", C.c_uint32), ("fixed_step", C.c_int32),
                ("clamp_negative", C.c_int32)]


class GpuKinLaunch(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("y", "h", "steps", "rejects", "pulses", "failed", "k", "src", "pulse",
                                          "period", "pulse_first", "pulse_count")] + [
        ("padded", C.c_uint32), ("lane_count", C.c_uint32), ("precision", C.c_uint32), ("duration", C.c_double)]


class GpuInfo(C.Structure):
    _fields_ = [("name", C.c_char * 128), ("sm_major", C.c_uint32), ("sm_minor", C.c_uint32),
                ("multiprocessors", C.c_uint32), ("total_bytes", C.c_uint64), ("free_bytes", C.c_uint64),
                ("arena_bytes", C.c_uint64)]


class GpuKinTuning(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("block", C.c_uint32), ("chunk", C.c_uint32), ("variant", C.c_uint32),
                ("ms", C.c_float)]


class GpuServeRequest(C.Structure):
    _fields_ = [("y0", C.c_void_p), ("k", C.c_void_p), ("cells", C.c_uint32), ("channel_cells", C.c_uint32),
                ("coupling_steps", C.c_uint32), ("precision", C.c_uint32), ("mechanism", C.c_uint32),
                ("reserved", C.c_uint32), ("dt", C.c_double), ("velocity_m_s", C.c_double), ("dx_m", C.c_double)]


class GpuServeStatus(C.Structure):
    _fields_ = [("state", C.c_uint32), ("error", C.c_int32), ("steps_completed", C.c_uint32),
                ("substeps", C.c_uint32), ("courant", C.c_double), ("admit_s", C.c_double), ("latency_s", C.c_double)]


class GpuServeStats(C.Structure):
    _fields_ = [("budget_bytes", C.c_uint64), ("in_use_bytes", C.c_uint64), ("peak_bytes", C.c_uint64),
                ("graph_launches", C.c_uint64), ("running", C.c_uint32), ("waiting", C.c_uint32),
                ("finished", C.c_uint32), ("reserved", C.c_uint32)]


assert C.sizeof(GpuServeRequest) == 64 and C.sizeof(GpuServeStatus) == 40 and C.sizeof(GpuServeStats) == 48
assert C.sizeof(KinMech) == 30044 and C.sizeof(KinMethod) == 200 and C.sizeof(KinControl) == 56
assert C.sizeof(GpuKinLaunch) == 120 and C.sizeof(GpuInfo) == 168

# The 16 exports the reference's loader resolves (src/gpu/gpu_api.h:112-115).
REFERENCE_EXPORTS = ("gpu_init", "gpu_error_string", "gpu_alloc", "gpu_arena_used", "gpu_arena_reset",
                     "gpu_copy_to_device", "gpu_copy_to_host", "gpu_sync", "gpu_step_points", "gpu_kin_set_mech",
                     "gpu_kin_advance", "gpu_host_register", "gpu_host_unregister", "gpu_kin_advance_async",
                     "gpu_kin_wait", "gpu_kin_set_mode")

_lib = None


class GpuDbdZones(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("y", "h", "steps", "rejects", "pulses", "failed", "k", "src", "pulse", "period",
                                          "pulse_first", "pulse_count", "pulse_index", "T_K", "p_Pa", "x_H2O",
                                          "power_W_cm3", "freq_Hz", "source_temp")] + \
               [("count", C.c_uint32), ("padded", C.c_uint32), ("n_species", C.c_uint32), ("n_reactions", C.c_uint32)]


class GpuAirSource(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("g_O2_diss", "f_O1D", "g_N2A", "g_N2_diss", "g_OH_per_100eV", "filament_J_cm3")]


class GpuNftTransport(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("rows", "hot", "cold", "sites", "out_sum", "evap_kg")] + \
               [(n, C.c_uint32) for n in ("groups", "cells", "sites_count", "site_offset", "site_stride", "substeps",
                                          "flush_denormals")] + \
               [("ref", C.c_float * 9)] + [(n, C.c_float) for n in ("T_amb", "radiant", "e0", "es_slope")]


class GpuError(RuntimeError):
    def __init__(self, code: int, where: str):
        msg = lib().gpu_error_string(code).decode() if _lib is not None else str(code)
        super().__init__(f"{where}: CUDA error {code} ({msg})")
        self.code = code


def lib() -> C.CDLL:
    """The module library (built by simstack_gb300.build / __graft_entry__.build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run `python -m simstack_gb300.build` (there is no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        vp, u32, u64, i32, d, f = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int32, C.c_double, C.c_float
        sig = {
            "gpu_init": (i32, [u32, u64, C.POINTER(GpuInfo)]),
            "gpu_error_string": (C.c_char_p, [i32]),
            "gpu_alloc": (vp, [u64]),
            "gpu_arena_used": (u64, []),
            "gpu_arena_reset": (None, []),
            "gpu_copy_to_device": (i32, [vp, vp, u64]),
            "gpu_copy_to_host": (i32, [vp, vp, u64]),
            "gpu_sync": (i32, []),
            "gpu_step_points": (i32, [vp, vp, vp, vp, vp, vp, u32, f]),
            "gpu_kin_set_mech": (i32, [C.POINTER(KinMech), C.POINTER(KinMethod), C.POINTER(KinControl)]),
            "gpu_kin_advance": (i32, [C.POINTER(GpuKinLaunch), C.POINTER(f)]),
            "gpu_host_register": (i32, [vp, u64]),
            "gpu_host_unregister": (i32, [vp]),
            "gpu_kin_advance_async": (i32, [C.POINTER(GpuKinLaunch), vp, vp, u64, u64]),
            "gpu_kin_wait": (i32, [C.POINTER(f), C.POINTER(f)]),
            "gpu_kin_set_mode": (i32, [u32]),
            "gpu_kin_advance_queue": (i32, [C.POINTER(GpuKinLaunch), C.POINTER(f)]),
            "gpu_kin_advance_pipelined": (i32, [C.POINTER(GpuKinLaunch), vp, vp, u64, u64, u32, C.POINTER(f)]),
            "gpu_kin_set_tuning": (i32, [C.POINTER(GpuKinTuning)]),
            "gpu_kin_get_tuning": (i32, [u32, C.POINTER(GpuKinTuning)]),
            "gpu_kin_autotune": (i32, [C.POINTER(GpuKinLaunch), u32, C.POINTER(GpuKinTuning)]),
            "gpu_kin_last_stats": (i32, [C.POINTER(u64), C.POINTER(f)]),
            "gpu_kin_set_refinement": (i32, [u32]),
            "gpu_kin_set_mixed_variant": (i32, [u32]),
            "gpu_kin_get_mixed_variant": (u32, []),
            "gpu_kin_set_wait_limit": (i32, [u32]),
            "gpu_kin_set_straggler_budget": (i32, [u32]),
            "gpu_kin_set_straggler_block": (i32, [u32]),
            "gpu_stack_limit": (i32, [u64, C.POINTER(u64)]),
            "gpu_kin_parked_cells": (i32, [C.POINTER(u32)]),
            "gpu_probe_throughput": (i32, [u32, C.POINTER(d)]),
            "gpu_stream": (vp, []),
            "gpu_copy_on_device": (i32, [vp, vp, u64]),
            "gpu_kin_advance_noalloc": (i32, [C.POINTER(KinMech), C.POINTER(KinMethod), C.POINTER(KinControl),
                                              C.POINTER(GpuKinLaunch), vp, i32]),
            "gpu_kin_coop_set_mech": (i32, [vp, C.POINTER(KinMethod), C.POINTER(KinControl)]),
            "gpu_kin_coop_advance": (i32, [C.POINTER(GpuKinLaunch), C.POINTER(f)]),
            "gpu_kin_coop_info": (i32, [C.POINTER(u64)]),
            "gpu_kin_coop_set_refinement": (i32, [u32]),
            "gpu_kin_coop_set_shape": (i32, [u32, u32, u32]),
            "gpu_kin_coop_set_smem_budget": (i32, [u32, u32]),
            "gpu_kin_coop_phase_cycles": (i32, [C.POINTER(u64)]),
            "gpu_advect": (i32, [vp, u32, u32, u32, u32, vp, d, u32, vp]),
            "gpu_serve_open": (i32, [u64, C.POINTER(KinControl)]),
            "gpu_serve_set_mech": (i32, [C.POINTER(KinMech), C.POINTER(KinMethod)]),
            "gpu_serve_submit": (i32, [C.POINTER(GpuServeRequest), C.POINTER(u64)]),
            "gpu_serve_set_coop_mech": (i32, [vp, C.POINTER(KinMethod), C.POINTER(KinControl)]),
            "gpu_serve_progress": (i32, [C.POINTER(u32), C.POINTER(u32), C.POINTER(u32)]),
            "gpu_serve_cancel": (i32, [u64]),
            "gpu_serve_poll": (i32, [u64, C.POINTER(GpuServeStatus)]),
            "gpu_serve_result": (i32, [u64, vp, vp, vp]),
            "gpu_serve_forget": (i32, [u64]),
            "gpu_serve_stats": (i32, [C.POINTER(GpuServeStats)]),
            "gpu_serve_close": (i32, []),
            "kin_model_new": (vp, []),
            "kin_model_air": (vp, []),
            "kin_model_free": (None, [vp]),
            "kin_model_add_species": (u32, [vp, C.c_char_p, i32]),
            "kin_model_add_reaction": (u32, [vp, C.c_char_p, i32, C.POINTER(d), i32]),
            "kin_model_finalize": (i32, [vp]),
            "kin_model_error": (C.c_char_p, [vp]),
            "kin_model_equation": (i32, [vp, u32, C.c_char_p, u32]),
            "kin_model_counts": (None, [vp, C.POINTER(u64)]),
            "kin_model_kinmech": (i32, [vp, C.POINTER(KinMech)]),
            "kin_mech_signature": (u64, [C.POINTER(KinMech)]),
            "kin_model_coop_image": (u64, [vp, vp, u64]),
            "kin_mech_coop_image": (u64, [C.POINTER(KinMech), vp, u64]),
            "kin_model_rate_constants": (None, [vp, d, d, vp]),
            "kin_model_rate_block": (None, [vp, vp, vp, u32, u32, vp]),
            "kin_method_coefficients": (KinMethod, [u32]),
            "kin_air_source_delta": (None, [vp, u32, d, d, vp]),
            "kin_air_source_temperature": (None, [vp, u32, u32, vp]),
            "gpu_dbd_prepare_source": (i32, [C.POINTER(GpuDbdZones), C.POINTER(GpuAirSource), u32, d, d]),
            "gpu_dbd_commit_pulses": (i32, [C.POINTER(GpuDbdZones)]),
            "gpu_dbd_flow_exchange": (i32, [C.POINTER(GpuDbdZones), d, d]),
            "gpu_dbd_step": (i32, [C.POINTER(GpuDbdZones), C.POINTER(GpuAirSource), u32, d, d, u32, u32, d, C.POINTER(f)]),
            "gpu_nft_transport": (i32, [C.POINTER(GpuNftTransport), C.POINTER(f)]),
            "sgb_workload_air": (None, [u64, u64, u32, u32, d, d, d, d, vp, vp, vp, vp]),
            "sgb_workload_air_source": (None, [u64, u64, u32, u32, d, d, vp, vp, vp, vp]),
            "sgb_workload_synthetic_mech": (vp, [u64, u32, u32, d, u32, d, d, vp]),
            "sgb_workload_synthetic_cells": (None, [u64, u64, u32, u32, u32, d, d, vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(code: int, where: str) -> None:
    if code != 0:
        raise GpuError(code, where)


def _p(a: np.ndarray | None):
    return None if a is None else a.ctypes.data


def aligned_empty(count: int, align: int = 256) -> np.ndarray:
    raw = np.empty(count + align // 8, np.float64)
    off = (-raw.ctypes.data % align) // 8
    return raw[off:off + count]


# --------------------------------------------------------------------------
# Mechanisms, methods, control.

class Model:
    """A mechanism compiled by the module's host-side symbolic phase."""

    def __init__(self, handle):
        if not handle:
            raise MemoryError("kin_model allocation failed")
        self.h = handle

    @classmethod
    def air(cls) -> "Model":
        return cls(lib().kin_model_air())

    @classmethod
    def new(cls) -> "Model":
        return cls(lib().kin_model_new())

    @classmethod
    def synthetic(cls, seed: int, species: int = 200, reactions: int = 1200, bimolecular: float = 0.7,
                  products: int = 1, lk_lo: float = -3.0, lk_hi: float = 9.0) -> "Model":
        k = np.zeros(reactions)
        m = cls(lib().sgb_workload_synthetic_mech(seed, species, reactions, bimolecular, products, lk_lo, lk_hi, _p(k)))
        m.k_const = k
        return m

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.kin_model_free(self.h)
            self.h = None

    def add_species(self, name: str, abstract: bool = False) -> int:
        return lib().kin_model_add_species(self.h, name.encode(), int(abstract))

    def add_reaction(self, equation: str, kind: str = "arr", params=(1.0, 0.0, 0.0), ref: int = 0) -> int:
        kinds = {"arr": 0, "m": 1, "troe": 2, "eqrev": 3}
        p = (C.c_double * 5)(*(list(params) + [0.0] * (5 - len(params))))
        return lib().kin_model_add_reaction(self.h, equation.encode(), kinds[kind], p, ref)

    def finalize(self) -> None:
        if lib().kin_model_finalize(self.h) != 0:
            raise ValueError(self.error)

    @property
    def error(self) -> str:
        return lib().kin_model_error(self.h).decode()

    def counts(self) -> dict:
        c = (C.c_uint64 * 7)()
        lib().kin_model_counts(self.h, c)
        return dict(zip(("n", "R", "nnz", "divs", "subs", "lower", "upper"), [int(v) for v in c]))

    @property
    def n(self) -> int:
        return self.counts()["n"]

    @property
    def R(self) -> int:
        return self.counts()["R"]

    def kinmech(self) -> KinMech:
        km = KinMech()
        if lib().kin_model_kinmech(self.h, C.byref(km)) != 0:
            raise ValueError("mechanism exceeds the KinMech capacities")
        return km

    def rate_constants(self, T: float, M: float) -> np.ndarray:
        k = np.zeros(max(self.R, 1))
        lib().kin_model_rate_constants(self.h, T, M, _p(k))
        return k[: self.R]


def model_equation(model: Model, r: int) -> str:
    buf = C.create_string_buffer(128)
    if not lib().kin_model_equation(model.h, r, buf, 128):
        raise IndexError(r)
    return buf.value.decode()


def kinmech_bytes(km: KinMech) -> bytes:
    return C.string_at(C.addressof(km), C.sizeof(km))


def signature(km: KinMech) -> int:
    return int(lib().kin_mech_signature(C.byref(km)))


def method(name: str = "rodas3") -> KinMethod:
    return lib().kin_method_coefficients(METHODS[name])


def control(rtol=1e-4, atol=ATOL_1E12_MOLAR, h_min=1e-14, h_max=0.0, h_start=1e-9, max_steps=1_000_000,
            fixed_step=0, clamp_negative=1) -> KinControl:
    """KinControl; defaults are the benchmark settings: rtol 1e-4, atol 1e-12 mol/L
    (6.022e8 cm^-3), the reference's h_min/h_start (src/sim/dbd.cpp:485-495),
    max_steps raised from 20,000 to 1e6."""
    return KinControl(rtol, atol, h_min, h_max, h_start, max_steps, fixed_step, clamp_negative)


# --------------------------------------------------------------------------
# Zone block: one contiguous float64 block, solver-written rows first
# (src/sim/dbd.cpp:60-83), so a download needs only the mutable prefix.

ROWS_ORDER = ("y", "h", "steps", "rejects", "pulses", "failed", "k", "src", "pulse", "period", "pulse_first",
              "pulse_count")


class ZoneBlock:
    """Host zone block for `cells` cells of an n-species, R-reaction mechanism."""

    def __init__(self, n: int, R: int, cells: int, pad_to: int = 8):
        self.n, self.R, self.cells = n, R, cells
        self.padded = P = max(pad_to, (cells + pad_to - 1) // pad_to * pad_to)
        rows = {"y": n, "h": 1, "steps": 1, "rejects": 1, "pulses": 1, "failed": 1, "k": R, "src": n, "pulse": n,
                "period": 1, "pulse_first": 1, "pulse_count": 1}
        self.row_offset = {}
        off = 0
        for name in ROWS_ORDER:
            self.row_offset[name] = off
            off += rows[name]
        self.rows = off
        self.mutable_rows = rows["y"] + 5
        self.data = aligned_empty(self.rows * P)
        self.data[:] = 0.0
        self.block = self.data.reshape(self.rows, P)
        self.views = {}
        for name in ROWS_ORDER:
            r0 = self.row_offset[name]
            v = self.block[r0:r0 + rows[name]]
            self.views[name] = v if rows[name] > 1 or name in ("y", "k", "src", "pulse") else v[0]

    def __getitem__(self, name: str) -> np.ndarray:
        return self.views[name]

    @property
    def nbytes(self) -> int:
        return self.data.nbytes

    def as_dict(self) -> dict:
        """Row views by name (the oracle's block argument)."""
        return dict(self.views)

    def launch(self, device_base: int, precision: int = 0, duration: float = 1.0, lane_count: int = 0) -> GpuKinLaunch:
        """GpuKinLaunch for a device mirror at `device_base` (same row offsets)."""
        L = GpuKinLaunch()
        for name in ROWS_ORDER:
            setattr(L, name, device_base + self.row_offset[name] * self.padded * 8)
        L.padded = self.padded
        L.lane_count = lane_count
        L.precision = precision
        L.duration = duration
        return L

    def copy(self) -> "ZoneBlock":
        z = ZoneBlock.__new__(ZoneBlock)
        z.__dict__.update({k: v for k, v in self.__dict__.items() if k not in ("data", "block", "views")})
        z.data = aligned_empty(self.data.size)
        z.data[:] = self.data
        z.block = z.data.reshape(self.rows, self.padded)
        z.views = {}
        for name in ROWS_ORDER:
            r0 = self.row_offset[name]
            cnt = self.views[name].shape[0] if self.views[name].ndim == 2 else 1
            v = z.block[r0:r0 + cnt]
            z.views[name] = v if self.views[name].ndim == 2 else v[0]
        return z


def air_cells(cells: int, seed: int = 1, first_cell: int = 0, pad_to: int = 8, T=(288.0, 303.0),
              log10_c=(-12.0, -2.0)) -> ZoneBlock:
    """Shipped-mechanism zone block with the seeded synthetic initial state
    (T ~ U[288, 303] K, pH ~ U[3, 7] drawn and unused, c ~ 10^U[-12, -2] mol/L,
    H2O = 55.5 mol/L; y in molecules/cm^3; k from the rate laws at T and 1 atm).
    Padding lanes copy cell 0, as the reference's dbd_zones_fill_padding does."""
    z = ZoneBlock(17, 44, cells, pad_to)
    Tv = np.zeros(z.padded)
    pH = np.zeros(z.padded)
    y = np.zeros((17, z.padded))
    k = np.zeros((44, z.padded))
    lib().sgb_workload_air(seed, first_cell, cells, z.padded, T[0], T[1], log10_c[0], log10_c[1], _p(y), _p(k), _p(Tv), _p(pH))
    for i in range(cells, z.padded):
        y[:, i] = y[:, 0]
        k[:, i] = k[:, 0]
        Tv[i] = Tv[0]
    z["y"][:] = y
    z["k"][:] = k
    z.T = Tv
    z.pH = pH
    return z


def air_source(z: ZoneBlock, seed: int, P0: float, decades: float = 3.0, first_cell: int = 0) -> np.ndarray:
    """Averaged discharge source (the uneven-stiffness workload) per cell into z['src']; returns power per cell."""
    src = np.zeros((17, z.padded))
    power = np.zeros(z.padded)
    y = np.ascontiguousarray(z["y"])
    lib().sgb_workload_air_source(seed, first_cell, z.padded, z.padded, P0, decades, _p(y), _p(np.ascontiguousarray(z.T)),
                                  _p(src), _p(power))
    z["src"][:] = src
    return power


def synthetic_cells(model: Model, cells: int, seed: int, log10_c=(-10.0, -3.0), first_cell: int = 0,
                    pad_to: int = 8) -> ZoneBlock:
    n, R = model.n, model.R
    z = ZoneBlock(n, R, cells, pad_to)
    y = np.zeros((n, z.padded))
    lib().sgb_workload_synthetic_cells(seed, first_cell, z.padded, z.padded, n, log10_c[0], log10_c[1], _p(y))
    z["y"][:] = y
    z["k"][:] = model.k_const[:, None]
    return z


# --------------------------------------------------------------------------
# The module (one device; the reference's GPU module semantics).

class Module:
    """gpu_init + helpers for device mirrors of zone blocks."""

    def __init__(self, device: int = 0, arena_bytes: int = 1 << 30):
        self.info = GpuInfo()
        check(lib().gpu_init(device, arena_bytes, C.byref(self.info)), "gpu_init")

    def set_mech(self, km: KinMech, meth: KinMethod | None = None, ctl: KinControl | None = None) -> None:
        meth = meth if meth is not None else method("rodas3")
        ctl = ctl if ctl is not None else control()
        self._keep = (km, meth, ctl)
        check(lib().gpu_kin_set_mech(C.byref(km), C.byref(meth), C.byref(ctl)), "gpu_kin_set_mech")

    def alloc(self, nbytes: int) -> int:
        p = lib().gpu_alloc(nbytes)
        if not p:
            raise MemoryError(f"gpu_alloc({nbytes}): device arena full")
        return p

    def reset_arena(self) -> None:
        lib().gpu_arena_reset()

    def upload(self, z: ZoneBlock, device_base: int | None = None) -> int:
        base = device_base if device_base is not None else self.alloc(z.nbytes)
        check(lib().gpu_copy_to_device(base, _p(z.data), z.nbytes), "gpu_copy_to_device")
        return base

    def download(self, z: ZoneBlock, device_base: int, mutable_only: bool = True) -> None:
        nbytes = z.mutable_rows * z.padded * 8 if mutable_only else z.nbytes
        check(lib().gpu_copy_to_host(_p(z.data), device_base, nbytes), "gpu_copy_to_host")

    def advance(self, L: GpuKinLaunch, queue: bool | None = None) -> float:
        ms = C.c_float()
        if queue:
            check(lib().gpu_kin_advance_queue(C.byref(L), C.byref(ms)), "gpu_kin_advance_queue")
        else:
            check(lib().gpu_kin_advance(C.byref(L), C.byref(ms)), "gpu_kin_advance")
        return ms.value

    def set_tuning(self, kind: int = 1, block: int = 128, variant: int = 0, ctas_per_sm: int = 0) -> None:
        t = GpuKinTuning(kind, block, ctas_per_sm, variant, 0.0)
        check(lib().gpu_kin_set_tuning(C.byref(t)), "gpu_kin_set_tuning")

    def tuning(self, precision: int = 0) -> GpuKinTuning:
        t = GpuKinTuning()
        check(lib().gpu_kin_get_tuning(precision, C.byref(t)), "gpu_kin_get_tuning")
        return t

    def autotune(self, L: GpuKinLaunch, kind: int = 1) -> GpuKinTuning:
        t = GpuKinTuning()
        check(lib().gpu_kin_autotune(C.byref(L), kind, C.byref(t)), "gpu_kin_autotune")
        return t

    def probe(self, kind: int) -> float:
        v = C.c_double()
        check(lib().gpu_probe_throughput(kind, C.byref(v)), "gpu_probe_throughput")
        return v.value

    def launches(self) -> int:
        n = C.c_uint64()
        lib().gpu_kin_last_stats(C.byref(n), None)
        return int(n.value)

    def integrate(self, z: ZoneBlock, duration: float, precision: int = 0, queue: bool | None = None,
                  device_base: int | None = None) -> float:
        """dbd_advance_gpu: upload the whole block, advance, download the
        solver-written prefix (src/sim/dbd.cpp:272-295). Returns kernel ms."""
        base = self.upload(z, device_base)
        ms = self.advance(z.launch(base, precision, duration), queue)
        self.download(z, base)
        return ms

    def set_mixed_variant(self, variant: int) -> None:
        """Precision 2: 0 = FP64 state with an FP64-residual refinement sweep, 1 = double-float state."""
        check(lib().gpu_kin_set_mixed_variant(variant), "gpu_kin_set_mixed_variant")

    def mixed_variant(self) -> int:
        return int(lib().gpu_kin_get_mixed_variant())

    def set_straggler_budget(self, attempts: int) -> None:
        """Cells still stepping after `attempts` attempts are finished by the cooperative kernel (0 = off)."""
        check(lib().gpu_kin_set_straggler_budget(attempts), "gpu_kin_set_straggler_budget")

    def parked_cells(self) -> int:
        c = C.c_uint32()
        check(lib().gpu_kin_parked_cells(C.byref(c)), "gpu_kin_parked_cells")
        return c.value

    def integrate_pipelined(self, z: ZoneBlock, duration: float, precision: int = 0, chunks: int = 4,
                            device_base: int | None = None) -> float:
        """Host block in, results back, with the copies overlapped with the kernels
        (gpu_kin_advance_pipelined); the host block should be page-locked. Returns device ms."""
        base = device_base if device_base is not None else self.alloc(z.nbytes)
        ms = C.c_float()
        L = z.launch(base, precision, duration, z.cells)
        check(lib().gpu_kin_advance_pipelined(C.byref(L), _p(z.data), base, z.rows, z.mutable_rows, chunks, C.byref(ms)),
              "gpu_kin_advance_pipelined")
        return ms.value

    # cooperative kernels (one CTA per cell): mechanisms beyond the KinMech tables
    def coop_set_mech(self, model: "Model", meth: KinMethod | None = None, ctl: KinControl | None = None) -> None:
        meth = meth if meth is not None else method("rodas3")
        ctl = ctl if ctl is not None else control()
        self._coop_keep = (model, meth, ctl)
        check(lib().gpu_kin_coop_set_mech(model.h, C.byref(meth), C.byref(ctl)), "gpu_kin_coop_set_mech")

    def coop_info(self) -> dict:
        out = (C.c_uint64 * 8)()
        check(lib().gpu_kin_coop_info(out), "gpu_kin_coop_info")
        return dict(zip(("n", "R", "nnz", "jac_entries", "l_entries", "u_entries", "lu_updates", "image_bytes"),
                        [int(v) for v in out]))

    def coop_advance(self, L: GpuKinLaunch) -> float:
        ms = C.c_float()
        check(lib().gpu_kin_coop_advance(C.byref(L), C.byref(ms)), "gpu_kin_coop_advance")
        return ms.value

    def coop_integrate(self, z: ZoneBlock, duration: float, precision: int = 0, lane_count: int = 0,
                       device_base: int | None = None) -> float:
        base = self.upload(z, device_base)
        ms = self.coop_advance(z.launch(base, precision, duration, lane_count))
        self.download(z, base)
        return ms


# --------------------------------------------------------------------------
# DBD zone driver helpers (host side of the reference's caller,
# src/sim/dbd.cpp:60-158): feed gas, rate constants, discharge source and the
# pulse schedule of one master step.

BOLTZMANN_J_K = 1.380649e-23
AIR_O2, AIR_N2, AIR_H2O = 15, 14, 16


def dbd_zones(count: int, T_K, x_H2O, power_W_cm3, freq_Hz, p_Pa: float = 101325.0, pad_to: int = 8) -> ZoneBlock:
    """Zones filled with humid-air feed gas (air_mech.cpp:280-288) at their
    operating points, rate constants at T and M = p/(kB T) (dbd.cpp:107-116);
    padding lanes copy zone 0's operating point (dbd.cpp:97-101)."""
    z = ZoneBlock(17, 44, count, pad_to)
    P = z.padded

    def full(v):
        a = np.zeros(P)
        a[:count] = np.broadcast_to(np.asarray(v, np.float64), (count,))
        a[count:] = a[0]
        return a

    z.T, z.x_H2O, z.power, z.freq = full(T_K), full(x_H2O), full(power_W_cm3), full(freq_Hz)
    z.p_Pa = np.full(P, p_Pa)
    z.pulse_index = np.zeros(P)
    model = Model.air()
    for i in range(P):
        total = z.p_Pa[i] / (BOLTZMANN_J_K * z.T[i]) * 1e-6
        dry = 1.0 - z.x_H2O[i]
        z["y"][:, i] = 0.0
        z["y"][AIR_N2, i] = total * dry * 0.79
        z["y"][AIR_O2, i] = total * dry * 0.21
        z["y"][AIR_H2O, i] = total * z.x_H2O[i]
        z["k"][:, i] = model.rate_constants(z.T[i], total)
    return z


def dbd_prepare_source(z: ZoneBlock, pulsed: bool, t0: float, t1: float) -> None:
    """One master step's discharge source and pulse schedule (dbd.cpp:123-152):
    pulsed = one radical injection per AC half-cycle at f64 absolute pulse times,
    averaged = the same energy as a per-second source."""
    P = z.padded
    y = np.ascontiguousarray(z["y"])
    d = np.zeros(17)
    for i in range(P):
        freq = z.freq[i]
        on = z.power[i] > 0.0 and freq > 0.0
        pulses_per_s = 2.0 * freq
        col = np.ascontiguousarray(y[:, i])
        if pulsed and on:
            lib().kin_air_source_delta(_p(col), 17, z.power[i] / pulses_per_s, z.T[i], _p(d))
            z["pulse"][:, i] = d
            z["src"][:, i] = 0.0
            period = 1.0 / pulses_per_s
            z["period"][i] = period
            nxt, count = z.pulse_index[i] + 1.0, 0.0
            while (nxt + count) * period <= t1:
                count += 1.0
            z["pulse_first"][i] = nxt * period - t0
            z["pulse_count"][i] = count
        else:
            lib().kin_air_source_delta(_p(col), 17, z.power[i] if on else 0.0, z.T[i], _p(d))
            z["src"][:, i] = d
            z["pulse"][:, i] = 0.0
            z["period"][i] = 0.0
            z["pulse_first"][i] = 0.0
            z["pulse_count"][i] = 0.0


def dbd_commit_pulses(z: ZoneBlock) -> None:
    z.pulse_index += z["pulse_count"]


DBD_HOST_ROWS = ("pulse_index", "T_K", "p_Pa", "x_H2O", "power_W_cm3", "freq_Hz")


def dbd_block(z: ZoneBlock) -> np.ndarray:
    """The zones as one float64 block in the reference's DbdZones layout (src/sim/dbd.cpp:60-83):
    the solver's rows, then pulse_index, T_K, p_Pa, x_H2O, power_W_cm3, freq_Hz, followed by
    the source's five temperature-factor rows (kin_air_source_temperature)."""
    P = z.padded
    extra = np.zeros((len(DBD_HOST_ROWS) + 5, P))
    for j, v in enumerate((z.pulse_index, z.T, z.p_Pa, z.x_H2O, z.power, z.freq)):
        extra[j] = v
    tf = np.zeros((5, P))
    lib().kin_air_source_temperature(_p(np.ascontiguousarray(z.T)), P, P, _p(tf))
    extra[len(DBD_HOST_ROWS):] = tf
    out = aligned_empty((z.rows + extra.shape[0]) * P).reshape(-1, P)   # 256-byte aligned, as the arena's blocks
    out[: z.rows] = z.block
    out[z.rows:] = extra
    return out


class DeviceZones:
    """A zone block kept in device memory for the device zone driver (gpu_dbd_*): uploaded
    once, stepped in place, downloaded when the caller wants it."""

    def __init__(self, module: "Module", z: ZoneBlock):
        self.z = z
        self.host = dbd_block(z)
        self.base = module.alloc(self.host.nbytes)
        check(lib().gpu_copy_to_device(self.base, _p(self.host), self.host.nbytes), "gpu_copy_to_device")
        P, rows = z.padded, z.rows
        self.g = GpuDbdZones()
        for name in ROWS_ORDER:
            setattr(self.g, name, self.base + z.row_offset[name] * P * 8)
        for j, name in enumerate(DBD_HOST_ROWS):
            setattr(self.g, name, self.base + (rows + j) * P * 8)
        self.g.source_temp = self.base + (rows + len(DBD_HOST_ROWS)) * P * 8
        self.g.count, self.g.padded, self.g.n_species, self.g.n_reactions = z.cells, P, z.n, z.R

    def step(self, t0: float, dt: float, pulsed: bool, precision: int = 0, chained: bool = False,
             residence_s: float = 0.0, source: GpuAirSource | None = None) -> float:
        ms = C.c_float()
        check(lib().gpu_dbd_step(C.byref(self.g), C.byref(source) if source is not None else None, int(pulsed), t0, dt,
                                 precision, int(chained), residence_s, C.byref(ms)), "gpu_dbd_step")
        return ms.value

    def download(self) -> np.ndarray:
        """The whole device block (reference layout) into self.host; returns it."""
        check(lib().gpu_copy_to_host(_p(self.host), self.base, self.host.nbytes), "gpu_copy_to_host")
        return self.host


SERVE_STATES = ("waiting", "running", "done", "failed", "cancelled")
DEFAULT_STRAGGLER_BUDGET = 600   # the module's default FP64 hand-off budget (gpu_kin_set_straggler_budget)


class Server:
    """The serving engine (gpu_serve_*): requests of cells integrated over 1 s
    coupling steps of chemistry + film advection, admitted while they fit the
    HBM budget, state device-resident until done. One host thread drives it
    through progress()."""

    def __init__(self, budget_bytes: int = 0, ctl: KinControl | None = None):
        self._ctl = ctl if ctl is not None else control()
        check(lib().gpu_serve_open(budget_bytes, C.byref(self._ctl)), "gpu_serve_open")
        self._species = {}

    def set_mech(self, km: KinMech, meth: KinMethod | None = None) -> None:
        meth = meth if meth is not None else method("rodas3")
        self._mech = (km, meth)
        check(lib().gpu_serve_set_mech(C.byref(km), C.byref(meth)), "gpu_serve_set_mech")
        self._table_shape = (int(km.species_count), int(km.reaction_count))

    def set_coop_mech(self, model: "Model", meth: KinMethod | None = None, ctl: KinControl | None = None) -> None:
        """Large mechanism for requests with mechanism = 2 (cooperative kernels); ctl = its step
        control in the model's own units (None: the engine's control)."""
        meth = meth if meth is not None else method("rodas3")
        self._coop = (model, meth, ctl)
        check(lib().gpu_serve_set_coop_mech(model.h, C.byref(meth), C.byref(ctl) if ctl is not None else None),
              "gpu_serve_set_coop_mech")
        self._coop_shape = (model.n, model.R)

    def submit(self, y0: np.ndarray, k: np.ndarray, coupling_steps: int, channel_cells: int, velocity_m_s: float,
               dx_m: float = 0.05, dt: float = 1.0, precision: int = 0, mechanism: int = 0) -> int:
        y0 = np.ascontiguousarray(y0, dtype=np.float64)
        k = np.ascontiguousarray(k, dtype=np.float64)
        n, R = (17, 44) if mechanism == 0 else getattr(self, "_table_shape" if mechanism == 1 else "_coop_shape", (0, 0))
        if (n, R) != (0, 0) and (y0.shape[0] != n or k.shape != (R, y0.shape[1])):   # unset mechanisms: the engine refuses
            raise ValueError(f"request arrays {y0.shape} / {k.shape} do not match the mechanism ({n} species, {R} reactions)")
        q = GpuServeRequest(_p(y0), _p(k), y0.shape[1], channel_cells, coupling_steps, precision, mechanism, 0, dt,
                            velocity_m_s, dx_m)
        rid = C.c_uint64()
        check(lib().gpu_serve_submit(C.byref(q), C.byref(rid)), "gpu_serve_submit")
        self._species[rid.value] = (y0.shape[0], y0.shape[1])
        return rid.value

    def progress(self) -> tuple[int, int, int]:
        r, w, f = C.c_uint32(), C.c_uint32(), C.c_uint32()
        check(lib().gpu_serve_progress(C.byref(r), C.byref(w), C.byref(f)), "gpu_serve_progress")
        return r.value, w.value, f.value

    def poll(self, rid: int) -> dict:
        st = GpuServeStatus()
        check(lib().gpu_serve_poll(rid, C.byref(st)), "gpu_serve_poll")
        return dict(state=SERVE_STATES[st.state], error=st.error, steps_completed=st.steps_completed,
                    substeps=st.substeps, courant=st.courant, admit_s=st.admit_s, latency_s=st.latency_s)

    def cancel(self, rid: int) -> None:
        check(lib().gpu_serve_cancel(rid), "gpu_serve_cancel")

    def result(self, rid: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        n, cells = self._species[rid]
        y, steps, failed = np.zeros((n, cells)), np.zeros(cells), np.zeros(cells)
        check(lib().gpu_serve_result(rid, _p(y), _p(steps), _p(failed)), "gpu_serve_result")
        return y, steps, failed

    def forget(self, rid: int) -> None:
        check(lib().gpu_serve_forget(rid), "gpu_serve_forget")
        self._species.pop(rid, None)

    def stats(self) -> dict:
        st = GpuServeStats()
        check(lib().gpu_serve_stats(C.byref(st)), "gpu_serve_stats")
        return {name: getattr(st, name) for name, _ in GpuServeStats._fields_ if name != "reserved"}

    def drain(self, timeout_s: float = 600.0, sleep_s: float = 2e-4) -> None:
        """Drives the engine until nothing is running or waiting."""
        import time
        t_end = time.monotonic() + timeout_s
        while True:
            running, waiting, _ = self.progress()
            if running == 0 and waiting == 0:
                return
            if time.monotonic() > t_end:
                raise TimeoutError(f"serving: {running} running, {waiting} waiting after {timeout_s} s")
            time.sleep(sleep_s)

    def close(self) -> None:
        check(lib().gpu_serve_close(), "gpu_serve_close")

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


# --------------------------------------------------------------------------
# NFT film transport (gpu_nft_transport): the reference's group arrays on the device.

NFT_LANES, NFT_FIELDS = 8, 9
# floats per element of each group array (src/sim/nft.cpp:134-178)
NFT_FLOATS = {"rows": 72, "hot": 32, "cold": 80, "sites": 288}


class NftTransport:
    """Device copies of G groups' NFT arrays (float32 views of the reference's layouts:
    rows [G][cells][9][8], hot [G][cells][4][8], cold [G][cells] 80 floats, sites
    [G][sites] 288 floats), packed group after group in the module's arena, and one
    window's transport over all of them."""

    def __init__(self, module: "Module", groups: int, cells: int, sites: int, site_offset: int, site_stride: int):
        self.groups, self.cells, self.sites = groups, cells, sites
        self.site_offset, self.site_stride = site_offset, site_stride
        self.shape = {"rows": groups * cells * 72, "hot": groups * cells * 32, "cold": groups * cells * 80,
                      "sites": max(1, groups * sites * 288), "out_sum": groups * 72, "evap_kg": groups * 8}
        self.dev = {}
        for name, n in self.shape.items():
            self.dev[name] = module.alloc(4 * n)
            if not self.dev[name]:
                raise GpuError(2, f"NftTransport: arena full ({name})")

    def upload(self, name: str, host: np.ndarray) -> None:
        host = np.ascontiguousarray(host, np.float32)
        assert host.size == self.shape[name] or (name == "sites" and self.sites == 0), (name, host.size)
        if host.size:
            check(lib().gpu_copy_to_device(self.dev[name], _p(host), host.nbytes), f"upload {name}")

    def download(self, name: str) -> np.ndarray:
        out = np.empty(self.shape[name], np.float32)
        check(lib().gpu_copy_to_host(_p(out), self.dev[name], out.nbytes), f"download {name}")
        return out

    def run(self, ref, T_amb: float, radiant: float, e0: float, es_slope: float, substeps: int,
            flush_denormals: bool = True) -> float:
        t = GpuNftTransport()
        for name in ("rows", "hot", "cold", "sites", "out_sum", "evap_kg"):
            setattr(t, name, self.dev[name])
        t.groups, t.cells, t.sites_count = self.groups, self.cells, self.sites
        t.site_offset, t.site_stride, t.substeps = self.site_offset, self.site_stride, substeps
        t.flush_denormals = int(flush_denormals)
        for k in range(NFT_FIELDS):
            t.ref[k] = float(np.float32(ref[k]))
        t.T_amb, t.radiant, t.e0, t.es_slope = (float(np.float32(v)) for v in (T_amb, radiant, e0, es_slope))
        ms = C.c_float()
        check(lib().gpu_nft_transport(C.byref(t), C.byref(ms)), "gpu_nft_transport")
        return ms.value
