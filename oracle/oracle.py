"""TEST INFRASTRUCTURE -- NOT PART OF THE PRODUCT.

ctypes bindings for the CPU oracle (``liboracle.so``, built from
``kin_oracle.cpp``) and, where it was built, for the reference's own CPU solver
(``_ref/libref.so`` and ``_ref/libref_big.so``, compiled from the reference
sources by ``oracle/Makefile``). Imported only by ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``.

Zone blocks are passed as the reference's SoA layout (``src/sim/dbd.cpp:40-58``):
``y[species][padded]``, ``h``, ``steps``, ``rejects``, ``pulses``, ``failed``,
``k[reaction][padded]``, ``src[species][padded]``, ``pulse[species][padded]``,
``period``, ``pulse_first``, ``pulse_count`` -- a dict of float64 numpy arrays.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libref.so")
REF_BIG_LIB = os.path.join(HERE, "_ref", "libref_big.so")
KINMECH_BYTES = 30044

METHOD_IDS = {"ros2": 0, "ros3": 1, "rodas3": 2}
RATE_KIND = {"arr": 0, "m": 1, "troe": 2, "eqrev": 3}


class Control(C.Structure):
    """KinControl (src/sim/kinetics/kin_mech.h:112-120)."""

    _fields_ = [("rtol", C.c_double), ("atol", C.c_double), ("h_min", C.c_double), ("h_max", C.c_double),
                ("h_start", C.c_double), ("max_steps", C.c_uint32), ("fixed_step", C.c_int32),
                ("clamp_negative", C.c_int32)]


class LaneArrays(C.Structure):
    """DbdLaneArrays (src/sim/dbd_lanes.h:13-19)."""

    _fields_ = [(n, C.c_void_p) for n in ("y", "h", "steps", "rejects", "pulses", "failed", "k", "src", "pulse",
                                          "period", "pulse_first", "pulse_count")] + [("padded", C.c_uint32)]


BLOCK_FIELDS = ("y", "h", "steps", "rejects", "pulses", "failed", "k", "src", "pulse", "period", "pulse_first",
                "pulse_count")


def aligned_zeros(shape, align: int = 64) -> np.ndarray:
    """float64 zeros whose data pointer is `align`-byte aligned (the reference's
    f64x4 lanes use aligned AVX loads; SoaPush aligns to 64 bytes)."""
    count = int(np.prod(shape))
    raw = np.zeros(count + align // 8, np.float64)
    off = (-raw.ctypes.data % align) // 8
    return raw[off:off + count].reshape(shape)


def lane_arrays(block: dict, padded: int) -> LaneArrays:
    la = LaneArrays()
    for name in BLOCK_FIELDS:
        arr = block[name]
        assert arr.dtype == np.float64 and arr.flags["C_CONTIGUOUS"], name
        setattr(la, name, arr.ctypes.data)
    la.padded = padded
    return la


def control(rtol=1e-4, atol=6.02214076e8, h_min=1e-14, h_max=0.0, h_start=1e-9, max_steps=1_000_000,
            fixed_step=0, clamp_negative=1) -> Control:
    return Control(rtol, atol, h_min, h_max, h_start, max_steps, fixed_step, clamp_negative)


def build(quiet: bool = True) -> None:
    """Compile liboracle.so with the oracle's Makefile (any host)."""
    out = subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        vp, u32, i32, d, u64 = C.c_void_p, C.c_uint32, C.c_int32, C.c_double, C.c_uint64
        L.or_mech_new.restype = vp
        L.or_mech_new_air.restype = vp
        L.or_mech_free.argtypes = [vp]
        L.or_add_species.argtypes = [vp, C.c_char_p, i32]
        L.or_add_species.restype = u32
        L.or_add_reaction.argtypes = [vp, C.c_char_p, i32, C.POINTER(d), i32]
        L.or_add_reaction.restype = u32
        L.or_finalize.argtypes = [vp]
        L.or_error.argtypes = [vp]
        L.or_error.restype = C.c_char_p
        L.or_counts.argtypes = [vp, C.POINTER(u64)]
        L.or_export_kinmech.argtypes = [vp, vp, C.POINTER(u64)]
        L.or_export_kinmech.restype = i32
        L.or_pattern.argtypes = [vp, vp]
        L.or_lu_ops.argtypes = [vp, vp, vp]
        L.or_rate_constants.argtypes = [vp, d, d, vp]
        L.or_fun.argtypes = [vp, vp, vp, vp, vp]
        L.or_jac.argtypes = [vp, vp, vp, vp]
        L.or_decomp_solve.argtypes = [vp, vp, d, vp, vp]
        L.or_integrate_f64.argtypes = [vp, i32, C.POINTER(Control), vp, vp, vp, C.POINTER(d), d, C.POINTER(d), vp]
        L.or_integrate_f64.restype = i32
        L.or_advance.argtypes = [vp, i32, C.POINTER(Control), C.POINTER(LaneArrays), u32, u32, d, u32, u32]
        L.or_advance.restype = i32
        L.or_advance_mixed.argtypes = [vp, i32, C.POINTER(Control), C.POINTER(LaneArrays), u32, u32, d, u32, u32, u32]
        L.or_advance_mixed.restype = i32
        L.or_source_delta.argtypes = [vp, u32, d, d, vp]
        L.or_advect.argtypes = [vp, u32, u32, u32, vp, d, u32]
        L.or_fnv1a.argtypes = [vp, u64]
        L.or_fnv1a.restype = u64
        L.or_rate_block.argtypes = [vp, vp, vp, u32, u32, vp]
        L.or_workload_air.argtypes = [u64, u64, u32, u32, u32, d, d, d, d, vp, vp, vp]
        L.or_workload_air_power.argtypes = [u64, u64, u32, d, d, vp]
        _lib = L
    return _lib


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


class Mechanism:
    """A mechanism in the oracle's wide-index tables."""

    def __init__(self, handle=None):
        self.h = handle if handle is not None else lib().or_mech_new()

    @classmethod
    def air(cls) -> "Mechanism":
        return cls(lib().or_mech_new_air())

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.or_mech_free(self.h)
            self.h = None

    def add_species(self, name: str, abstract: bool = False) -> int:
        return lib().or_add_species(self.h, name.encode(), int(abstract))

    def add_reaction(self, equation: str, kind: str = "arr", params=(1.0, 0.0, 0.0), ref: int = 0) -> int:
        p = (C.c_double * 5)(*(list(params) + [0.0] * (5 - len(params))))
        return lib().or_add_reaction(self.h, equation.encode(), RATE_KIND[kind], p, ref)

    def finalize(self) -> None:
        lib().or_finalize(self.h)

    @property
    def error(self) -> str:
        return lib().or_error(self.h).decode()

    def counts(self) -> dict:
        c = (C.c_uint64 * 8)()
        lib().or_counts(self.h, c)
        keys = ("n", "R", "nnz", "pivots", "updates", "lower", "upper", "failed")
        return dict(zip(keys, [int(v) for v in c]))

    def kinmech(self):
        """(bytes, fnv1a) of the reference-layout KinMech, or (None, None) if it does not fit."""
        buf = np.zeros(KINMECH_BYTES, np.uint8)
        sig = C.c_uint64()
        ok = lib().or_export_kinmech(self.h, _ptr(buf), C.byref(sig))
        return (buf.tobytes(), int(sig.value)) if ok else (None, None)

    def pattern(self) -> np.ndarray:
        n = self.counts()["n"]
        out = np.zeros(n * n, np.uint8)
        lib().or_pattern(self.h, _ptr(out))
        return out.reshape(n, n)

    def lu_ops(self):
        c = self.counts()
        piv = np.zeros((max(c["pivots"], 1), 4), np.uint32)
        upd = np.zeros((max(c["updates"], 1), 2), np.uint32)
        lib().or_lu_ops(self.h, _ptr(piv), _ptr(upd))
        return piv[: c["pivots"]], upd[: c["updates"]]

    def rate_constants(self, T: float, M: float) -> np.ndarray:
        k = np.zeros(max(self.counts()["R"], 1))
        lib().or_rate_constants(self.h, T, M, _ptr(k))
        return k[: self.counts()["R"]]

    def fun(self, k, src, y) -> np.ndarray:
        f = np.zeros(len(y))
        lib().or_fun(self.h, _ptr(np.ascontiguousarray(k, np.float64)), _ptr(np.ascontiguousarray(src, np.float64)),
                     _ptr(np.ascontiguousarray(y, np.float64)), _ptr(f))
        return f

    def jac(self, k, y) -> np.ndarray:
        out = np.zeros(self.counts()["nnz"])
        lib().or_jac(self.h, _ptr(np.ascontiguousarray(k, np.float64)), _ptr(np.ascontiguousarray(y, np.float64)), _ptr(out))
        return out

    def decomp_solve(self, jac, ghinv, b):
        x = np.array(b, np.float64)
        lu = np.zeros(self.counts()["nnz"])
        lib().or_decomp_solve(self.h, _ptr(np.ascontiguousarray(jac, np.float64)), ghinv, _ptr(x), _ptr(lu))
        return x, lu

    def integrate(self, method: str, ctl: Control, k, src, y0, t_end: float, h0: float = 0.0):
        y = np.array(y0, np.float64)
        t = C.c_double(0.0)
        h = C.c_double(h0)
        stats = np.zeros(4)
        lib().or_integrate_f64(self.h, METHOD_IDS[method], C.byref(ctl), _ptr(np.ascontiguousarray(k, np.float64)),
                               _ptr(np.ascontiguousarray(src, np.float64)), _ptr(y), C.byref(t), t_end, C.byref(h),
                               _ptr(stats))
        return y, t.value, h.value, stats

    def advance(self, method: str, ctl: Control, block: dict, padded: int, begin: int, end: int, duration: float,
                precision: int = 0, threads: int = 0) -> None:
        la = lane_arrays(block, padded)
        rc = lib().or_advance(self.h, METHOD_IDS[method], C.byref(ctl), C.byref(la), begin, end, duration, precision,
                              threads)
        if rc != 0:
            raise RuntimeError(f"or_advance failed: {rc}")


def advance_mixed(mech: "Mechanism", method: str, ctl: Control, block: dict, padded: int, begin: int, end: int,
                  duration: float, sweeps: int = 1, variant: int = 0, threads: int = 0) -> None:
    """Model of the GPU module's mixed-precision path; used to check the GPU's mixed
    kernel bit for bit. variant 0: FP32 chemistry, FP64 residual refinement, FP64
    state and control; variant 1: double-float state, FP32 stage vectors / LU /
    solves, double-float stage right-hand sides."""
    la = lane_arrays(block, padded)
    rc = lib().or_advance_mixed(mech.h, METHOD_IDS[method], C.byref(ctl), C.byref(la), begin, end, duration, sweeps,
                                variant, threads)
    if rc != 0:
        raise RuntimeError(f"or_advance_mixed failed: {rc}")


def source_delta(y: np.ndarray, energy_J_cm3: float, T_K: float) -> np.ndarray:
    y = np.ascontiguousarray(y, np.float64)
    out = np.zeros(len(y))
    lib().or_source_delta(_ptr(y), len(y), energy_J_cm3, T_K, _ptr(out))
    return out


def advect(x: np.ndarray, inlet: np.ndarray, courant: float, substeps: int) -> None:
    """In place on a C-contiguous [species][cells] float64 block."""
    assert x.flags["C_CONTIGUOUS"] and x.dtype == np.float64
    inlet = np.ascontiguousarray(inlet, np.float64)
    lib().or_advect(_ptr(x), x.shape[0], x.shape[1], x.shape[1], _ptr(inlet), courant, substeps)


def air_block(cells: int, seed: int = 1, first_cell: int = 0, pad_to: int = 8, T=(288.0, 303.0),
              log10_c=(-12.0, -2.0), rates: str = "reference", source_P0: float = 0.0, source_decades: float = 3.0):
    """The shipped-mechanism workload as a zone block (dict of 64-byte aligned float64 rows,
    `padded` lanes), built without the GPU module: the same seeded draws as the module's
    workload generator, rate constants from the reference's own kin_eval_rate_constants
    (oracle/_ref) when rates == "reference" and it was built, else from the oracle's
    restatement of it. Padding lanes copy cell 0. Returns (block, padded, rates_used)."""
    n, R = 17, 44
    P = max(pad_to, (cells + pad_to - 1) // pad_to * pad_to)
    block = {"y": aligned_zeros((n, P)), "k": aligned_zeros((R, P)), "src": aligned_zeros((n, P)),
             "pulse": aligned_zeros((n, P))}
    for name in ("h", "steps", "rejects", "pulses", "failed", "period", "pulse_first", "pulse_count"):
        block[name] = aligned_zeros(P)
    T_v, M_v = np.zeros(P), np.zeros(P)
    lib().or_workload_air(seed, first_cell, cells, P, n, T[0], T[1], log10_c[0], log10_c[1], _ptr(block["y"]),
                          _ptr(T_v), _ptr(M_v))
    used = "reference" if rates == "reference" and ref_available() else "oracle"
    if used == "reference":
        ref().ref_air_rate_block(_ptr(T_v), _ptr(M_v), cells, P, _ptr(block["k"]))
    else:
        m = Mechanism.air()
        lib().or_rate_block(m.h, _ptr(T_v), _ptr(M_v), cells, P, _ptr(block["k"]))
    for i in range(cells, P):
        block["y"][:, i] = block["y"][:, 0]
        block["k"][:, i] = block["k"][:, 0]
        T_v[i] = T_v[0]
    if source_P0 > 0.0:   # the uneven-stiffness workload's averaged discharge source per second, every lane
        power = np.zeros(P)
        lib().or_workload_air_power(seed, first_cell, P, source_P0, source_decades, _ptr(power))
        for i in range(P):
            col = np.ascontiguousarray(block["y"][:, i])
            block["src"][:, i] = (ref_air_source_delta(col, power[i], T_v[i]) if used == "reference"
                                  else source_delta(col, power[i], T_v[i]))
    return block, P, used


def fnv1a(data: bytes) -> int:
    buf = np.frombuffer(data, np.uint8).copy()
    return int(lib().or_fnv1a(_ptr(buf), len(buf)))


# ---------------------------------------------------------------------------
# The reference's own CPU solver (only where oracle/_ref was built).

_ref = None
_ref_big = None


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def ref() -> C.CDLL:
    global _ref
    if _ref is None:
        L = C.CDLL(REF_LIB)
        vp, u32, i32, d, u64 = C.c_void_p, C.c_uint32, C.c_int32, C.c_double, C.c_uint64
        L.ref_kinmech_size.restype = u64
        L.ref_air_kinmech.argtypes = [vp, C.POINTER(u64), C.POINTER(u64)]
        L.ref_air_kinmech.restype = i32
        L.ref_air_rate_constants.argtypes = [d, d, vp]
        L.ref_air_source_delta.argtypes = [vp, d, d, vp]
        L.ref_air_advance.argtypes = [i32, C.POINTER(Control), C.POINTER(LaneArrays), u32, u32, d, i32]
        L.ref_air_advance.restype = i32
        L.ref_robertson.argtypes = [i32, C.POINTER(Control), d, vp, vp]
        L.ref_robertson.restype = i32
        L.ref_air_rate_block.argtypes = [vp, vp, u32, u32, vp]
        L.ref_dbd_run.argtypes = [vp, u32, u32, i32, u32, d, i32, d, C.POINTER(Control), u32, u32]
        L.ref_dbd_run.restype = i32
        L.ref_air_advance_threads.argtypes = [i32, C.POINTER(Control), C.POINTER(LaneArrays), u32, u32, d, u32]
        L.ref_air_advance_threads.restype = i32
        L.ref_gpu_load.argtypes = [C.c_char_p, u64]
        L.ref_gpu_load.restype = i32
        L.ref_dbd_hybrid_run.argtypes = [vp, u32, u32, i32, u32, d, i32, d, C.POINTER(Control), u32, u32, i32, vp, vp, vp]
        L.ref_dbd_hybrid_run.restype = i32
        _ref = L
    return _ref


def ref_air_kinmech():
    buf = np.zeros(KINMECH_BYTES, np.uint8)
    sig, gen = C.c_uint64(), C.c_uint64()
    assert ref().ref_air_kinmech(_ptr(buf), C.byref(sig), C.byref(gen)) == 1
    return buf.tobytes(), int(sig.value), int(gen.value)


def ref_air_rate_constants(T: float, M: float, R: int = 44) -> np.ndarray:
    k = np.zeros(R)
    ref().ref_air_rate_constants(T, M, _ptr(k))
    return k


def ref_air_source_delta(y, energy_J_cm3, T_K) -> np.ndarray:
    y = np.ascontiguousarray(y, np.float64)
    out = np.zeros(len(y))
    ref().ref_air_source_delta(_ptr(y), energy_J_cm3, T_K, _ptr(out))
    return out


REF_VARIANTS = {"f64x4_gen": 0, "f64x4_table": 1, "f64_table": 2, "f32x8_gen": 3, "f32_gen": 4}


def ref_air_advance(method: str, ctl: Control, block: dict, padded: int, begin: int, end: int, duration: float,
                    variant: str = "f64x4_gen") -> None:
    la = lane_arrays(block, padded)
    rc = ref().ref_air_advance(METHOD_IDS[method], C.byref(ctl), C.byref(la), begin, end, duration, REF_VARIANTS[variant])
    if rc != 0:
        raise RuntimeError(f"ref_air_advance: {rc}")


def ref_air_advance_threads(method: str, ctl: Control, block: dict, padded: int, begin: int, end: int,
                            duration: float, threads: int) -> None:
    """Lanes [begin, end) (multiples of 8) through the reference's production CPU path,
    dbd_advance_threads (f64x4 lanes, generated AirGenOps, ~4 lane chunks per thread),
    on `threads` host threads."""
    la = lane_arrays(block, padded)
    rc = ref().ref_air_advance_threads(METHOD_IDS[method], C.byref(ctl), C.byref(la), begin, end, duration, threads)
    if rc != 0:
        raise RuntimeError(f"ref_air_advance_threads: {rc}")


def ref_dbd_run(block: np.ndarray, count: int, padded: int, pulsed: bool, steps: int, dt: float, ctl: Control,
                chained: bool = False, residence_s: float = 0.0, threads: int = 1, f32_lanes: bool = False) -> None:
    """`steps` master steps of dt of the reference's own zone driver (prepare_source, f64x4
    generated advance, commit_pulses, plug flow when chained) on a float64 block in the
    reference's DbdZones layout, in place."""
    assert block.dtype == np.float64 and block.flags["C_CONTIGUOUS"]
    rc = ref().ref_dbd_run(block.ctypes.data, count, padded, 0 if pulsed else 1, steps, dt, int(chained), residence_s,
                           C.byref(ctl), threads, int(f32_lanes))
    if rc != 0:
        raise RuntimeError(f"ref_dbd_run: {rc}")


def ref_gpu_load(path: str, arena_bytes: int) -> None:
    """Loads a GPU module with the reference's own loader (platform/linux_gpu.cpp:7-31),
    which calls its gpu_init: do this in a process that has not initialised the module."""
    rc = ref().ref_gpu_load(path.encode(), arena_bytes)
    if rc != 0:
        raise RuntimeError(f"ref_gpu_load({path}): {rc}")


def ref_dbd_hybrid_run(block: np.ndarray, count: int, padded: int, pulsed: bool, steps: int, dt: float, ctl: Control,
                       threads: int, precision: int, force_split: int = -1, chained: bool = False,
                       residence_s: float = 0.0):
    """`steps` master steps of the reference's zone driver with its hybrid CPU+GPU advance
    (dbd.cpp:336-463) on the module loaded by ref_gpu_load, in place. Returns per-step arrays
    (split, step wall ms, GPU launch-to-completion ms)."""
    assert block.dtype == np.float64 and block.flags["C_CONTIGUOUS"]
    split = np.zeros(steps, np.uint32)
    step_ms = np.zeros(steps, np.float32)
    gpu_ms = np.zeros(steps, np.float32)
    rc = ref().ref_dbd_hybrid_run(block.ctypes.data, count, padded, 0 if pulsed else 1, steps, dt, int(chained),
                                  residence_s, C.byref(ctl), threads, precision, force_split, split.ctypes.data,
                                  step_ms.ctypes.data, gpu_ms.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"ref_dbd_hybrid_run: {rc}")
    return split, step_ms, gpu_ms


def ref_robertson(method: str, ctl: Control, t_end: float = 40.0):
    y = np.array([1.0, 0.0, 0.0])
    stats = np.zeros(4)
    ref().ref_robertson(METHOD_IDS[method], C.byref(ctl), t_end, _ptr(y), _ptr(stats))
    return y, stats


class RefBigMechanism:
    """The reference's builder with larger KIN_MAX_* capacities (u16 tables)."""

    def __init__(self):
        global _ref_big
        if _ref_big is None:
            L = C.CDLL(REF_BIG_LIB)
            vp, u32, i32, d, u64 = C.c_void_p, C.c_uint32, C.c_int32, C.c_double, C.c_uint64
            L.ref_big_new.restype = vp
            L.ref_big_free.argtypes = [vp]
            L.ref_big_add_species.argtypes = [vp, C.c_char_p, i32]
            L.ref_big_add_reaction.argtypes = [vp, C.c_char_p, i32, C.POINTER(d), i32]
            L.ref_big_finalize.argtypes = [vp]
            L.ref_big_error.argtypes = [vp]
            L.ref_big_error.restype = C.c_char_p
            L.ref_big_counts.argtypes = [vp, C.POINTER(u64)]
            L.ref_big_lu_ops.argtypes = [vp, vp, vp]
            L.ref_big_rate_constants.argtypes = [vp, d, d, vp]
            L.ref_big_advance.argtypes = [vp, i32, C.POINTER(Control), C.POINTER(LaneArrays), u32, u32, d, i32]
            L.ref_big_advance.restype = i32
            _ref_big = L
        self.L = _ref_big
        self.h = self.L.ref_big_new()

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ref_big_free(self.h)
            self.h = None

    def add_species(self, name, abstract=False):
        return self.L.ref_big_add_species(self.h, name.encode(), int(abstract))

    def add_reaction(self, equation, kind="arr", params=(1.0, 0.0, 0.0), ref=0):
        p = (C.c_double * 5)(*(list(params) + [0.0] * (5 - len(params))))
        return self.L.ref_big_add_reaction(self.h, equation.encode(), RATE_KIND[kind], p, ref)

    def finalize(self):
        self.L.ref_big_finalize(self.h)

    @property
    def error(self):
        return self.L.ref_big_error(self.h).decode()

    def counts(self):
        c = (C.c_uint64 * 8)()
        self.L.ref_big_counts(self.h, c)
        return dict(zip(("n", "R", "nnz", "pivots", "updates", "lower", "upper", "failed"), [int(v) for v in c]))

    def lu_ops(self):
        c = self.counts()
        piv = np.zeros((max(c["pivots"], 1), 4), np.uint32)
        upd = np.zeros((max(c["updates"], 1), 2), np.uint32)
        self.L.ref_big_lu_ops(self.h, _ptr(piv), _ptr(upd))
        return piv[: c["pivots"]], upd[: c["updates"]]

    def rate_constants(self, T, M):
        R = self.counts()["R"]
        k = np.zeros(max(R, 1))
        self.L.ref_big_rate_constants(self.h, T, M, _ptr(k))
        return k[:R]

    def advance(self, method, ctl, block, padded, begin, end, duration, variant=0):
        la = lane_arrays(block, padded)
        rc = self.L.ref_big_advance(self.h, METHOD_IDS[method], C.byref(ctl), C.byref(la), begin, end, duration, variant)
        if rc != 0:
            raise RuntimeError(f"ref_big_advance: {rc}")


# ---------------------------------------------------------------------------
# The reference's NFT channel system (oracle/_ref/libref_nft.so, only where the
# reference sources exist): nft_run, the window split at the transport, and
# nft_transport on caller arrays.

REF_NFT_LIB = os.path.join(HERE, "_ref", "libref_nft.so")
NFT_LANES, NFT_FIELDS = 8, 9
_ref_nft = None


def ref_nft_available() -> bool:
    return os.path.exists(REF_NFT_LIB)


def ref_nft() -> C.CDLL:
    global _ref_nft
    if _ref_nft is None:
        L = C.CDLL(REF_NFT_LIB)
        vp, u32, f32, u64 = C.c_void_p, C.c_uint32, C.c_float, C.c_uint64
        L.ref_nft_create.argtypes = [u32, f32, u32]
        L.ref_nft_create.restype = vp
        L.ref_nft_destroy.argtypes = [vp]
        L.ref_nft_info.argtypes = [vp, vp]
        L.ref_nft_run.argtypes = [vp, u32, u32]
        for name in ("ref_nft_window_prepare", "ref_nft_window_transport", "ref_nft_window_finish"):
            getattr(L, name).argtypes = [vp]
        L.ref_nft_window_inputs.argtypes = [vp, vp, vp]
        L.ref_nft_window_inputs.restype = u32
        L.ref_nft_group_arrays.argtypes = [vp, u32, vp]
        L.ref_nft_digest.argtypes = [vp]
        L.ref_nft_digest.restype = u64
        L.ref_nft_layout.argtypes = [vp]
        L.ref_nft_transport_arrays.argtypes = [vp, vp, vp, vp, vp, vp, u32, u32, u32, u32, vp, vp, u32, u32]
        _ref_nft = L
    return _ref_nft


def ref_nft_layout() -> dict:
    out = np.zeros(16, np.uint64)
    ref_nft().ref_nft_layout(out.ctypes.data)
    keys = ("lanes", "fields", "row_bytes", "hot_bytes", "cold_bytes", "site_bytes", "hot_c", "hot_kT", "hot_bT",
            "hot_ko", "cold_kw", "cold_kr", "cold_ge", "cold_ev", "site_drop", "site_removed")
    return {k: int(v) for k, v in zip(keys, out)}


class RefNftSystem:
    """A reference NftSystem (nft_init with nft_default_params, rails / length / plants set)."""

    def __init__(self, rails: int, rail_length_m: float = 0.0, plants_per_rail: int = 0):
        self.L = ref_nft()
        self.h = self.L.ref_nft_create(rails, rail_length_m, plants_per_rail)
        info = np.zeros(8, np.uint32)
        self.L.ref_nft_info(self.h, info.ctypes.data)
        (self.rails, self.groups, self.cells, self.sites, self.site_offset, self.site_stride, self.substeps,
         self.lanes) = (int(v) for v in info)
        self.layout = ref_nft_layout()

    def close(self):
        if self.h:
            self.L.ref_nft_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def run(self, windows: int, scalar_lanes: bool = False):
        self.L.ref_nft_run(self.h, windows, int(scalar_lanes))

    def prepare(self):
        self.L.ref_nft_window_prepare(self.h)

    def transport(self):
        self.L.ref_nft_window_transport(self.h)

    def finish(self):
        self.L.ref_nft_window_finish(self.h)

    def inputs(self):
        """This window's inlet ref[9], env (T_amb, radiant, e0, es_slope) and substeps."""
        ref = np.zeros(NFT_FIELDS, np.float32)
        env = np.zeros(4, np.float32)
        self.substeps = int(self.L.ref_nft_window_inputs(self.h, ref.ctypes.data, env.ctypes.data))
        return ref, env, self.substeps

    def digest(self) -> int:
        return int(self.L.ref_nft_digest(self.h))

    def group_views(self, g: int) -> dict:
        """numpy views (float32, no copy) of group g's arrays in the reference's layout."""
        ptrs = (C.c_void_p * 6)()
        self.L.ref_nft_group_arrays(self.h, g, ptrs)
        lay = self.layout

        def view(p, nbytes):
            return np.ctypeslib.as_array((C.c_float * (nbytes // 4)).from_address(p))

        return {"rows": view(ptrs[0], lay["row_bytes"] * self.cells),
                "hot": view(ptrs[1], lay["hot_bytes"] * self.cells),
                "cold": view(ptrs[2], lay["cold_bytes"] * self.cells),
                "sites": view(ptrs[3], lay["site_bytes"] * self.sites),
                "out_sum": view(ptrs[4], 4 * NFT_FIELDS * NFT_LANES),
                "evap_kg": view(ptrs[5], 4 * NFT_LANES)}


def ref_nft_transport_arrays(rows, hot, cold, sites, cells, sites_count, site_offset, site_stride, ref, env, substeps,
                             ieee: bool = False):
    """The reference's nft_transport<f32x8> of one group over float32 arrays (32-byte aligned),
    in place, in this host's denormal mode (ieee = False) or without it; returns
    (out_sum[9*8], evap_kg[8])."""
    for a in (rows, hot, cold, sites):
        assert a.dtype == np.float32 and a.ctypes.data % 32 == 0 and a.flags["C_CONTIGUOUS"]
    out_sum = np.zeros(NFT_FIELDS * NFT_LANES, np.float32)
    evap = np.zeros(NFT_LANES, np.float32)
    ref = np.ascontiguousarray(ref, np.float32)
    env = np.ascontiguousarray(env, np.float32)
    ref_nft().ref_nft_transport_arrays(rows.ctypes.data, hot.ctypes.data, cold.ctypes.data, sites.ctypes.data,
                                       out_sum.ctypes.data, evap.ctypes.data, cells, sites_count, site_offset,
                                       site_stride, ref.ctypes.data, env.ctypes.data, substeps, int(ieee))
    return out_sum, evap
