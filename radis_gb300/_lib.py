"""ctypes binding of ``libradisgb.so`` (the C ABI in include/radis_gb300.h).

The product path has no CPU fallback: if the library is missing or the CUDA
runtime cannot be loaded, every entry point raises ``NativeLibraryError``.
"""
from __future__ import annotations

import ctypes as C
import os
import weakref

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libradisgb.so")

RG_OK = 0
STATUS = {1: "RG_ERR_ARG", 2: "RG_ERR_CUDA", 3: "RG_ERR_OOM", 4: "RG_ERR_UNSORTED",
          5: "RG_ERR_RANGE", 6: "RG_ERR_TIMEOUT", 7: "RG_ERR_STATE"}

# every symbol the header declares (checked by the CPU test suite)
EXPORTS = [
    "rg_abi_version", "rg_last_error", "rg_ctx_create", "rg_ctx_destroy", "rg_lines_upload",
    "rg_lines_free", "rg_lines_count", "rg_plan_create", "rg_plan_free", "rg_plan_grid", "rg_grid_estimate",
    "rg_grid_skeleton",
    "rg_synthesize", "rg_synthesize_host", "rg_debug_ldm", "rg_plan_stage_times",
    "rg_server_create", "rg_server_submit", "rg_server_wait", "rg_server_stats_get", "rg_server_destroy",
    "rg_synthesize_static", "rg_backward", "rg_jvp", "rg_synthesize_quantities",
    "rg_synthesize_quantities_host", "rg_slit_convolve",
    "rg_lines_set_partition", "rg_partition_eval", "rg_plan_stage_times_gauss", "rg_plan_test_scatter_stall",
    "rg_test_flush_order",
    "rg_hitran_count", "rg_hitran_parse",
]


class NativeLibraryError(RuntimeError):
    pass


class RgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class LineArrays(C.Structure):
    _fields_ = [("n", C.c_int64), ("v0", C.c_void_p), ("s_ref", C.c_void_p),
                ("e_low", C.c_void_p), ("g_air", C.c_void_p), ("g_self", C.c_void_p),
                ("n_air", C.c_void_p), ("delta", C.c_void_p), ("iso", C.c_void_p)]


class HitranColumns(C.Structure):
    _fields_ = [("n", C.c_int64), ("id", C.c_void_p), ("iso", C.c_void_p)] + \
        [(k, C.c_void_p) for k in ("v0", "s_ref", "a", "g_air", "g_self", "e_low", "n_air", "delta", "gp", "gpp")]


class Isotopes(C.Structure):
    _fields_ = [("n_iso", C.c_int), ("molar_mass", C.c_double * 16), ("t_ref", C.c_double)]


class PlanDesc(C.Structure):
    _fields_ = [("vmin", C.c_double), ("dv", C.c_double), ("n_v", C.c_int64),
                ("dxG", C.c_double), ("dxL", C.c_double), ("n_G", C.c_int), ("n_L", C.c_int),
                ("folding_thresh", C.c_double), ("n_ft", C.c_int64), ("accumulator", C.c_int32),
                ("axes_window", C.c_int32), ("layout", C.c_int32), ("layout_tol", C.c_double)]


class Conditions(C.Structure):
    _fields_ = [("T", C.c_double), ("p_bar", C.c_double), ("x", C.c_double),
                ("q_ratio", C.c_void_p)]


class Grid(C.Structure):
    _fields_ = [("log_wG_min", C.c_double), ("dxG", C.c_double), ("log_wL_min", C.c_double),
                ("dxL", C.c_double), ("n_G", C.c_int), ("n_L", C.c_int), ("n_ft", C.c_int64),
                ("n1", C.c_int64), ("n2", C.c_int64)]

    def axes(self):
        """(log_wG_min, dxG, N_G, log_wL_min, dxL, N_L) as the oracle takes them."""
        return (self.log_wG_min, self.dxG, self.n_G, self.log_wL_min, self.dxL, self.n_L)


class SpectrumInfo(C.Structure):
    _fields_ = [("grid", Grid), ("log_scale", C.c_double), ("stage_ms", C.c_float * 6),
                ("lines_in_window", C.c_int64), ("fft_rows", C.c_int32), ("merged_rows", C.c_int32),
                ("merged_ext", C.c_int32), ("gauss_ms", C.c_float), ("accum_bits", C.c_int32),
                ("layout", C.c_int32), ("layout_err", C.c_float)]


class Request(C.Structure):
    _fields_ = [("lines", C.c_void_p), ("grid", PlanDesc), ("cond", Conditions), ("out_host", C.c_void_p)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("failed", C.c_int64),
                ("in_flight", C.c_int64), ("queued", C.c_int64), ("device_bytes", C.c_int64),
                ("host_need_ms", C.c_double), ("host_launch_ms", C.c_double), ("host_copy_ms", C.c_double)]


_lib = None


def load(path: str | None = None):
    """Load (once) and return the native library; raise loudly if absent."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise NativeLibraryError(
            f"{p} is missing: build it with `python -m radis_gb300._build` "
            "(there is no CPU fallback for the synthesis path)")
    try:
        lib = C.CDLL(p)
    except OSError as e:   # e.g. libcudart.so.13 not found
        raise NativeLibraryError(f"cannot load {p}: {e}") from e
    vp, i64 = C.c_void_p, C.c_int64
    sig = {
        "rg_abi_version": ([], C.c_int),
        "rg_last_error": ([], C.c_char_p),
        "rg_ctx_create": ([C.c_int, C.POINTER(vp)], C.c_int),
        "rg_ctx_destroy": ([vp], C.c_int),
        "rg_lines_upload": ([vp, C.POINTER(LineArrays), C.POINTER(Isotopes), C.POINTER(vp)], C.c_int),
        "rg_lines_free": ([vp], C.c_int),
        "rg_lines_count": ([vp, C.POINTER(i64)], C.c_int),
        "rg_plan_create": ([vp, C.POINTER(PlanDesc), C.POINTER(vp)], C.c_int),
        "rg_plan_free": ([vp], C.c_int),
        "rg_plan_grid": ([vp, C.POINTER(Conditions), C.POINTER(Grid)], C.c_int),
        "rg_grid_estimate": ([C.POINTER(LineArrays), C.POINTER(Isotopes), C.POINTER(PlanDesc),
                              C.POINTER(Conditions), C.POINTER(Grid)], C.c_int),
        "rg_grid_skeleton": ([C.POINTER(Grid), C.c_double, C.c_double, C.c_double, C.c_int32,
                              C.POINTER(C.c_int32), vp, vp, C.POINTER(C.c_double)], C.c_int),
        "rg_synthesize": ([vp, C.POINTER(Conditions), vp, vp, C.c_int, C.POINTER(SpectrumInfo)], C.c_int),
        "rg_synthesize_host": ([vp, C.POINTER(Conditions), vp, vp, C.c_int, C.POINTER(SpectrumInfo)],
                               C.c_int),
        "rg_plan_stage_times": ([vp, C.POINTER(C.c_double), C.POINTER(i64)], C.c_int),
        "rg_plan_stage_times_gauss": ([vp, C.POINTER(C.c_double)], C.c_int),
        "rg_plan_test_scatter_stall": ([vp, C.c_int32, i64], C.c_int),
        "rg_test_flush_order": ([C.c_int32, vp, vp, C.c_int32, C.POINTER(C.c_int32)], C.c_int),
        "rg_debug_ldm": ([vp, C.POINTER(Conditions), vp, i64, C.POINTER(SpectrumInfo)], C.c_int),
        "rg_server_create": ([vp, C.c_int, i64, C.POINTER(vp)], C.c_int),
        "rg_server_submit": ([vp, C.POINTER(Request), C.POINTER(i64)], C.c_int),
        "rg_server_wait": ([vp, i64, C.c_double, C.POINTER(SpectrumInfo), C.POINTER(C.c_double),
                            C.POINTER(C.c_double), C.POINTER(C.c_double)], C.c_int),
        "rg_server_stats_get": ([vp, C.POINTER(ServerStats)], C.c_int),
        "rg_server_destroy": ([vp], C.c_int),
        "rg_synthesize_static": ([vp, C.POINTER(PlanDesc), C.POINTER(Conditions), vp, vp,
                                  C.POINTER(SpectrumInfo)], C.c_int),
        "rg_backward": ([vp, C.POINTER(Conditions), vp, vp, C.POINTER(C.c_double), vp,
                         C.POINTER(SpectrumInfo)], C.c_int),
        "rg_jvp": ([vp, C.POINTER(Conditions), vp, vp, vp, C.POINTER(SpectrumInfo)], C.c_int),
        "rg_synthesize_quantities": ([vp, C.POINTER(Conditions), C.c_double, vp, vp, C.POINTER(SpectrumInfo)],
                                     C.c_int),
        "rg_synthesize_quantities_host": ([vp, C.POINTER(Conditions), C.c_double, vp, vp, C.c_int,
                                           C.POINTER(SpectrumInfo)], C.c_int),
        "rg_slit_convolve": ([vp, vp, i64, vp, C.c_int32, C.c_double, C.c_int32, vp, vp], C.c_int),
        "rg_lines_set_partition": ([vp, C.c_int32, i64, vp, vp, C.c_int32], C.c_int),
        "rg_partition_eval": ([i64, vp, vp, C.c_int32, C.c_double, C.POINTER(C.c_double),
                               C.POINTER(C.c_double)], C.c_int),
        "rg_hitran_count": ([vp, i64, C.c_int32, C.POINTER(i64)], C.c_int),
        "rg_hitran_parse": ([vp, i64, C.c_int32, C.POINTER(HitranColumns)], C.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def check(code: int):
    if code != RG_OK:
        msg = load().rg_last_error()
        raise RgError(code, msg.decode() if msg else "")


def ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


PARTITION_KINDS = {"linear": 0, "cubic": 1}   # RG_Q_LINEAR, RG_Q_CUBIC


def partition_eval(T, Q, kind: str, t: float):
    """Host-only rg_partition_eval: (Q(t), dQ/dT(t)) of a table."""
    T = np.ascontiguousarray(T, dtype=np.float64)
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    q, dq = C.c_double(), C.c_double()
    check(load().rg_partition_eval(len(T), ptr(T), ptr(Q), PARTITION_KINDS[kind], float(t), C.byref(q),
                                   C.byref(dq)))
    return q.value, dq.value


# HitranColumns field -> column name of the line dicts used in this package
HITRAN_COLUMNS = {"id": "id", "iso": "iso", "v0": "v0", "s_ref": "S_ref", "a": "A", "g_air": "g_air",
                  "g_self": "g_self", "e_low": "El", "n_air": "n_air", "delta": "delta", "gp": "gp",
                  "gpp": "gpp"}


def hitran_parse(text, threads: int = 0, columns=None) -> dict:
    """Host-only rg_hitran_count + rg_hitran_parse over the bytes of a
    HITRAN-160 file (any 1-D uint8 buffer).  Returns {name: array}: id and iso
    int64, the rest float64; ``columns`` restricts the columns converted."""
    buf = np.frombuffer(text, dtype=np.uint8) if not isinstance(text, np.ndarray) else text
    if buf.ndim != 1 or buf.dtype != np.uint8 or not buf.flags.c_contiguous:
        raise ValueError("text must be a contiguous 1-D uint8 buffer")
    lib = load()
    addr = buf.ctypes.data_as(C.c_void_p) if buf.size else None
    n = C.c_int64()
    check(lib.rg_hitran_count(addr, buf.size, int(threads), C.byref(n)))
    want = HITRAN_COLUMNS if columns is None else {k: v for k, v in HITRAN_COLUMNS.items() if v in columns}
    out = {}
    cols = HitranColumns(n=n.value)
    for field, name in want.items():
        a = np.empty(n.value, dtype=np.int32 if field in ("id", "iso") else np.float64)
        out[name] = a
        setattr(cols, field, a.ctypes.data_as(C.c_void_p).value if n.value else None)
    check(lib.rg_hitran_parse(addr, buf.size, int(threads), C.byref(cols)))
    for k in ("id", "iso"):
        if k in out:
            out[k] = out[k].astype(np.int64)
    return out


class Context:
    """One device and its stream (rg_ctx)."""

    def __init__(self, device: int = 0):
        lib = load()
        h = C.c_void_p()
        check(lib.rg_ctx_create(int(device), C.byref(h)))
        self._h = h
        self.device = device
        self._children = weakref.WeakSet()

    @property
    def handle(self):
        if not self._h:
            raise RgError(7, "context is closed")
        return self._h

    def slit_convolve(self, in_dev_ptr: int, n: int, slit_dev_ptr: int, n_slit: int, wstep: float,
                      valid: bool, out_dev_ptr: int, stream_ptr: int | None = None):
        """rg_slit_convolve: out = wstep * (in conv slit)['same'] on the device,
        NaN on the boundary points when ``valid``."""
        check(load().rg_slit_convolve(self.handle, C.c_void_p(in_dev_ptr), int(n), C.c_void_p(slit_dev_ptr),
                                      int(n_slit), float(wstep), 1 if valid else 0, C.c_void_p(out_dev_ptr),
                                      C.c_void_p(stream_ptr) if stream_ptr else None))

    def close(self):
        """Close the line lists (and their plans) still open, then the context."""
        if getattr(self, "_h", None):
            for child in list(self._children):
                child.close()
            check(load().rg_ctx_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Lines:
    """Device-resident line list (rg_lines).  Arrays are copied at construction;
    v0 must be ascending (sort with ``sort_lines`` first)."""

    COLS = ("v0", "S_ref", "El", "g_air", "g_self", "n_air", "delta", "iso")

    def __init__(self, ctx: Context, lines: dict, molar_mass, t_ref: float = 296.0):
        lib = load()
        self.ctx = ctx
        self._keep = dict(
            v0=np.ascontiguousarray(lines["v0"], dtype=np.float64),
            s=np.ascontiguousarray(lines["S_ref"], dtype=np.float64),
            el=np.ascontiguousarray(lines["El"], dtype=np.float32),
            ga=np.ascontiguousarray(lines["g_air"], dtype=np.float32),
            gs=np.ascontiguousarray(lines["g_self"], dtype=np.float32),
            na=np.ascontiguousarray(lines["n_air"], dtype=np.float32),
        )
        k = self._keep
        d = lines.get("delta")
        k["dl"] = None if d is None else np.ascontiguousarray(d, dtype=np.float32)
        iso = lines.get("iso")
        k["iso"] = None if iso is None else np.ascontiguousarray(iso, dtype=np.uint8)
        mm = np.atleast_1d(np.asarray(molar_mass, dtype=np.float64))
        self.n_iso = len(mm)
        la = LineArrays(len(k["v0"]), ptr(k["v0"]), ptr(k["s"]), ptr(k["el"]), ptr(k["ga"]),
                        ptr(k["gs"]), ptr(k["na"]), ptr(k["dl"]), ptr(k["iso"]))
        iso_s = Isotopes()
        iso_s.n_iso = self.n_iso
        for i, m in enumerate(mm):
            iso_s.molar_mass[i] = float(m)
        iso_s.t_ref = float(t_ref)
        h = C.c_void_p()
        check(lib.rg_lines_upload(ctx.handle, C.byref(la), C.byref(iso_s), C.byref(h)))
        self._h = h
        self._children = weakref.WeakSet()
        ctx._children.add(self)
        self.n = len(k["v0"])
        self.molar_mass = mm
        self.t_ref = t_ref
        self._keep = None   # host copies no longer needed

    @property
    def handle(self):
        if not self._h:
            raise RgError(7, "line list is closed")
        return self._h

    def set_partition(self, iso: int, T, Q, kind: str = "cubic"):
        """Tabulated Q(T) of isotopologue ``iso`` (rg_lines_set_partition):
        'cubic' (CDSD-style spline) or 'linear' (np.interp).  With a table for
        every isotopologue, q_ratio=None means Q(Tref)/Q(T) from the tables."""
        T = np.ascontiguousarray(T, dtype=np.float64)
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        if T.shape != Q.shape or T.ndim != 1:
            raise ValueError("T and Q must be 1-D arrays of the same length")
        check(load().rg_lines_set_partition(self.handle, int(iso), len(T), ptr(T), ptr(Q), PARTITION_KINDS[kind]))

    def close(self):
        """Close the plans still open on this list, then the list."""
        if getattr(self, "_h", None):
            for child in list(self._children):
                child.close()
            check(load().rg_lines_free(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Plan:
    """Spectral grid + workspace over one line list (rg_plan)."""

    def __init__(self, lines: Lines, vmin: float, dv: float, n_v: int, dxG=None, dxL=None,
                 n_G=None, n_L=None, folding_thresh: float = 1e-6, n_ft: int = 0, accumulator: int = 0,
                 axes_window: bool = False, layout: int = 0, layout_tol: float = 0.0):
        """``accumulator``: fixed-point width of the scatter (0: from the
        densest grid column, 32 or 64: forced).  ``axes_window``: the Gaussian
        node axis spans only the lines that can reach the window (instead of
        the whole list).  ``layout``: rows of the FFT stage (0: the fewest,
        1: node rows, 2: merged rows where possible, 3: skeleton rows where
        possible); ``layout_tol``: the skeleton decomposition's error bound
        (0: 1e-8)."""
        lib = load()
        self.lines = lines
        d = PlanDesc(float(vmin), float(dv), int(n_v), float(dxG or 0.0), float(dxL or 0.0),
                     int(n_G or 0), int(n_L or 0), float(folding_thresh), int(n_ft), int(accumulator),
                     1 if axes_window else 0, int(layout), float(layout_tol))
        h = C.c_void_p()
        check(lib.rg_plan_create(lines.handle, C.byref(d), C.byref(h)))
        self._h = h
        lines._children.add(self)
        self.vmin, self.dv, self.n_v = float(vmin), float(dv), int(n_v)

    @property
    def handle(self):
        if not self._h:
            raise RgError(7, "plan is closed")
        return self._h

    def _cond(self, T, p_bar, x, q_ratio):
        if q_ratio is None:
            return Conditions(float(T), float(p_bar), float(x), None), None
        q = None
        if q_ratio is not None:
            q = np.ascontiguousarray(np.broadcast_to(np.asarray(q_ratio, np.float64),
                                                     (self.lines.n_iso,)))
        return Conditions(float(T), float(p_bar), float(x), ptr(q)), q

    def grid(self, T, p_bar, x, q_ratio=None) -> Grid:
        c, _q = self._cond(T, p_bar, x, q_ratio)
        g = Grid()
        check(load().rg_plan_grid(self.handle, C.byref(c), C.byref(g)))
        return g

    def synthesize_host(self, T, p_bar, x, q_ratio=None, out=None, timing=False):
        """Blocking: returns (float32 array n_v, SpectrumInfo); abscoeff in cm-1
        is ``out * exp(info.log_scale)``; ``timing`` fills info.stage_ms."""
        c, _q = self._cond(T, p_bar, x, q_ratio)
        if out is None:
            out = np.empty(self.n_v, dtype=np.float32)
        elif out.dtype != np.float32 or not out.flags.c_contiguous or out.size < self.n_v:
            raise ValueError(f"out must be a C-contiguous float32 array of >= {self.n_v} values")
        info = SpectrumInfo()
        rc = load().rg_synthesize_host(self.handle, C.byref(c), out.ctypes.data, None, 1 if timing else 0,
                                       C.byref(info))
        if rc != RG_OK:
            check(rc)
        return out, info

    def synthesize_device(self, T, p_bar, x, out_dev_ptr: int, stream_ptr: int | None = None,
                          q_ratio=None, timing: int = 0):
        """Enqueue on a caller stream into a caller device buffer (n_v floats).
        timing: 0 none, 1 synchronous per-stage times in the returned info,
        2 per-stage events into the plan's ring (read with ``stage_times``)."""
        c, _q = self._cond(T, p_bar, x, q_ratio)
        info = SpectrumInfo()
        check(load().rg_synthesize(self.handle, C.byref(c), C.c_void_p(out_dev_ptr),
                                   C.c_void_p(stream_ptr) if stream_ptr else None,
                                   int(timing), C.byref(info)))
        return info

    def _dlnq(self, dlnq_dT):
        if dlnq_dT is None:
            return None
        return np.ascontiguousarray(np.broadcast_to(np.asarray(dlnq_dT, np.float64), (self.lines.n_iso,)))

    def backward(self, T, p_bar, x, grad_out_dev_ptr: int, q_ratio=None, dlnq_dT=None,
                 stream_ptr: int | None = None):
        """Reverse mode: sum_k g[k] d abscoeff_k / d(T, p_bar, x) for the n_v
        floats g at ``grad_out_dev_ptr`` (node axes fixed at these conditions).
        ``dlnq_dT``: d ln(Q(Tref)/Q(T))/dT per isotopologue.  Blocking; returns
        a float64 array of 3."""
        c, _q = self._cond(T, p_bar, x, q_ratio)
        dq = self._dlnq(dlnq_dT)
        out = (C.c_double * 3)()
        check(load().rg_backward(self.handle, C.byref(c), ptr(dq), C.c_void_p(grad_out_dev_ptr), out,
                                 C.c_void_p(stream_ptr) if stream_ptr else None, None))
        return np.array(list(out))

    def jvp(self, T, p_bar, x, out_dev_ptr: int, q_ratio=None, dlnq_dT=None, stream_ptr: int | None = None):
        """Forward mode: enqueue d abscoeff / d(T, p_bar, x) x exp(-info.log_scale)
        into 3 rows of n_v floats at ``out_dev_ptr``; returns the info."""
        c, _q = self._cond(T, p_bar, x, q_ratio)
        dq = self._dlnq(dlnq_dT)
        info = SpectrumInfo()
        check(load().rg_jvp(self.handle, C.byref(c), ptr(dq), C.c_void_p(out_dev_ptr),
                            C.c_void_p(stream_ptr) if stream_ptr else None, C.byref(info)))
        return info

    def synthesize_quantities(self, T, p_bar, x, path_length, out_dev_ptr: int, stream_ptr: int | None = None,
                              q_ratio=None):
        """Enqueue the spectrum and the device post-processing into 5 rows of
        n_v floats at ``out_dev_ptr``: abscoeff, absorbance (both x
        exp(-info.log_scale)), emissivity, transmittance, radiance."""
        c, _q = self._cond(T, p_bar, x, q_ratio)
        info = SpectrumInfo()
        check(load().rg_synthesize_quantities(self.handle, C.byref(c), float(path_length),
                                              C.c_void_p(out_dev_ptr),
                                              C.c_void_p(stream_ptr) if stream_ptr else None, C.byref(info)))
        return info

    QUANTITIES = ("abscoeff", "absorbance", "emissivity_noslit", "transmittance_noslit", "radiance_noslit")

    def synthesize_quantities_host(self, T, p_bar, x, path_length, q_ratio=None, timing=False, out=None):
        """Blocking: ({quantity: float32 array n_v}, SpectrumInfo) with the
        post-processing fused into the spectrum's last kernel.  abscoeff and
        absorbance are in units of exp(info.log_scale); emissivity,
        transmittance and radiance (mW/cm2/sr/nm) in physical units.  ``out``:
        optional float32 buffer of 5 n_v (page-locked memory is written by the
        kernel itself)."""
        c, _q = self._cond(T, p_bar, x, q_ratio)
        if out is None:
            out = np.empty(5 * self.n_v, dtype=np.float32)
        info = SpectrumInfo()
        check(load().rg_synthesize_quantities_host(self.handle, C.byref(c), float(path_length), ptr(out), None,
                                                   1 if timing else 0, C.byref(info)))
        rows = out.reshape(5, self.n_v)
        return {k: rows[i] for i, k in enumerate(self.QUANTITIES)}, info

    def test_scatter_stall(self, withhold: bool, wait_cycles: int = 0):
        """Test hook (rg_plan_test_scatter_stall): with ``withhold`` the next
        spectra's scatter receives no line copies and its bounded waits run
        out (RG_ERR_TIMEOUT); ``wait_cycles`` bounds those waits (0: default)."""
        check(load().rg_plan_test_scatter_stall(self.handle, 1 if withhold else 0, int(wait_cycles)))

    def gauss_time(self):
        """Gaussian-stage part (ms, summed) of the fft-col sum that the last
        ``stage_times`` call returned (merged layout; 0 otherwise)."""
        g = C.c_double()
        check(load().rg_plan_stage_times_gauss(self.handle, C.byref(g)))
        return g.value

    def stage_times(self):
        """(sum of ms per stage [scatter, fft-col, fft-row+voigt, ifft-row,
        ifft-col, total], count) of spectra enqueued with timing=2."""
        s = (C.c_double * 6)()
        n = C.c_int64()
        check(load().rg_plan_stage_times(self.handle, s, C.byref(n)))
        return list(s), n.value

    def debug_ldm(self, T, p_bar, x, q_ratio=None):
        """Scatter only; returns (LDM [N_G, N_L, n_v] float32, info)."""
        c, _q = self._cond(T, p_bar, x, q_ratio)
        g = self.grid(T, p_bar, x, q_ratio)
        buf = np.empty(g.n_G * g.n_L * self.n_v, dtype=np.float32)
        info = SpectrumInfo()
        check(load().rg_debug_ldm(self.handle, C.byref(c), ptr(buf), buf.size, C.byref(info)))
        return buf.reshape(g.n_G, g.n_L, self.n_v), info

    def close(self):
        if getattr(self, "_h", None):
            check(load().rg_plan_free(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def sort_lines(lines: dict) -> dict:
    """Stable sort of a column dict by v0 (the CPU path sorts by shiftwav with
    mergesort, radis/lbl/base.py:2370; the GPU kernels need v0 order)."""
    v0 = np.asarray(lines["v0"])
    if np.all(v0[1:] >= v0[:-1]):
        return lines
    order = np.argsort(v0, kind="stable")
    return {k: (np.asarray(v)[order] if v is not None and np.ndim(v) == 1 and len(v) == len(v0) else v)
            for k, v in lines.items()}


def _line_arrays(lines: dict):
    keep = dict(
        v0=np.ascontiguousarray(lines["v0"], dtype=np.float64),
        s=np.ascontiguousarray(lines["S_ref"], dtype=np.float64),
        el=np.ascontiguousarray(lines["El"], dtype=np.float32),
        ga=np.ascontiguousarray(lines["g_air"], dtype=np.float32),
        gs=np.ascontiguousarray(lines["g_self"], dtype=np.float32),
        na=np.ascontiguousarray(lines["n_air"], dtype=np.float32))
    d, iso = lines.get("delta"), lines.get("iso")
    keep["dl"] = None if d is None else np.ascontiguousarray(d, dtype=np.float32)
    keep["iso"] = None if iso is None else np.ascontiguousarray(iso, dtype=np.uint8)
    la = LineArrays(len(keep["v0"]), ptr(keep["v0"]), ptr(keep["s"]), ptr(keep["el"]),
                    ptr(keep["ga"]), ptr(keep["gs"]), ptr(keep["na"]), ptr(keep["dl"]),
                    ptr(keep["iso"]))
    return la, keep


def grid_estimate(lines: dict, molar_mass, vmin, dv, n_v, T, p_bar, x, dxG=None, dxL=None,
                  n_G=None, n_L=None, t_ref=296.0, q_ratio=None, n_ft=0, axes_window=False) -> Grid:
    """Host-only (no GPU): the LDM grid a plan would use (rg_grid_estimate)."""
    la, keep = _line_arrays(lines)
    mm = np.atleast_1d(np.asarray(molar_mass, dtype=np.float64))
    iso_s = Isotopes()
    iso_s.n_iso = len(mm)
    for i, m in enumerate(mm):
        iso_s.molar_mass[i] = float(m)
    iso_s.t_ref = float(t_ref)
    d = PlanDesc(float(vmin), float(dv), int(n_v), float(dxG or 0.0), float(dxL or 0.0),
                 int(n_G or 0), int(n_L or 0), 1e-6, int(n_ft), 0, 1 if axes_window else 0)
    q = None if q_ratio is None else np.ascontiguousarray(
        np.broadcast_to(np.asarray(q_ratio, np.float64), (len(mm),)))
    c = Conditions(float(T), float(p_bar), float(x), ptr(q))
    g = Grid()
    check(load().rg_grid_estimate(C.byref(la), C.byref(iso_s), C.byref(d), C.byref(c), C.byref(g)))
    return g


def grid_skeleton(grid: Grid, dv: float, folding_thresh: float = 1e-6, tol: float = 0.0, r_max: int = 64):
    """Host-only (no GPU): the skeleton layout of a node grid
    (rg_grid_skeleton).  Returns (nodes int32[R], coef float64[R, n_G n_L],
    largest sampled error)."""
    n = int(grid.n_G) * int(grid.n_L)
    r_max = max(1, min(int(r_max), n))
    nodes = np.zeros(r_max, np.int32)
    coef = np.zeros((r_max, n), np.float64)
    R, err = C.c_int32(), C.c_double()
    check(load().rg_grid_skeleton(C.byref(grid), float(dv), float(folding_thresh), float(tol), r_max,
                                  C.byref(R), nodes.ctypes.data, coef.ctypes.data, C.byref(err)))
    return nodes[:R.value].copy(), coef[:R.value].copy(), err.value


def flush_order(n_nodes: int):
    """Host-only test hook (rg_test_flush_order): the node order in which the
    scatter's flush projects a tile on the tensor cores, as (nodes int32[8 S],
    real bool[8 S]) for S steps of 8 nodes."""
    cap = 8 * ((int(n_nodes) + 7) // 8 + 64)
    nodes = np.zeros(cap, np.int32)
    real = np.zeros(cap, np.uint8)
    cnt = C.c_int32()
    check(load().rg_test_flush_order(int(n_nodes), nodes.ctypes.data, real.ctypes.data, cap, C.byref(cnt)))
    return nodes[:cnt.value].copy(), real[:cnt.value].astype(bool)


class Server:
    """Continuous-batching spectrum server over resident line lists
    (rg_server_*): ``submit`` queues a request and returns a ticket at once;
    the native worker admits requests into CUDA stream slots as slots and
    device memory free up; ``wait`` returns the spectrum."""

    def __init__(self, ctx: Context, slots: int = 8, mem_budget: int = 16 << 30):
        h = C.c_void_p()
        check(load().rg_server_create(ctx.handle, int(slots), int(mem_budget), C.byref(h)))
        self._h = h
        self.ctx = ctx
        self._keep = {}
        ctx._children.add(self)

    @property
    def handle(self):
        if not self._h:
            raise RgError(7, "server is closed")
        return self._h

    def submit(self, lines: Lines, vmin, dv, n_v, T, p_bar, x, dxG=None, dxL=None, n_G=None,
               n_L=None, q_ratio=None, out=None, folding_thresh=1e-6, accumulator=0, axes_window=False,
               layout=0, layout_tol=0.0) -> int:
        if out is None:
            out = np.empty(int(n_v), dtype=np.float32)
        q = None if q_ratio is None else np.ascontiguousarray(
            np.broadcast_to(np.asarray(q_ratio, np.float64), (lines.n_iso,)))
        req = Request(lines.handle.value,
                      PlanDesc(float(vmin), float(dv), int(n_v), float(dxG or 0.0), float(dxL or 0.0),
                               int(n_G or 0), int(n_L or 0), float(folding_thresh), 0, int(accumulator),
                               1 if axes_window else 0, int(layout), float(layout_tol)),
                      Conditions(float(T), float(p_bar), float(x), ptr(q)), out.ctypes.data)
        t = C.c_int64()
        check(load().rg_server_submit(self.handle, C.byref(req), C.byref(t)))
        self._keep[t.value] = (out, q, lines)
        return t.value

    def wait(self, ticket: int, timeout_ms: float = -1.0):
        """(spectrum float32 array, SpectrumInfo, (t_submit, t_start, t_done))."""
        info = SpectrumInfo()
        ts, t0, t1 = C.c_double(), C.c_double(), C.c_double()
        try:
            check(load().rg_server_wait(self.handle, int(ticket), float(timeout_ms), C.byref(info),
                                        C.byref(ts), C.byref(t0), C.byref(t1)))
        finally:
            kept = self._keep.pop(ticket, None)
        return kept[0], info, (ts.value, t0.value, t1.value)

    def stats(self) -> ServerStats:
        st = ServerStats()
        check(load().rg_server_stats_get(self.handle, C.byref(st)))
        return st

    def close(self):
        if getattr(self, "_h", None):
            check(load().rg_server_destroy(self._h))
            self._h = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def synthesize_static(lines: Lines, vmin, dv, n_v, T, p_bar, x, out_dev_ptr: int, dxG=None, dxL=None,
                      n_G=None, n_L=None, q_ratio=None, stream_ptr: int | None = None,
                      folding_thresh=1e-6, accumulator=0, axes_window=False) -> SpectrumInfo:
    """Allocation-free spectrum (rg_synthesize_static): every scratch buffer
    comes from the library's static 64 MiB device array, so nothing is
    allocated on the device during the call.  ``out_dev_ptr``: caller-owned
    device buffer of n_v floats.  Blocking."""
    d = PlanDesc(float(vmin), float(dv), int(n_v), float(dxG or 0.0), float(dxL or 0.0),
                 int(n_G or 0), int(n_L or 0), float(folding_thresh), 0, int(accumulator),
                 1 if axes_window else 0)
    q = None if q_ratio is None else np.ascontiguousarray(
        np.broadcast_to(np.asarray(q_ratio, np.float64), (lines.n_iso,)))
    c = Conditions(float(T), float(p_bar), float(x), ptr(q))
    info = SpectrumInfo()
    check(load().rg_synthesize_static(lines.handle, C.byref(d), C.byref(c), C.c_void_p(out_dev_ptr),
                                      C.c_void_p(stream_ptr) if stream_ptr else None, C.byref(info)))
    return info
