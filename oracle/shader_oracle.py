"""Second oracle: the reference's GPU (Vulkan) path restated on the CPU --
TEST INFRASTRUCTURE ONLY (imported by ``tests/``).

``shader_oracle.c`` restates the arithmetic of the two compute shaders
(radis/gpu/vulkan/shaders/cmdFillLDM.comp:75-145 and
cmdApplyLineshapes.comp:51-90) in FP32, as they run, and in FP64; the FFTs
around them (VkFFT in the reference, radis/gpu/gpu.py:268,277) are scipy's
rfft/irfft in the same precision.  The host scalars follow
radis/gpu/params.py:123-155 (set_pTQ) with the node axes given explicitly.

Conventions can be taken from the reference's CPU path instead of its GPU
path (``cpu_conventions=True``): pressure in atm in the shift and the widths
(radis/lbl/broadening.py:1063), the CPU Doppler constant (k_b in CGS,
radis/phys/constants.py:75) and the number density of
radis/lbl/factory.py:908-912.  The intensity is always given as S_ref and
converted to the Einstein-A based S0 the shader takes (with Q(Tref) = 1:
S0 = S_ref exp(c2 El / Tref) / (1 - exp(-c2 v0 / Tref)), Q(T) = 1 / Qratio),
which is the same intensity.  With CPU conventions the FP64 build equals the
FP64 CPU oracle up to rounding, so the FP32 build measures the FP32 error of
the reference's GPU design alone.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

from . import ldm_oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "shader_oracle.c")
LIB = os.path.join(HERE, "libshader_oracle.so")
KB_SCIPY = 1.380649e-23 * 1e7   # erg/K: the GPU path's Boltzmann constant (radis/gpu/gpu.py:5,146)

_lib = None


class Params(C.Structure):
    _fields_ = [("v_min", C.c_double), ("dv", C.c_double), ("n_v", C.c_int64), ("n_row", C.c_int64),
                ("dxG", C.c_double), ("dxL", C.c_double), ("log_wG_min", C.c_double), ("log_wL_min", C.c_double),
                ("n_G", C.c_int32), ("n_L", C.c_int32), ("p", C.c_double), ("log_2p", C.c_double),
                ("hlog_T", C.c_double), ("log_rT", C.c_double), ("c2T", C.c_double), ("N", C.c_double),
                ("x_self", C.c_double), ("x_air", C.c_double), ("log_c2Mm", C.c_double * 16),
                ("Q", C.c_double * 16)]


def build(force=False):
    """Compile shader_oracle.c twice (FP32, FP64) into libshader_oracle.so."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    with tempfile.TemporaryDirectory() as d:
        objs = []
        for tag, defs in (("f32", ["-DREAL=float", "-DSUFFIX=_f32"]),
                          ("f64", ["-DREAL=double", "-DSUFFIX=_f64", "-DREAL_IS_DOUBLE"])):
            o = os.path.join(d, f"shader_{tag}.o")
            subprocess.run(["gcc", "-O2", "-fPIC", "-ffp-contract=off", "-std=c99", *defs, "-c", SRC, "-o", o],
                           check=True)
            objs.append(o)
        tmp = LIB + f".tmp{os.getpid()}"
        subprocess.run(["gcc", "-shared", "-o", tmp, *objs, "-lm"], check=True)
        os.replace(tmp, LIB)
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(LIB)
        vp, i64 = C.c_void_p, C.c_int64
        for tag in ("f32", "f64"):
            f = getattr(lib, f"fill_ldm_{tag}")
            f.argtypes = [C.POINTER(Params), i64, vp, vp, vp, vp, vp, vp, vp, vp, vp]
            f.restype = None
            g = getattr(lib, f"apply_lineshapes_{tag}")
            g.argtypes = [C.POINTER(Params), i64, i64, vp, vp]
            g.restype = None
        _lib = lib
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def synthesize(lines, T, p_bar, x, vmin, dv, n_v, axes, n_ft, molar_mass=28.0, Qref_Qgas=1.0, real="f32",
               cpu_conventions=True):
    """Absorption coefficient on v = vmin + k dv, k < n_v, through the restated
    shaders.  ``axes`` = (log_wG_min, dxG, N_G, log_wL_min, dxL, N_L) (FWHM);
    ``molar_mass`` and ``Qref_Qgas`` scalars or per-isotope arrays indexed by
    the ``iso`` column."""
    lib = load()
    dt = np.float32 if real == "f32" else np.float64
    lg0, dxG, NG, ll0, dxL, NL = axes
    v0 = np.ascontiguousarray(lines["v0"], np.float64)
    n = len(v0)
    iso = lines.get("iso")
    iso_u = None if iso is None else np.ascontiguousarray(iso, np.uint32)
    n_iso = 1 if iso is None else int(iso_u.max()) + 1
    M = np.broadcast_to(np.asarray(molar_mass, np.float64), (n_iso,)) if np.ndim(molar_mass) == 0 else \
        np.asarray(molar_mass, np.float64)
    Qr = np.broadcast_to(np.asarray(Qref_Qgas, np.float64), (n_iso,)) if np.ndim(Qref_Qgas) == 0 else \
        np.asarray(Qref_Qgas, np.float64)
    El = np.ascontiguousarray(lines["El"], np.float64)
    S0 = np.asarray(lines["S_ref"], np.float64) * np.exp(O.HC_K * El / O.TREF) / \
        (1.0 - np.exp(-O.HC_K * v0 / O.TREF))
    P = Params()
    P.v_min, P.dv, P.n_v, P.n_row = float(vmin), float(dv), int(n_v), int(n_ft)
    P.dxG, P.dxL, P.log_wG_min, P.log_wL_min = float(dxG), float(dxL), float(lg0), float(ll0)
    P.n_G, P.n_L = int(NG), int(NL)
    p = p_bar / 1.01325 if cpu_conventions else p_bar          # atm (CPU) or bar (GPU)
    kb = O.KB_CGS if cpu_conventions else KB_SCIPY
    P.p, P.log_2p = p, float(np.log(2.0 * p))
    P.hlog_T, P.log_rT, P.c2T = 0.5 * np.log(T), float(np.log(O.TREF / T)), O.HC_K / T
    P.N = (p_bar * 1e5) / (O.KB_SI * T) * 1e-6
    P.x_self, P.x_air = float(x), 1.0 - float(x)
    for i in range(n_iso):
        # log FWHM_G - log v0 - 0.5 log T (radis/gpu/params.py:31-40, radis/lbl/broadening.py:170-172)
        P.log_c2Mm[i] = float(np.log(2.0 / O.C_CGS * np.sqrt(2.0 * O.NA * kb * np.log(2.0) / M[i])))
        P.Q[i] = 1.0 / float(Qr[i])
    da = np.ascontiguousarray(lines.get("delta", np.zeros(n)), np.float64)
    cols = [np.ascontiguousarray(lines[k], np.float64) for k in ("n_air", "g_self", "g_air")]
    ldm = np.zeros((NL, NG, n_ft), dtype=dt)
    getattr(lib, f"fill_ldm_{real}")(C.byref(P), n, _ptr(iso_u), _ptr(v0), _ptr(da), _ptr(S0), _ptr(El),
                                     _ptr(cols[0]), _ptr(cols[1]), _ptr(cols[2]), _ptr(ldm))
    import scipy.fft as sfft
    ft = np.ascontiguousarray(sfft.rfft(ldm, axis=2))          # complex64 for f32, complex128 for f64
    n_bins = ft.shape[2]
    spec = np.zeros(n_bins, dtype=ft.dtype)
    getattr(lib, f"apply_lineshapes_{real}")(C.byref(P), int(n_ft), int(n_bins), _ptr(ft), _ptr(spec))
    return sfft.irfft(spec, n=n_ft)[:n_v].astype(np.float64)
