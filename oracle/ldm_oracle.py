"""CPU oracle for the equilibrium LDM/DIT synthesis -- TEST INFRASTRUCTURE ONLY.

This module checks the product and is never part of it: only ``tests/``, the smoke
check in ``__graft_entry__`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` may import it.  The GPU product path never calls it and
fails loudly when its CUDA library is missing.

It restates, in FP64 numpy, RADIS 0.17.1's CPU ``broadening_method='fft'`` LDM
path (the reference cannot be imported here: pandas/astropy/numba/hapi are
absent).  Every function cites the reference line it follows (paths relative
to the radis project root).  The restatement is pinned against golden vectors
produced by running the reference's own functions (``tests/golden``).

Deliberate, documented generalisations of the reference:

* the FFT length ``n_ft`` is an input (the CPU path uses exactly ``2*N_v``,
  ``radis/lbl/broadening.py:2340-2343``; the GPU path uses a fast even length
  >= 2*N_v, ``radis/gpu/gpu.py:22-29,136``).  With ``n_ft = 2*N_v`` the
  oracle reproduces the CPU path.
* the LDM node axes are inputs ``(log_w_min, dx, N)`` for wG and wL (FWHM)
  so that the oracle runs on exactly the grid the GPU plan chose.
* out-of-window lines are dropped as the GPU shader does
  (``radis/gpu/vulkan/shaders/cmdFillLDM.comp:102``: k0 < 0 or k1 >= N_v).
"""
from __future__ import annotations

import numpy as np

# --- constants (radis/phys/constants.py:22,33,38,60,69) ---------------------
H_SI = 6.62607015e-34
C_SI = 2.99792458e8
KB_SI = 1.3806490e-23
NA = 6.02214076e23
HC_K = H_SI * C_SI / KB_SI * 100.0          # c2 = hc/k in cm.K (constants.py:69)
C_CGS = 2.99792458e10                        # constants.py:78
KB_CGS = 1.380648813e-16                     # erg/K, as the CPU path uses (constants.py:75)
TREF = 296.0                                 # radis/lbl/factory.py:424


# --- per-line physics --------------------------------------------------------
def line_strength_eq(S_ref, El, v0, T, Tref=TREF, Qref_Qgas=1.0):
    """S(T) from S(Tref): radis/lbl/base.py:2664-2677 (HITRAN A.11)."""
    return (S_ref * Qref_Qgas * np.exp(-HC_K * El * (1.0 / T - 1.0 / Tref))
            * (1.0 - np.exp(-HC_K * v0 / T)) / (1.0 - np.exp(-HC_K * v0 / Tref)))


def doppler_hwhm(v0, molar_mass, T):
    """Gaussian HWHM: radis/lbl/broadening.py:170-172 (df.wav, not shiftwav:
    broadening.py:1449)."""
    return (v0 / C_CGS) * np.sqrt((2.0 * NA * KB_CGS * T * np.log(2.0)) / molar_mass)


def lorentz_hwhm(g_air, g_self, n_air, p_atm, x, T, Tref=TREF):
    """Collisional HWHM, self + air only, Tdpsel absent -> n_air for both:
    radis/lbl/broadening.py:368-381 (p in atm, broadening.py:1063)."""
    t = (Tref / T) ** n_air
    return t * g_air * p_atm * (1.0 - x) + t * g_self * p_atm * x


def shifted_position(v0, delta, p_atm):
    """Pressure-shifted line centre: radis/lbl/base.py:2358-2360."""
    return v0 + delta * p_atm


def number_density(p_bar, T, x):
    """Molecule number density (cm-3): radis/lbl/factory.py:908-912."""
    return x * ((p_bar * 1e5) / (KB_SI * T)) * 1e-6


# --- lineshapes in Fourier space ---------------------------------------------
def gaussian_ft(f, hwhm):
    """radis/lbl/broadening.py:229-253."""
    return np.exp(-((2.0 * np.pi * f * hwhm) ** 2) / (4.0 * np.log(2.0)))


def lorentzian_ft(f, hwhm):
    """radis/lbl/broadening.py:584-608."""
    return np.exp(-2.0 * np.pi * f * hwhm)


def voigt_ft(f, hwhm_g, hwhm_l):
    """radis/lbl/broadening.py:828-852."""
    return gaussian_ft(f, hwhm_g) * lorentzian_ft(f, hwhm_l)


def lineshape_ft(n_ft, dv, wG, wL, folding_thresh=1e-6):
    """Normalised, folded Voigt FT on the rfft bins of length ``n_ft``:
    radis/lbl/broadening.py:1896-1926 (w = rfftfreq(2N, wstep) generalised to
    rfftfreq(n_ft, dv); folding while voigt_FT(n/(2 dv)) >= folding_thresh;
    normalised to bin 0).  wG, wL are FWHM."""
    f = np.fft.rfftfreq(n_ft, dv)
    w_fold = (f, f[::-1])
    prof = voigt_ft(f, wG / 2.0, wL / 2.0)
    n = 1
    while voigt_ft(n / (2.0 * dv), wG / 2.0, wL / 2.0) >= folding_thresh:
        prof = prof + voigt_ft(n / (2.0 * dv) + w_fold[n & 1], wG / 2.0, wL / 2.0)
        n += 1
    return prof / prof[0]


def fold_count(dv, wG, wL, folding_thresh=1e-6):
    """Number of folding terms the loop of ``lineshape_ft`` adds."""
    n = 1
    while voigt_ft(n / (2.0 * dv), wG / 2.0, wL / 2.0) >= folding_thresh:
        n += 1
    return n - 1


# --- LDM axes -----------------------------------------------------------------
def cpu_w_axis(w_dat, log_p):
    """CPU node axis from data: radis/lbl/broadening.py:1823-1836 (FWHM)."""
    w_min = w_dat.min()
    if w_min < 0:
        w_min = w_dat[w_dat > 0].min()
    w_max = w_dat.max() + 1e-4
    N = np.ceil((np.log(w_max) - np.log(w_min)) / log_p) + 1
    return w_min * np.exp(log_p * np.arange(N))


def axis_values(log_min, dx, n):
    """Node FWHMs of a log-uniform axis (the GPU's wG_l = exp(log_wG_min + l dxG),
    radis/gpu/vulkan/shaders/cmdApplyLineshapes.comp:76-80)."""
    return np.exp(log_min + dx * np.arange(n))


# --- scatter + convolution ------------------------------------------------------
def ldm_scatter(kpos, log_wG, log_wL, I, n_v, axes, n_rows=None, out=None):
    """Distribute line intensities on the (k, l, m) grid with 2x2x2 linear
    weights: indices radis/lbl/broadening.py:2151-2154,2253-2263; simple
    weights :2305-2318; 8x add.at :2478-2485 (misc/arrays.py:472-502).

    ``kpos`` is the fractional spectral index (v - vmin)/dv.  ``axes`` =
    (log_wG_min, dxG, N_G, log_wL_min, dxL, N_L).  Returns LDM[n_rows, N_G, N_L]
    (n_rows defaults to n_v) in FP64; with ``out`` (an LDM of that shape) the
    lines are added to it instead."""
    lg0, dxG, NG, ll0, dxL, NL = axes
    n_rows = n_v if n_rows is None else n_rows
    k0 = np.floor(kpos).astype(np.int64)
    keep = (k0 >= 0) & (k0 + 1 < n_v)
    k0 = k0[keep]
    tv = kpos[keep] - k0
    pl = (log_wG[keep] - lg0) / dxG
    pm = (log_wL[keep] - ll0) / dxL
    if pl.size and (pl.min() < -1e-3 or pl.max() > NG - 1 + 1e-3 or pm.min() < -1e-3
                    or pm.max() > NL - 1 + 1e-3):
        raise ValueError("line widths fall outside the LDM node axes")
    # a line sitting exactly on the first/last node stays in the edge cell
    # (rounding can put it a hair outside); np.interp in the reference clamps
    # the same way (broadening.py:2151-2154)
    l0 = np.clip(np.floor(pl).astype(np.int64), 0, NG - 2)
    m0 = np.clip(np.floor(pm).astype(np.int64), 0, NL - 2)
    tG = pl - l0
    tL = pm - m0
    Ik = I[keep]
    LDM = np.zeros((n_rows, NG, NL)) if out is None else out
    Iv0 = Ik * (1 - tv)
    Iv1 = Ik * tv
    w00 = (1 - tG) * (1 - tL)
    w01 = (1 - tG) * tL
    w10 = tG * (1 - tL)
    w11 = tG * tL
    for kk, Iv in ((k0, Iv0), (k0 + 1, Iv1)):
        np.add.at(LDM, (kk, l0, m0), Iv * w00)
        np.add.at(LDM, (kk, l0, m0 + 1), Iv * w01)
        np.add.at(LDM, (kk, l0 + 1, m0), Iv * w10)
        np.add.at(LDM, (kk, l0 + 1, m0 + 1), Iv * w11)
    return LDM


def ldm_convolve(LDM, n_v, dv, axes, n_ft, folding_thresh=1e-6, fft_workers=1):
    """Sum over nodes of rfft(LDM row) x folded Voigt FT, one irfft, /dv:
    radis/lbl/broadening.py:2521-2530.  Returns the first n_v samples."""
    import scipy.fft as sfft
    lg0, dxG, NG, ll0, dxL, NL = axes
    wG = axis_values(lg0, dxG, NG)
    wL = axis_values(ll0, dxL, NL)
    acc = np.zeros(n_ft // 2 + 1, dtype=np.complex128)
    for l in range(NG):
        rows = np.zeros((NL, n_ft))
        rows[:, :LDM.shape[0]] = LDM[:, l, :].T
        spec = sfft.rfft(rows, axis=1, workers=fft_workers)
        for m in range(NL):
            acc += spec[m] * lineshape_ft(n_ft, dv, wG[l], wL[m], folding_thresh)
    out = sfft.irfft(acc, n=n_ft, workers=fft_workers)[:n_v]
    return out / dv


def line_quantities(lines, T, p_bar, x, vmin, dv, Tref=TREF, Qref_Qgas=1.0,
                    molar_mass=None):
    """Per-line (kpos, log wG, log wL, S) for conditions (T, p_bar, x).

    ``lines``: dict with v0, S_ref, El, g_air, g_self, n_air, delta and
    optionally iso (int); ``molar_mass`` scalar or per-iso array;
    ``Qref_Qgas`` scalar or per-iso array indexed by iso."""
    p_atm = p_bar / 1.01325                              # broadening.py:1063
    v0 = np.asarray(lines["v0"], dtype=np.float64)
    iso = lines.get("iso")
    M = np.asarray(molar_mass, dtype=np.float64)
    Mi = M if M.ndim == 0 else M[iso]
    Q = np.asarray(Qref_Qgas, dtype=np.float64)
    Qi = Q if Q.ndim == 0 else Q[iso]
    S = line_strength_eq(np.asarray(lines["S_ref"], np.float64),
                         np.asarray(lines["El"], np.float64), v0, T, Tref, Qi)
    wG = 2.0 * doppler_hwhm(v0, Mi, T)
    wL = 2.0 * lorentz_hwhm(np.asarray(lines["g_air"], np.float64),
                            np.asarray(lines["g_self"], np.float64),
                            np.asarray(lines["n_air"], np.float64), p_atm, x, T, Tref)
    vs = shifted_position(v0, np.asarray(lines.get("delta", np.zeros_like(v0)), np.float64), p_atm)
    kpos = (vs - vmin) / dv
    return kpos, np.log(wG), np.log(wL), S


def synthesize(lines, T, p_bar, x, vmin, dv, n_v, axes, n_ft, Tref=TREF,
               Qref_Qgas=1.0, molar_mass=28.0, folding_thresh=1e-6, fft_workers=1,
               return_ldm=False, line_chunk=None):
    """Absorption coefficient (cm-1) on v = vmin + k dv, k < n_v, in FP64.

    Follows radis/lbl/factory.py:859-912 (linestrength -> HWHM -> lineshift ->
    LDM broadening -> x density).  ``line_chunk``: scale and scatter the lines
    in blocks of that many (bounds the host memory of very long lists; the
    LDM is the same sum)."""
    n = len(lines["v0"])
    step = n if not line_chunk else int(line_chunk)
    LDM = None
    for a in range(0, max(n, 1), max(step, 1)):
        part = lines if step >= n else {k: (v[a:a + step] if np.ndim(v) == 1 and len(v) == n else v)
                                        for k, v in lines.items()}
        kpos, lgG, lgL, S = line_quantities(part, T, p_bar, x, vmin, dv, Tref,
                                            Qref_Qgas, molar_mass)
        LDM = ldm_scatter(kpos, lgG, lgL, S, n_v, axes, out=LDM)
    spec = ldm_convolve(LDM, n_v, dv, axes, n_ft, folding_thresh, fft_workers)
    out = spec * number_density(p_bar, T, x)
    if return_ldm:
        return out, LDM * number_density(p_bar, T, x)
    return out


def planck_nm(lambda_nm, T):
    """Blackbody radiance in mW/cm2/sr/nm at wavelength ``lambda_nm`` (nm):
    radis/phys/blackbody.py:35-74 (SI h, c, k; x 1e-10 from W/sr/m3)."""
    lbd = np.asarray(lambda_nm, np.float64) * 1e-9
    return (2 * H_SI * C_SI ** 2 / lbd ** 5) / np.expm1(H_SI * C_SI / (lbd * KB_SI * T)) * 1e-10


def quantities(abscoeff, vmin, dv, T, path_length):
    """The spectral quantities of eq_spectrum_gpu from the absorption
    coefficient (cm-1) on v = vmin + k dv: absorbance = abscoeff L;
    emissivity = -expm1(-absorbance); transmittance = 1 - emissivity;
    radiance = emissivity x Planck(1e7 / v nm, T) in mW/cm2/sr/nm
    (radis/lbl/factory.py:1284-1297, radis/spectrum/equations.py:21-44)."""
    a = np.asarray(abscoeff, np.float64)
    v = vmin + dv * np.arange(a.size)
    absorbance = a * path_length
    emissivity = -np.expm1(-absorbance)
    return {"abscoeff": a, "absorbance": absorbance, "emissivity_noslit": emissivity,
            "transmittance_noslit": 1.0 - emissivity,
            "radiance_noslit": emissivity * planck_nm(1e7 / v, T)}


def envelope_axes(lines, T, p_bar, x, dxG=None, dxL=None, NG=None, NL=None,
                  molar_mass=28.0, Tref=TREF, eps=1e-4):
    """Brute-force restatement of the GPU node-axis rule (radis/gpu/params.py:
    8-117) used to cross-check the library's hull code: log_wL bounds are the
    envelopes of log(min|max(g_self, g_air)) + n_air log(Tref/T) + log(2 p);
    log_wG bounds the min/max of log v0 + log_c2Mm + 0.5 log T; the top is
    raised by eps in log space; N = ceil(span/dx)+1, or dx = span/(N-1) when
    the node count is fixed.  Pressure enters in atm, as in the CPU path's
    widths (radis/lbl/broadening.py:1063); the Vulkan path uses bar there
    (radis/gpu/params.py:144)."""
    p_atm = p_bar / 1.01325
    v0 = np.asarray(lines["v0"], np.float64)
    iso = lines.get("iso")
    M = np.asarray(molar_mass, np.float64)
    Mi = M if M.ndim == 0 else M[iso]
    log_c2Mm = np.log(2.0 * doppler_hwhm(1.0, Mi, 1.0))
    lg = np.log(v0) + log_c2Mm + 0.5 * np.log(T)
    ga = np.asarray(lines["g_air"], np.float64)
    gs = np.asarray(lines["g_self"], np.float64)
    na = np.asarray(lines["n_air"], np.float64)
    t = np.log(Tref / T)
    ll_lo = np.min(np.log(np.minimum(ga, gs)) + na * t) + np.log(2 * p_atm)
    ll_hi = np.max(np.log(np.maximum(ga, gs)) + na * t) + np.log(2 * p_atm)
    out = []
    for lo, hi, dx, n in ((lg.min(), lg.max(), dxG, NG), (ll_lo, ll_hi, dxL, NL)):
        hi = hi + eps
        if n is None:
            n = int(np.ceil((hi - lo) / dx) + 1)
        else:
            dx = (hi - lo) / (n - 1)
        out += [lo, dx, n]
    return tuple(out)
