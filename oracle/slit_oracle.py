"""CPU oracle for the instrument slit -- TEST INFRASTRUCTURE ONLY.

Only ``tests/`` and ``bench.py``'s CPU legs may import this module; the GPU
slit (``rg_slit_convolve`` and ``radis_gb300.slit``) never calls it.

FP64 numpy restatement of RADIS 0.17.1's slit generation and convolution
(``radis/tools/slit.py``, paths relative to the radis project root), pinned
against golden vectors produced by running the reference's own functions
(``tests/golden/make_golden_slit.py``).  The convolution is a direct
``np.convolve`` where the reference uses ``scipy.signal.oaconvolve``: the
same sum, different FFT-free rounding (~1e-16 relative).
"""
from __future__ import annotations

import numpy as np


def _normalise(w, I, norm_by):
    """Area / max normalisation (slit.py:1625-1635, 1763-1773, 1879-1889)."""
    if norm_by == "area":
        return I / np.trapezoid(I, x=w)
    if norm_by == "max":
        return I / np.max(I)
    if norm_by is None:
        return I
    raise ValueError(f"Unknown normalization type: `norm_by` = {norm_by}")


def triangular_slit(FWHM, wstep, center=0.0, norm_by="area", scale=1.0, footerspacing=0):
    """slit.py:1607-1637: descending slope of a = int(FWHM / wstep) points
    from 1 with slope 1 / (FWHM - wstep), one extra zero when wstep does not
    divide FWHM (Python float modulo), mirrored about the peak.  The abscissa
    of the half slit is linspace(0, len * wstep, len) (spacing len/(len-1)
    wstep, as in the reference)."""
    slope = 1.0 / (FWHM - wstep)
    n = int(FWHM / wstep)
    half = 1.0 - np.arange(n) * slope * wstep
    pad = int(footerspacing) + (1 if FWHM % wstep else 0)
    half = np.concatenate([half, np.zeros(pad)])
    wh = np.linspace(0.0, len(half) * wstep, len(half))
    I = np.concatenate([half[:0:-1], half])
    w = np.concatenate([-wh[:0:-1], wh]) + center
    return w, _normalise(w, I, norm_by) * scale


def trapezoidal_slit(top, base, wstep, center=0.0, norm_by="area", scale=1.0, footerspacing=0):
    """slit.py:1731-1775: an odd number b of ones on top, slopes of
    a = int(FWHM / wstep) - b steps (FWHM = (top + base) / 2), the last slope
    point clipped at 0 or followed by one extra zero."""
    if top > base:
        top, base = base, top
    FWHM = (base + top) / 2.0
    b = 2 * int(top / wstep // 2) + 1
    slope = 1.0 / (FWHM - b * wstep)
    n = int(FWHM / wstep) - b
    side = 1.0 - np.arange(n + 1) * slope * wstep
    if side.size == 0:
        side = np.ones(1)
    pad = int(footerspacing)
    if side[-1] < 0:
        side[-1] = 0.0
    elif side[-1] > 0:
        pad += 1
    side = np.concatenate([side, np.zeros(pad)])
    I = np.concatenate([side[:0:-1], np.ones(b), side[1:]])
    w = wstep * np.linspace(-len(I) / 2, len(I) / 2, len(I)) + center
    return w, _normalise(w, I, norm_by) * scale


def gaussian_slit(FWHM, wstep, center=0.0, norm_by="area", calc_range=4, scale=1.0, footerspacing=0):
    """slit.py:1862-1891: exp(-w^2 / (2 sigma^2)) on 2a + 1 points,
    a = 2 int(calc_range sigma // wstep / 2), sigma = FWHM / (2 sqrt(2 ln 2)),
    with f zeros on each side."""
    f = int(footerspacing)
    sigma = FWHM / 2.0 / np.sqrt(2.0 * np.log(2.0))
    a = 2 * int(calc_range * sigma // wstep / 2)
    w0 = wstep * np.linspace(-a, a, 2 * a + 1)
    I = np.concatenate([np.zeros(f), np.exp(-(w0 ** 2) / (2.0 * sigma ** 2)), np.zeros(f)])
    w = wstep * np.linspace(-(a + f), a + f, 2 * a + 2 * f + 1) + center
    return w, _normalise(w, I, norm_by) * scale


def slit_on_grid(w_slit, I_slit, wstep, k=1):
    """slit.py:685-711: reverse a descending slit; if its steps are not the
    spectrum's, resample it by an interpolating spline of order k on
    arange(w_slit[0], w_slit[-1] + wstep, wstep)."""
    w_slit = np.asarray(w_slit, dtype=np.float64)
    I_slit = np.asarray(I_slit, dtype=np.float64)
    if w_slit[-1] < w_slit[0]:
        w_slit, I_slit = w_slit[::-1], I_slit[::-1]
    if np.allclose(np.diff(w_slit), wstep):
        return I_slit
    from scipy.interpolate import splev, splrep
    w_new = np.arange(w_slit[0], w_slit[-1] + wstep, wstep)
    return splev(w_new, splrep(w_slit, I_slit, k=k))


def convolve_with_slit(w, I, w_slit, I_slit, mode="valid", k=1):
    """slit.py:666-745 + remove_boundary (slit.py:1063-1072): the spectrum
    step is the smallest |diff(w)|; out = (I conv slit)[same] * wstep; in
    'valid' mode the first int((la-1)/2) and last int(la/2) points become NaN,
    la = min(len(I), len(slit))."""
    w = np.asarray(w, dtype=np.float64)
    I = np.asarray(I, dtype=np.float64)
    wstep = np.abs(np.diff(w)).min()
    s = slit_on_grid(w_slit, I_slit, wstep, k)
    full = np.convolve(I, s)                       # length len(I) + len(s) - 1
    lo = (len(s) - 1) // 2
    out = full[lo:lo + len(I)] * wstep             # 'same': centred part
    if mode == "valid":
        la = min(len(I), len(s))
        a, b = int((la - 1) / 2), int(la / 2)
        out[:a] = np.nan
        out[len(out) - b:] = np.nan
    elif mode != "same":
        raise ValueError(f"Unexpected mode: {mode}")
    return w, out
