"""Instrument slit with the convolution on the GPU.

The reference applies the slit on the CPU after its GPU path: ``gpuApp.iterate``
accepts ``slit_FWHM`` and leaves it unused (radis/gpu/gpu.py:308-310,
params.py:152), and ``Spectrum.apply_slit`` (radis/spectrum/spectrum.py:
3127-3579) calls ``radis/tools/slit.py:convolve_with_slit``.  Here the slit
function is generated on the host exactly as the reference generates it (a
few thousand points at most), and the convolution over the spectrum -- the
n_v x n_slit part -- runs on the device through ``rg_slit_convolve``.

Paths below are relative to the radis project root.
"""
from __future__ import annotations

import numpy as np

from . import _lib as L

SLIT_SHAPES = ["triangular", "trapezoidal", "gaussian"]   # slit.py:59


def _normalise(w, I, norm_by):
    # slit.py:1625-1635 (area by the trapezoidal rule, or peak to 1)
    if norm_by == "area":
        return I / np.trapezoid(I, x=w)
    if norm_by == "max":
        return I / np.max(I)
    if norm_by is None:
        return I
    raise ValueError(f"Unknown normalization type: `norm_by` = {norm_by}")


def triangular_slit(FWHM, wstep, center=0.0, norm_by="area", scale=1.0, footerspacing=0):
    """Triangle of FWHM (slit.py:1522-1650): a = int(FWHM / wstep) points on
    each slope, one more zero when wstep does not divide FWHM, abscissa of the
    half slit linspace(0, len * wstep, len) as in the reference."""
    slope = 1.0 / (FWHM - wstep)
    I = 1.0 - np.arange(int(FWHM / wstep)) * slope * wstep
    I = np.hstack((I, np.zeros(int(footerspacing) + (1 if FWHM % wstep else 0))))
    w = np.linspace(0.0, len(I) * wstep, len(I))
    I = np.hstack((I[1:][::-1], I))
    w = np.hstack((-w[1:][::-1], w)) + center
    return w, _normalise(w, I, norm_by) * scale


def trapezoidal_slit(top, base, wstep, center=0.0, norm_by="area", scale=1.0, footerspacing=0):
    """Trapezoid of given top and base widths (slit.py:1651-1785)."""
    if top > base:
        top, base = base, top
    FWHM = (base + top) / 2.0
    b = 2 * int(top / wstep // 2) + 1
    slope = 1.0 / (FWHM - b * wstep)
    I = 1.0 - np.arange(int(FWHM / wstep) - b + 1) * slope * wstep
    if len(I) == 0:
        I = np.ones(1)
    f = int(footerspacing)
    if I[-1] < 0:
        I[-1] = 0.0
    elif I[-1] > 0:
        f += 1
    I = np.hstack((I, np.zeros(f)))
    I = np.hstack((I[1:][::-1], np.ones(b), I[1:]))
    w = wstep * np.linspace(-len(I) / 2, len(I) / 2, len(I)) + center
    return w, _normalise(w, I, norm_by) * scale


def gaussian_slit(FWHM, wstep, center=0.0, norm_by="area", calc_range=4, scale=1.0, footerspacing=0):
    """Gaussian of FWHM sampled over +-calc_range sigma (slit.py:1786-1891)."""
    f = int(footerspacing)
    sigma = FWHM / 2.0 / np.sqrt(2.0 * np.log(2.0))
    a = 2 * int(calc_range * sigma // wstep / 2)
    w0 = wstep * np.linspace(-a, a, 2 * a + 1)
    I = np.hstack((np.zeros(f), np.exp(-(w0 ** 2) / (2.0 * sigma ** 2)), np.zeros(f)))
    w = wstep * np.linspace(-(a + f), a + f, 2 * a + 2 * f + 1) + center
    return w, _normalise(w, I, norm_by) * scale


def get_slit_function(slit_function, unit="cm-1", norm_by="area", shape="triangular", center_wavespace=0.0,
                      return_unit="cm-1", wstep=None, calc_range=4):
    """Slit (w, I) from a FWHM (triangular / gaussian), a (top, base) pair
    (trapezoidal) or sampled arrays (w, I) renormalised by ``norm_by``
    (slit.py:65-475 for a slit given in the spectrum's own wavespace; the
    nm <-> cm-1 conversion of the reference is not provided)."""
    if unit != return_unit:
        raise NotImplementedError(f"slit in {unit} for a spectrum in {return_unit}: only the spectrum's own "
                                  "wavespace is supported")
    if wstep is None or not wstep > 0:
        raise ValueError("wstep (the spectrum step) is required")
    if isinstance(slit_function, (tuple, list)) and len(slit_function) == 2 \
            and np.ndim(slit_function[0]) == 1 and np.size(slit_function[0]) > 2:
        w, I = (np.asarray(x, dtype=np.float64) for x in slit_function)
        return w, _normalise(w, I, norm_by)
    if isinstance(slit_function, (tuple, list)):
        if shape != "trapezoidal":
            raise ValueError("a (top, base) slit needs shape='trapezoidal'")
        top, base = slit_function
        return trapezoidal_slit(top, base, wstep, center=center_wavespace, norm_by=norm_by)
    if shape == "triangular":
        return triangular_slit(float(slit_function), wstep, center=center_wavespace, norm_by=norm_by)
    if shape == "gaussian":
        return gaussian_slit(float(slit_function), wstep, center=center_wavespace, norm_by=norm_by,
                             calc_range=calc_range)
    raise ValueError(f"slit shape {shape!r}: one of {SLIT_SHAPES} (trapezoidal takes (top, base))")


def slit_on_grid(w_slit, I_slit, wstep, k=1):
    """The slit sampled on the spectrum step (slit.py:685-711): reversed if
    descending, resampled by an interpolating spline of order k on
    arange(w_slit[0], w_slit[-1] + wstep, wstep) unless its steps already
    equal wstep (np.allclose, as the reference decides)."""
    w_slit = np.asarray(w_slit, dtype=np.float64)
    I_slit = np.asarray(I_slit, dtype=np.float64)
    if w_slit[-1] < w_slit[0]:
        w_slit, I_slit = w_slit[::-1], I_slit[::-1]
    if np.any(np.isnan(I_slit)):
        raise ValueError("Slit has nan value")
    if not (I_slit >= 0).all():
        raise ValueError("Slit is partially negative")
    if np.allclose(np.diff(w_slit), wstep):
        return I_slit
    from scipy.interpolate import splev, splrep
    w_new = np.arange(w_slit[0], w_slit[-1] + wstep, wstep)
    return splev(w_new, splrep(w_slit, I_slit, k=k))


_CTX = {}


def _context(device):
    c = _CTX.get(device)
    if c is None:
        c = _CTX[device] = L.Context(device)
    return c


def convolve_device(I_dev, slit, wstep, mode="valid", out=None, ctx=None, stream=None):
    """Slit convolution of a float32 CUDA tensor ``I_dev`` (the spectrum on a
    grid of step ``wstep``) with ``slit`` (already on that step; numpy array
    or tensor): returns a new float32 tensor, ``wstep * (I conv slit)``
    ['same'], NaN on the boundary points in 'valid' mode."""
    import torch

    if mode not in ("valid", "same"):
        raise ValueError(f"Unexpected mode: {mode}")
    if not (I_dev.is_cuda and I_dev.dtype == torch.float32 and I_dev.dim() == 1):
        raise ValueError("I_dev must be a 1-D float32 CUDA tensor")
    dev = I_dev.device
    I_dev = I_dev.contiguous()
    s = torch.as_tensor(np.asarray(slit, dtype=np.float32) if not torch.is_tensor(slit) else slit,
                        dtype=torch.float32, device=dev).contiguous()
    if out is None:
        out = torch.empty_like(I_dev)
    ctx = ctx or _context(dev.index or 0)
    st = stream if stream is not None else (torch.cuda.current_stream(dev).cuda_stream or 1)
    ctx.slit_convolve(I_dev.data_ptr(), I_dev.numel(), s.data_ptr(), s.numel(), float(wstep), mode == "valid",
                      out.data_ptr(), st)
    return out


def convolve_with_slit(w, I, w_slit, I_slit, mode="valid", k=1, device=0, assert_evenly_spaced=True):
    """Drop-in for radis/tools/slit.py:convolve_with_slit on an evenly spaced
    spectrum: returns (w, I_conv) as numpy arrays (float64 axis, float32
    values) with the convolution computed on the GPU."""
    import torch

    w = np.asarray(w, dtype=np.float64)
    if len(w) < 2:
        raise ValueError("spectrum needs at least two points")
    wstep = np.abs(np.diff(w)).min()                                # slit.py:670-676
    if assert_evenly_spaced and not np.allclose(np.diff(w), np.diff(w).mean(), atol=wstep * 1e-3):
        raise ValueError("Spectrum is not evenly spaced. Cannot apply slit function.")
    s = slit_on_grid(w_slit, I_slit, wstep, k)
    dev = torch.device("cuda", device)
    I_dev = torch.as_tensor(np.asarray(I, dtype=np.float32), device=dev)
    out = convolve_device(I_dev, s, wstep, mode=mode)
    return w, out.cpu().numpy()
