"""GPU instrument slit (rg_slit_convolve, radis_gb300.slit, Spectrum.apply_slit)
against the FP64 slit oracle, which is pinned to the reference's own
radis/tools/slit.py (tests/test_oracle_slit.py).

Tolerance: max |I_gpu - I_oracle| <= 1e-5 x max |I_oracle| (FP32 spectrum
and taps, FP32 accumulation over up to a few thousand taps), with NaN at
exactly the oracle's positions in 'valid' mode."""
import os

import numpy as np
import pytest

from oracle import slit_oracle as SO
from radis_gb300 import _lib as L
from radis_gb300 import slit as S

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_slit.npz"))
TOL = 1e-5


def _check(got, want):
    assert np.array_equal(np.isnan(got), np.isnan(want))
    ok = ~np.isnan(want)
    assert np.max(np.abs(got[ok] - want[ok])) <= TOL * np.nanmax(np.abs(want))


@pytest.mark.parametrize("name", ["tri", "trisame", "trap", "gau", "fine1", "fine3"])
def test_golden_cases(native_lib, name):
    w, I = G["spec_w"], G["spec_I"]
    mode, k = G[f"conv_{name}_mode"]
    mode = "same" if mode == 0 else "valid"
    ws, Is = G[f"conv_{name}_slit_w"], G[f"conv_{name}_slit_I"]
    _, got = S.convolve_with_slit(w, I, ws, Is, mode=mode, k=int(k))
    _check(got.astype(np.float64), G[f"conv_{name}_I"])
    _, ref = SO.convolve_with_slit(w, I.astype(np.float32).astype(np.float64), ws, Is, mode=mode, k=int(k))
    _check(got.astype(np.float64), ref)


@pytest.mark.parametrize("shape,fwhm", [("triangular", 1.0), ("gaussian", 0.8), ("trapezoidal", (0.6, 1.4))])
def test_long_slits_multi_pass(native_lib, shape, fwhm):
    # 200 001 points at 0.002 cm-1: slits of 500-2000 taps, several 512-tap passes
    rng = np.random.default_rng(5)
    n, dv = 200001, 0.002
    w = 1900.0 + dv * np.arange(n)
    I = np.exp(-np.convolve(rng.exponential(0.02, n), np.ones(7) / 7, mode="same")).astype(np.float32)
    if shape == "trapezoidal":
        ws, Is = SO.trapezoidal_slit(fwhm[0], fwhm[1], dv)
    elif shape == "gaussian":
        ws, Is = SO.gaussian_slit(fwhm, dv)
    else:
        ws, Is = SO.triangular_slit(fwhm, dv)
    for mode in ("valid", "same"):
        _, got = S.convolve_with_slit(w, I, ws, Is, mode=mode)
        _, ref = SO.convolve_with_slit(w, I.astype(np.float64), ws, Is, mode=mode)
        _check(got.astype(np.float64), ref)


def test_spectrum_apply_slit(native_lib):
    from radis_gb300 import synthetic as Sy
    from radis_gb300.spectrum import Spectrum

    ctx = L.Context(0)
    try:
        ln = L.Lines(ctx, Sy.co_like(), 28.0)
        plan = L.Plan(ln, 1900.0, 0.002, 200001, dxG=Sy.DXG_DEFAULT, dxL=Sy.DXL_DEFAULT)
        a, info = plan.synthesize_host(700.0, 1.01325, 0.1)
        assert info.log_scale == 0.0
        w = 1900.0 + 0.002 * np.arange(200001)
        s = Spectrum({"wavenumber": w, "abscoeff": a.astype(np.float64)},
                     conditions={"path_length": 10.0, "Tgas": 700.0})
        s.apply_slit(0.5, unit="cm-1", shape="triangular")
        # the slit is generated with the spectrum's smallest step, as apply_slit does (spectrum.py:3370)
        ws, Is = SO.triangular_slit(0.5, np.abs(np.diff(w)).min(), center=w[len(w) // 2])
        for q in ("transmittance", "radiance", "emissivity"):
            # in the stored units: get() on the cm-1 axis would give radiance per cm-1
            # (x 1e7 / nu^2), which does not commute with the convolution
            ref_in = s.get(q + "_noslit", Iunit=s.units[q + "_noslit"])[1].astype(np.float32).astype(np.float64)
            _, ref = SO.convolve_with_slit(w, ref_in, ws, Is, mode="valid")
            _check(s.get(q, Iunit=s.units[q])[1].astype(np.float64), ref)
        assert s.conditions["slit_function"] == 0.5
        plan.close()
        ln.close()
    finally:
        ctx.close()


def test_errors(native_lib):
    ctx = L.Context(0)
    try:
        x = torch.ones(1000, device="cuda")
        k = torch.ones(11, device="cuda")
        with pytest.raises(L.RgError):   # out overlaps in
            ctx.slit_convolve(x.data_ptr(), 1000, k.data_ptr(), 11, 0.01, True, x.data_ptr() + 40)
        with pytest.raises(L.RgError):   # empty slit
            ctx.slit_convolve(x.data_ptr(), 1000, k.data_ptr(), 0, 0.01, True, torch.empty_like(x).data_ptr())
        with pytest.raises(ValueError):
            S.convolve_device(x, np.ones(3), 0.01, mode="full")
        # 'same' with a unit slit is the identity times wstep
        y = S.convolve_device(torch.arange(1000, dtype=torch.float32, device="cuda"), np.ones(1), 0.5, mode="same")
        assert torch.equal(y.cpu(), 0.5 * torch.arange(1000, dtype=torch.float32))
    finally:
        ctx.close()
