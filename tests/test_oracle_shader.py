"""The second oracle: the reference's GPU (Vulkan) path restated in C
(oracle/shader_oracle.c: the arithmetic of cmdFillLDM.comp and
cmdApplyLineshapes.comp, FP32 as the shaders run and FP64), CPU only.

* With the CPU path's conventions (pressure in atm in the shift and widths,
  the CPU Doppler constant) the FP64 restatement equals the FP64 CPU oracle
  to rounding: the shader method and the CPU FFT-LDM method are the same
  algorithm on the same node axes when no node folds.
* In FP32 the same restatement is ~2.6e-3 of the peak away on the 10k-line
  CO-like case (200 001 points at 0.002 cm-1): the reference GPU design does
  not meet 1e-4 there.  The error shrinks as the lines move to lower
  wavenumbers (FP32 v0 rounding) down to a floor set by the FP32 grid index
  (ulp 1/64 of a step at index 2e5); this library's scatter computes both
  in double-float.
"""
import numpy as np
import pytest

from oracle import ldm_oracle as O
from oracle import shader_oracle as SO
from radis_gb300 import synthetic as S

T, P, X, DV, N_V, N_FT = 700.0, 1.01325, 0.1, 0.002, 200001, 409600


def _case(shift=0.0):
    lines = S.co_like(10000)
    lines["El"] = np.minimum(lines["El"], 3000.0)   # keeps the FP32 S0 of the shader form in range
    lines["v0"] = lines["v0"] + shift
    axes = O.envelope_axes(lines, T, P, X, dxG=0.14, dxL=0.2, molar_mass=28.0)
    assert O.fold_count(DV, np.exp(axes[0]), np.exp(axes[3])) == 0   # the shader path has no folding
    ref = O.synthesize(lines, T, P, X, 1900.0 + shift, DV, N_V, axes, N_FT, molar_mass=28.0, fft_workers=4)
    return lines, axes, ref


def _err(a, ref):
    return float(np.max(np.abs(a - ref)) / np.max(np.abs(ref)))


@pytest.fixture(scope="module")
def case():
    return _case()


def test_fp64_restatement_equals_cpu_oracle(case):
    lines, axes, ref = case
    a = SO.synthesize(lines, T, P, X, 1900.0, DV, N_V, axes, N_FT, molar_mass=28.0, real="f64")
    assert _err(a, ref) < 1e-12


def test_fp32_error_of_the_reference_gpu_design(case):
    lines, axes, ref = case
    e0 = _err(SO.synthesize(lines, T, P, X, 1900.0, DV, N_V, axes, N_FT, molar_mass=28.0, real="f32"), ref)
    assert 1e-3 < e0 < 1e-2
    lo, axes_lo, ref_lo = _case(shift=-1500.0)   # lines at 400-800 cm-1: 4x finer FP32 v0
    e1 = _err(SO.synthesize(lo, T, P, X, 400.0, DV, N_V, axes_lo, N_FT, molar_mass=28.0, real="f32"), ref_lo)
    assert 1e-4 < e1 < e0 / 2
