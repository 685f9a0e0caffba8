"""Slit oracle pinned to the reference: the restated slit generators and
convolution against golden vectors produced by running RADIS 0.17.1's own
``radis/tools/slit.py`` functions (``tests/golden/make_golden_slit.py``).

Tolerances: slit shapes 1e-12 relative to their peak (same arithmetic);
convolution 1e-12 of the spectrum's peak (np.convolve against the reference's
oaconvolve) with NaN at exactly the same positions."""
import os

import numpy as np
import pytest

from oracle import slit_oracle as SO

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_slit.npz"))


def _close(got, want, rel=1e-12):
    assert got.shape == want.shape
    assert np.max(np.abs(got - want)) <= rel * np.max(np.abs(want))


@pytest.mark.parametrize("i", range(5))
def test_triangular(i):
    fwhm, ws, c, sc, area = G[f"tri{i}_args"]
    w, I = SO.triangular_slit(fwhm, ws, center=c, norm_by="area" if area else "max", scale=sc)
    _close(w - c, G[f"tri{i}_w"] - c)
    _close(I, G[f"tri{i}_I"])


@pytest.mark.parametrize("i", range(4))
def test_trapezoidal(i):
    top, base, ws, area = G[f"trap{i}_args"]
    w, I = SO.trapezoidal_slit(top, base, ws, norm_by="area" if area else "max")
    _close(w, G[f"trap{i}_w"])
    _close(I, G[f"trap{i}_I"])


@pytest.mark.parametrize("i", range(4))
def test_gaussian(i):
    fwhm, ws, cr = G[f"gau{i}_args"]
    w, I = SO.gaussian_slit(fwhm, ws, calc_range=cr)
    _close(w, G[f"gau{i}_w"])
    _close(I, G[f"gau{i}_I"])


@pytest.mark.parametrize("name", ["tri", "trisame", "trap", "gau", "fine1", "fine3"])
def test_convolve_with_slit(name):
    w, I = G["spec_w"], G["spec_I"]
    mode, k = G[f"conv_{name}_mode"]
    _, got = SO.convolve_with_slit(w, I, G[f"conv_{name}_slit_w"], G[f"conv_{name}_slit_I"],
                                   mode="same" if mode == 0 else "valid", k=int(k))
    want = G[f"conv_{name}_I"]
    assert np.array_equal(np.isnan(got), np.isnan(want))
    ok = ~np.isnan(want)
    assert np.max(np.abs(got[ok] - want[ok])) <= 1e-12 * np.nanmax(np.abs(want))
