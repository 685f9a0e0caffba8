"""Wave units, media and quantity units of Spectrum.get (CPU).

* Air wavelengths equal the reference's own vacuum2air / air2vacuum /
  Ciddor index (radis/phys/air.py, run by tests/golden/make_golden_units.py)
  bit for bit.
* Radiance per nm <-> per cm-1 keeps the integral over the band, the check
  the reference documents for convert_rad2cm (radis/phys/units.py); prefix
  changes are exact powers of ten; conversions round-trip.
* Spectrum.get follows the reference's rules (radis/spectrum/spectrum.py:
  1183-1420): 'default' wave unit from the conditions, 'nm' in the
  spectrum's medium, radiance switched to per nm / per cm-1 with the wave
  unit, abscoeff in cm-1 or m-1, dimensionless quantities only '' or '1'.
"""
import os
import warnings

import numpy as np
import pytest

from radis_gb300 import units as U
from radis_gb300.spectrum import Spectrum

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_units.npz"))
_trapezoid = getattr(np, "trapezoid", None) or np.trapz


def test_air_wavelengths_match_reference():
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        assert np.array_equal(U.vacuum2air(G["vac_nm"]), G["air_nm"])
        assert np.array_equal(U.air_index(G["vac_nm"] * 1e-3), G["index"])
        assert np.array_equal(U.air2vacuum(G["vac_nm"]), G["air2vac_nm"])
    with pytest.warns(UserWarning):
        assert U.air_index(np.array([0.25]))[0] == 1.0


def test_radiance_band_integral_is_unit_independent():
    nu = np.linspace(2000.0, 2400.0, 400001)                 # cm-1
    L_nm = np.exp(-((nu - 2200.0) / 30.0) ** 2) + 0.1        # mW/cm2/sr/nm
    L_cm = U.convert_radiance(L_nm, "mW/cm2/sr/nm", "mW/cm2/sr/cm-1", nu)
    lam = 1e7 / nu
    int_nm = -_trapezoid(L_nm, lam)                          # lam decreases with nu
    int_cm = _trapezoid(L_cm, nu)
    assert abs(int_nm / int_cm - 1) < 1e-9
    np.testing.assert_allclose(L_cm, L_nm * 1e7 / nu ** 2, rtol=1e-14)


def test_radiance_prefixes_and_round_trips():
    nu = np.array([500.0, 2000.0, 8000.0])
    I = np.array([1.0, 2.0, 3.0])
    f = lambda a, b: U.convert_radiance(I, a, b, nu)
    np.testing.assert_allclose(f("mW/cm2/sr/nm", "W/cm2/sr/nm"), 1e-3 * I, rtol=1e-15)
    np.testing.assert_allclose(f("mW/cm2/sr/nm", "mW/m2/sr/nm"), 1e4 * I, rtol=1e-15)
    np.testing.assert_allclose(f("mW/cm2/sr/nm", "mW/cm2/sr/µm"), 1e3 * I, rtol=1e-15)
    np.testing.assert_allclose(f("mW/cm2/sr/nm", "mW/sr/cm2/nm"), I, rtol=1e-15)
    np.testing.assert_allclose(f("W/m2/sr/m", "mW/cm2/sr/nm"), 1e3 * 1e-4 * 1e-9 * I, rtol=1e-15)
    for a, b in (("mW/cm2/sr/nm", "W/m2/sr/cm-1"), ("uW/cm2/sr/cm-1", "W/m2/sr/um")):
        back = U.convert_radiance(f(a, b), b, a, nu)
        np.testing.assert_allclose(back, I, rtol=1e-14)
    with pytest.raises(ValueError):
        f("mW/cm2/nm", "W/cm2/sr/nm")
    np.testing.assert_allclose(U.convert_per_length(I, "cm-1", "m-1"), 100 * I, rtol=1e-15)


def _spectrum(**cond):
    w = np.linspace(2000.0, 2010.0, 1001)
    c = dict(path_length=2.0, Tgas=800.0)
    c.update(cond)
    s = Spectrum(dict(wavenumber=w, abscoeff=np.linspace(0.0, 0.5, 1001)), conditions=c)
    return s, w


def test_get_wave_units_and_medium():
    s, w = _spectrum()
    assert np.array_equal(s.get("abscoeff")[0], w)
    assert np.array_equal(s.get("abscoeff", wunit="nm_vac")[0], 1e7 / w)
    np.testing.assert_array_equal(s.get("abscoeff", wunit="nm")[0], U.vacuum2air(1e7 / w))
    np.testing.assert_array_equal(s.get("abscoeff", wunit="nm_air")[0], U.vacuum2air(1e7 / w))
    sv, _ = _spectrum(medium="vacuum", default_output_unit="nm")
    assert np.array_equal(sv.get("abscoeff")[0], 1e7 / w)                # default -> nm -> vacuum
    assert np.array_equal(sv.get("abscoeff", wunit="nm_air")[0], U.vacuum2air(1e7 / w))
    with pytest.raises(ValueError):
        s.get("abscoeff", wunit="GHz")


def test_get_quantity_units():
    s, w = _spectrum()
    k = s.get("abscoeff")[1]
    np.testing.assert_allclose(s.get("abscoeff", Iunit="m-1")[1], 100 * k, rtol=1e-15)
    r_nm = s.get("radiance_noslit", wunit="nm")[1]                       # stored: mW/cm2/sr/nm
    r_cm = s.get("radiance_noslit")[1]                                   # cm-1 axis: per cm-1
    np.testing.assert_allclose(r_cm, r_nm * 1e7 / w ** 2, rtol=1e-14)
    np.testing.assert_array_equal(s.get("radiance_noslit", Iunit="mW/cm2/sr/nm")[1], r_nm)
    np.testing.assert_allclose(s.get("radiance_noslit", wunit="nm", Iunit="W/cm2/sr/nm")[1], 1e-3 * r_nm,
                               rtol=1e-15)
    t = s.get("transmittance_noslit", Iunit="1")[1]
    np.testing.assert_allclose(t, np.exp(-2.0 * k), rtol=1e-12)
    with pytest.raises(ValueError):
        s.get("transmittance_noslit", Iunit="cm-1")


def test_crop_in_wavelength_and_accessors():
    s, w = _spectrum()
    lam_air = U.vacuum2air(1e7 / w)
    np.testing.assert_array_equal(s.get_wavelength(), lam_air)
    np.testing.assert_array_equal(s.get_wavelength("vacuum"), 1e7 / w)
    assert s.get_waveunit() == "cm-1" and np.array_equal(s.get_wavenumber(), w)
    lo, hi = lam_air[600], lam_air[400]                 # wavelength falls as wavenumber rises
    c = s.crop(lo, hi, wunit="nm", inplace=False)
    assert np.array_equal(c.get("abscoeff")[0], w[400:601])
    assert len(s.get("abscoeff")[0]) == 1001            # not in place
    v = s.crop(1e7 / w[700], 1e7 / w[300], wunit="nm_vac")
    assert v is s and np.array_equal(s.get("abscoeff")[0], w[300:701])
