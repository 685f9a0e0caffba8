"""CPU checks of the drop-in front end: HITRAN-160 I/O, the factory grid and
the host-side derived quantities (no GPU)."""
import os

import numpy as np
import pytest

from radis_gb300 import SpectrumFactory, hitran
from radis_gb300 import synthetic as S
from radis_gb300.spectrum import Spectrum, derived_quantities, planck_nm

# The reference's own HITRAN fixture, read where the reference tree is available:
# RADIS_REFERENCE_ROOT names the radis project root (the test is skipped without it).
_REF_ROOT = os.environ.get("RADIS_REFERENCE_ROOT", "")
REF_FIXTURE = os.path.join(_REF_ROOT, "radis", "test", "files", "hitran_co_3iso_2000_2300cm.par") if _REF_ROOT else ""


def test_hitran_roundtrip_idempotent(tmp_path):
    lines = S.co_like(500)
    lines["delta"] = np.random.default_rng(3).uniform(-0.005, 0, 500)
    p1, p2 = tmp_path / "a.par", tmp_path / "b.par"
    hitran.write_hitran160(p1, lines)
    r1 = hitran.read_hitran160(p1)
    hitran.write_hitran160(p2, r1)
    assert open(p1).read() == open(p2).read()
    assert all(len(x.rstrip("\n")) == 160 for x in open(p1))
    np.testing.assert_allclose(r1["v0"], lines["v0"], atol=1e-6)
    np.testing.assert_allclose(r1["S_ref"], lines["S_ref"], rtol=6e-4)
    np.testing.assert_allclose(r1["n_air"], lines["n_air"], atol=5e-3)


@pytest.mark.skipif(not REF_FIXTURE or not os.path.exists(REF_FIXTURE),
                    reason="RADIS_REFERENCE_ROOT unset or the reference tree is absent")
def test_hitran_reads_reference_fixture():
    d = hitran.read_hitran160(REF_FIXTURE)
    assert len(d["v0"]) == 573
    assert set(np.unique(d["iso"])) == {1, 2, 3}
    assert np.all(d["id"] == 5)
    assert d["v0"].min() >= 2000 and d["v0"].max() <= 2300


def test_factory_grid_and_margins():
    sf = SpectrumFactory(2000.0, 2010.0, wstep=0.01, molecule="CO", neighbour_lines=1.0)
    assert len(sf.wavenumber) == 1001
    assert sf.woutrange == (100, 1101)
    np.testing.assert_allclose(sf.wavenumber_calc[sf.woutrange[0]], 2000.0)
    np.testing.assert_allclose(sf.wavenumber[-1], 2010.0)
    with pytest.raises(ValueError):
        sf.eq_spectrum_gpu(300.0)            # no database loaded
    # the GPU path always runs the LDM with the FFT; the factory's method is only recorded
    assert SpectrumFactory(2000, 2010, broadening_method="voigt").params.broadening_method == "voigt"


def test_factory_ranges_and_output_unit():
    """wmin/wmax + wunit, wavenum_*, wavelength_* in air or vacuum
    (radis/lbl/base.py get_wavenumber_range); the input range sets the
    spectra's default output unit."""
    from radis_gb300 import units as U
    sf = SpectrumFactory(wavelength_min=4500.0, wavelength_max=4600.0, wstep=0.01, molecule="CO")
    assert sf.input_wunit == "nm"
    assert sf.input.wavenum_min == pytest.approx(float(U.nm_air2cm(4600.0)), rel=1e-15)
    assert sf.input.wavenum_max == pytest.approx(float(U.nm_air2cm(4500.0)), rel=1e-15)
    assert sf.input.wavenum_min > 1e7 / 4600.0 * (1 - 3e-4)          # air -> vacuum shifts by ~2.7e-4
    sv = SpectrumFactory(wavelength_min=4500.0, wavelength_max=4600.0, medium="vacuum", molecule="CO")
    assert sv.input_wunit == "nm_vac" and sv.input.wavenum_min == pytest.approx(1e7 / 4600.0, rel=1e-15)
    assert SpectrumFactory(4.5, 4.6, wunit="um", molecule="CO").input.wavenum_max == pytest.approx(
        float(U.nm_air2cm(4500.0)), rel=1e-15)
    assert SpectrumFactory(4500, 4600, wunit="nm_vac").input_wunit == "nm_vac"
    assert SpectrumFactory(200000, 201000, wunit="m-1").input.wavenum_min == pytest.approx(2000.0)
    assert SpectrumFactory(wavenum_min=2000, wavenum_max=2010).input_wunit == "cm-1"
    with pytest.raises(ValueError):
        SpectrumFactory(2000, 2010, wavenum_min=2000, wavenum_max=2010)
    with pytest.raises(ValueError):
        SpectrumFactory(2010, 2000)
    with pytest.raises(ValueError):
        SpectrumFactory(wavenum_min=2000, wavenum_max=2010, wunit="cm-1")
    with pytest.raises(NotImplementedError):
        SpectrumFactory(2000, 2010, medium="water")
    with pytest.raises(ValueError):
        SpectrumFactory(2000, 2010, species="CO", molecule="CO2")


def test_derived_quantities():
    w = np.linspace(2000, 2100, 11)
    k = np.linspace(0, 2, 11)
    a, e, t, r = derived_quantities(w, k, 3.0, 1000.0)
    np.testing.assert_allclose(a, 3 * k)
    np.testing.assert_allclose(t, np.exp(-3 * k), rtol=1e-12)
    np.testing.assert_allclose(e, 1 - np.exp(-3 * k), rtol=1e-12, atol=1e-15)
    # Planck in mW/cm2/sr/nm: 2hc^2/l^5/(exp(hc/lkT)-1) * 1e-10 (blackbody.py:64-69)
    lam = 1e7 / w * 1e-9
    h, c, kb = 6.62607015e-34, 2.99792458e8, 1.380649e-23
    ref = 2 * h * c ** 2 / lam ** 5 / (np.exp(h * c / (lam * kb * 1000.0)) - 1) * 1e-10
    np.testing.assert_allclose(planck_nm(1e7 / w, 1000.0), ref, rtol=1e-12)
    np.testing.assert_allclose(r, e * ref, rtol=1e-12)


def test_spectrum_get_and_crop():
    w = np.linspace(2000, 2001, 101)
    s = Spectrum(dict(wavenumber=w, abscoeff=np.full(101, 0.5)),
                 conditions=dict(path_length=2.0, Tgas=500.0))
    ww, T = s.get("transmittance_noslit")
    np.testing.assert_allclose(T, np.exp(-1.0))
    s.crop(2000.2, 2000.4)
    assert s.get("abscoeff")[0][0] == pytest.approx(2000.2)
    with pytest.warns(UserWarning):
        assert s.recalc_gpu("abscoeff", Tgas=600) is None


def test_calc_spectrum_arguments():
    """The reference's argument order (radis/lbl/calc.py:37-75) and the
    checks made before any device work: GPU mode only, equilibrium only."""
    import inspect

    from radis_gb300.factory import calc_spectrum
    names = list(inspect.signature(calc_spectrum).parameters)
    assert names[:12] == ["wmin", "wmax", "wunit", "Tgas", "Tvib", "Trot", "Telec", "pressure", "species",
                          "isotope", "mole_fraction", "diluent"]
    lines = S.co_like(100)
    with pytest.raises(NotImplementedError):
        calc_spectrum(2000, 2010, Tgas=700.0, mode="cpu", databank=lines)
    with pytest.raises(NotImplementedError):
        calc_spectrum(2000, 2010, Tgas=700.0, Tvib=2000.0, databank=lines)
