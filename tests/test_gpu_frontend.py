"""The drop-in front end on the GPU: gpuApp (Einstein-A S0 input), the
factory's eq_spectrum_gpu on a HITRAN-160 databank file, recalc_gpu and
exit_gpu (the reference's test_gpu.py:60-197 checks, against the oracle)."""
import numpy as np
import pytest

from oracle import ldm_oracle as O
from radis_gb300 import SpectrumFactory, calc_spectrum, gpuApp, hitran
from radis_gb300 import synthetic as S
from radis_gb300.spectrum import GPUInitWarning

pytestmark = pytest.mark.gpu
TOL = 1e-4


def rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def test_gpuapp_einstein_form(native_lib):
    rng = np.random.default_rng(41)
    n = 20000
    lines = S.uniform_lines(n, 2100.0, 2120.0, seed=41, delta=(-0.004, 0.0))
    iso = rng.integers(1, 3, n)
    Mm = np.array([0.0, 28.0, 29.0])
    Q = [lambda T: 1.0, lambda T: 0.37 * T, lambda T: 0.8 * T ** 1.1]
    Qref = np.array([q(296.0) for q in Q])
    # S0 giving S_ref at 296 K: inverse of the gpuApp conversion
    S0 = lines["S_ref"] * Qref[iso] * np.exp(O.HC_K * lines["El"].astype(float) / 296.0) \
        / (-np.expm1(-O.HC_K * lines["v0"] / 296.0))
    vmin, dv, Nv = 2100.0, 0.002, 10001
    app = gpuApp(vmin, Nv, dv, S.DXG_DEFAULT, S.DXL_DEFAULT, lines["v0"], lines["delta"],
                 lines["n_air"], S0, lines["El"], np.stack([lines["g_self"], lines["g_air"]]), iso,
                 Mm, Q)
    T, p, x = 1100.0, 0.7, 0.3
    k, times = app.iterate(p, T, x)
    assert set(times) >= {"scatter", "total"}
    n_L, n_G = app.get_griddims()
    g = app.last_info.grid
    assert (n_L, n_G) == (g.n_L, g.n_G)
    qr = np.array([Qref[i] / Q[i](T) for i in range(3)])
    lines["iso"] = iso
    ref = O.synthesize(lines, T, p, x, vmin, dv, Nv, g.axes(), g.n_ft, Qref_Qgas=qr,
                       molar_mass=np.array([1.0, 28.0, 29.0]))
    assert rel(k, ref) <= TOL
    app.free()
    app.free()   # idempotent, as gpu.py:376-380
    with pytest.raises(RuntimeError):
        app.iterate(p, T, x)


@pytest.fixture(scope="module")
def co_par(tmp_path_factory):
    """The 10k-line CO-like list written as a local HITRAN-160 databank."""
    p = tmp_path_factory.mktemp("db") / "co_10k.par"
    hitran.write_hitran160(p, S.co_like())
    return p


def test_eq_spectrum_gpu_matches_oracle(native_lib, co_par):
    sf = SpectrumFactory(1900.0, 2300.0, wstep=0.002, molecule="CO", isotope="1",
                         pressure=1.01325, mole_fraction=0.1, path_length=1.0)
    sf.load_databank(co_par)
    s = sf.eq_spectrum_gpu(Tgas=700.0, name="GPU")
    assert set(s.get_vars()) >= {"abscoeff", "absorbance", "emissivity_noslit",
                                 "transmittance_noslit", "radiance_noslit"}
    for key in ("calculation_time", "lines_calculated", "thermal_equilibrium", "diluents",
                "radis_version", "gpu_backend", "spectral_points", "add_at_used", "NwL", "NwG"):
        assert key in s.conditions
    d = hitran.read_hitran160(co_par)
    g = s.gpu_app.last_info.grid
    ref = O.synthesize(d, 700.0, 1.01325, 0.1, 1900.0, 0.002, 200001, g.axes(), g.n_ft,
                       molar_mass=27.994915)
    w, k = s.get("abscoeff")
    assert len(w) == 200001
    assert rel(k, ref) <= TOL
    # recalc_gpu at 3x the path length: 3x the absorbance (test_gpu.py:137-197, rtol 1e-4)
    A1 = s.get("absorbance")[1]
    A3 = s.recalc_gpu("absorbance", path_length=3.0)
    np.testing.assert_allclose(A3, 3 * A1, rtol=1e-4, atol=1e-4 * np.max(A1))
    # new temperature: same as a fresh factory call
    k2 = s.recalc_gpu("abscoeff", Tgas=1500.0)
    s2 = sf.eq_spectrum_gpu(Tgas=1500.0, path_length=3.0, exit_gpu=True)
    assert s2.gpu_app is None
    assert rel(k2, s2.get("abscoeff")[1]) <= 1e-6
    s.exit_gpu()
    with pytest.warns(GPUInitWarning):
        s.recalc_gpu(Tgas=800.0)


def test_calc_spectrum_gpu_mode(native_lib):
    lines = S.uniform_lines(5000, 2000.0, 2050.0, seed=43)
    s = calc_spectrum(2000.0, 2050.0, Tgas=900.0, pressure=2.0, mole_fraction=0.2,
                      path_length=5.0, molecule="CO2", isotope="1", databank=lines, wstep=0.005)
    w, t = s.get("transmittance_noslit")
    assert len(w) == 10001 and np.all((t >= 0) & (t <= 1))
    g = s.gpu_app.last_info.grid
    ref = O.synthesize(lines, 900.0, 2.0, 0.2, 2000.0, 0.005, 10001, g.axes(), g.n_ft,
                       molar_mass=43.98983)
    assert rel(s.get("abscoeff")[1], ref) <= TOL
    s.exit_gpu()
