"""CPU-only checks of the native library: it builds, loads, exports every
symbol the header declares, and its host-side grid rules (the reference's
radis/gpu/params.py) are right.  No compute call needs a GPU here."""
import os
import re
import subprocess

import numpy as np
import pytest

from oracle import ldm_oracle as O
from radis_gb300 import _lib as L
from radis_gb300 import synthetic as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "radis_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\*?(rg_\w+)\s*\(", txt, re.M)))


def test_exports_match_header(native_lib):
    declared = header_symbols()
    assert declared, "no rg_ symbols parsed from the header"
    assert sorted(L.EXPORTS) == declared
    for name in declared:
        assert hasattr(native_lib, name)
    out = subprocess.run(["nm", "-D", "--defined-only", L.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (rg_\w+)", out))
    assert set(declared) <= exported


def test_abi_version(native_lib):
    assert native_lib.rg_abi_version() == 3


def test_grid_matches_reference_params(native_lib, golden):
    rows = golden["grid/rows"]
    dxG, dxL = float(golden["grid/dxG"]), float(golden["grid/dxL"])
    for gi in (0, 1):
        v0 = golden[f"grid{gi}/in_v0"]
        lines = dict(v0=v0, S_ref=np.full(len(v0), 1e-20), El=np.zeros(len(v0), np.float32),
                     g_air=golden[f"grid{gi}/in_g_air"], g_self=golden[f"grid{gi}/in_g_self"],
                     n_air=golden[f"grid{gi}/in_n_air"])
        for _, T, p, lgmin, NG, llmin, NL in rows[rows[:, 0] == gi]:
            # the reference puts bar into log(2p); the build uses atm (CPU path)
            g = L.grid_estimate(lines, 28.0, 1900.0, 0.01, 1000, T, p * 1.01325, 0.1, dxG=dxG, dxL=dxL)
            assert (g.n_G, g.n_L) == (NG, NL)
            assert abs(g.log_wG_min - lgmin) < 2e-5
            assert abs(g.log_wL_min - llmin) < 2e-5


@pytest.mark.parametrize("T,p,x", [(300.0, 1.0, 0.1), (1500.0, 0.1, 0.9), (250.0, 10.0, 0.5),
                                   (3000.0, 0.5, 0.01)])
def test_grid_matches_brute_force(native_lib, T, p, x):
    lines = S.uniform_lines(20000, 2000.0, 2100.0, seed=7)
    lines["iso"] = (np.arange(20000) % 3).astype(np.uint8)
    mm = [28.0, 29.0, 30.0]
    g = L.grid_estimate(lines, mm, 2000.0, 0.01, 10001, T, p, x, dxG=S.DXG_DEFAULT, dxL=S.DXL_DEFAULT)
    ax = O.envelope_axes(lines, T, p, x, dxG=S.DXG_DEFAULT, dxL=S.DXL_DEFAULT,
                         molar_mass=np.array(mm))
    assert (g.n_G, g.n_L) == (ax[2], ax[5])
    assert abs(g.log_wG_min - ax[0]) < 1e-9 and abs(g.log_wL_min - ax[3]) < 1e-9
    gf = L.grid_estimate(lines, mm, 2000.0, 0.01, 10001, T, p, x, n_G=8, n_L=16)
    axf = O.envelope_axes(lines, T, p, x, NG=8, NL=16, molar_mass=np.array(mm))
    assert (gf.n_G, gf.n_L) == (8, 16)
    np.testing.assert_allclose([gf.dxG, gf.dxL], [axf[1], axf[4]], rtol=1e-9)


def test_every_line_inside_its_axes(native_lib):
    """Every line's (log wG, log wL) falls inside [node 0, node N-1) of the grid."""
    lines = S.uniform_lines(50000, 2000.0, 2400.0, seed=9)
    for T, p, x in [(296.0, 1.0, 0.0), (296.0, 1.0, 1.0), (2000.0, 3.0, 0.37)]:
        g = L.grid_estimate(lines, 44.0, 2000.0, 0.01, 40001, T, p, x, dxG=0.1, dxL=0.1)
        _, lgG, lgL, _ = O.line_quantities(lines, T, p, x, 2000.0, 0.01, molar_mass=44.0)
        pl = (lgG - g.log_wG_min) / g.dxG
        pm = (lgL - g.log_wL_min) / g.dxL
        assert pl.min() >= -1e-9 and pl.max() < g.n_G - 1
        assert pm.min() >= -1e-9 and pm.max() < g.n_L - 1


@pytest.mark.parametrize("n_v", [2, 17, 1000, 200001, 400001, 1500001, 2000001])
def test_fft_length(native_lib, n_v):
    lines = S.uniform_lines(100, 2000.0, 2001.0, seed=1)
    g = L.grid_estimate(lines, 28.0, 2000.0, 0.001, n_v, 296.0, 1.0, 0.1, dxG=0.14, dxL=0.2)
    assert g.n_ft >= 2 * n_v and g.n_ft == g.n1 * g.n2
    assert g.n1 & (g.n1 - 1) == 0 and g.n2 % 32 == 0
    m = g.n2 // 32
    for pr in (2, 3, 5):
        while m % pr == 0:
            m //= pr
    assert m == 1
    assert g.n_ft <= 1.1 * 2 * n_v + 8192


def test_grid_errors(native_lib):
    lines = S.uniform_lines(100, 2000.0, 2001.0, seed=1)
    with pytest.raises(L.RgError) as e:
        L.grid_estimate(lines, 28.0, 2000.0, 0.001, 1, 296.0, 1.0, 0.1, dxG=0.14, dxL=0.2)
    assert e.value.code == 1
    bad = dict(lines)
    bad["g_air"] = np.zeros(100, np.float32)
    bad["g_self"] = np.zeros(100, np.float32)
    with pytest.raises(L.RgError) as e:
        L.grid_estimate(bad, 28.0, 2000.0, 0.001, 1000, 296.0, 1.0, 0.1, dxG=0.14, dxL=0.2)
    assert e.value.code == 1
    with pytest.raises(L.RgError) as e:   # node spacing so fine the grid exceeds the kernel limits
        L.grid_estimate(lines, 28.0, 2000.0, 0.001, 1000, 296.0, 1.0, 0.1, dxG=1e-4, dxL=1e-4)
    assert e.value.code == 5
    with pytest.raises(L.RgError):
        L.grid_estimate(lines, 28.0, 2000.0, 0.001, 1000, -5.0, 1.0, 0.1, dxG=0.14, dxL=0.2)
    iso = dict(lines)
    iso["iso"] = np.full(100, 3, np.uint8)
    with pytest.raises(L.RgError):
        L.grid_estimate(iso, [28.0, 29.0], 2000.0, 0.001, 1000, 296.0, 1.0, 0.1, dxG=0.14, dxL=0.2)


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(L.NativeLibraryError):
        saved = L._lib
        L._lib = None
        try:
            L.load(str(tmp_path / "nope.so"))
        finally:
            L._lib = saved


def test_grid_independent_of_line_order(native_lib):
    """The host envelopes split their passes over threads (>= 2^18 lines per
    chunk); the merges reproduce the sequential result, so the grid does not
    depend on how the lines fall into chunks: a shuffled list of 600k lines
    (several chunks) gives the same grid bit for bit, and so do the error
    reports of a bad line in a late chunk."""
    lines = S.co2_like(600_000, seed=3)
    perm = np.random.default_rng(4).permutation(600_000)
    shuf = {k: (v[perm] if isinstance(v, np.ndarray) else v) for k, v in lines.items()}
    for kw in (dict(n_G=8, n_L=16), dict(dxG=0.1, dxL=0.2)):
        for T, p, x in ((296.0, 1.0, 0.1), (2500.0, 0.2, 0.7)):
            a = L.grid_estimate(lines, 44.0, 2000.0, 0.001, 400001, T, p, x, **kw)
            b = L.grid_estimate(shuf, 44.0, 2000.0, 0.001, 400001, T, p, x, **kw)
            assert bytes(a) == bytes(b)
    bad = dict(lines)
    bad["v0"] = lines["v0"].copy()
    bad["v0"][[555_555, 555_556]] = -1.0
    with pytest.raises(L.RgError, match=r"v0\[555555\]"):
        L.grid_estimate(bad, 44.0, 2000.0, 0.001, 400001, 296.0, 1.0, 0.1, n_G=8, n_L=16)


def test_window_axes_cover_window_lines(native_lib):
    """axes_window: the Gaussian node axis of a narrow window of a wide list
    spans the lines that can reach the window -- every such line's log wG lies
    on the axis -- with far fewer nodes than the whole-list axis; the
    Lorentzian axis is unchanged.  A window with no line falls back to the
    whole list."""
    import numpy as np

    from oracle import ldm_oracle as O
    lines = S.h2o_like(400_000, seed=4)
    T, p, x, dv = 2000.0, 1.0, 0.2, 0.005
    kw = dict(dxG=S.DXG_DEFAULT, dxL=S.DXL_DEFAULT)
    full = L.grid_estimate(lines, 18.0, 3700.0, dv, 10001, T, p, x, **kw)
    win = L.grid_estimate(lines, 18.0, 3700.0, dv, 10001, T, p, x, axes_window=True, **kw)
    assert win.n_G < full.n_G / 4
    assert (win.n_L, win.log_wL_min, win.dxL) == (full.n_L, full.log_wL_min, full.dxL)
    v0 = np.asarray(lines["v0"])
    sel = (v0 >= 3700.0 - dv) & (v0 <= 3700.0 + 10000 * dv + dv)
    lgG = np.log(2.0 * O.doppler_hwhm(v0[sel], 18.0, T))
    top = win.log_wG_min + (win.n_G - 1) * win.dxG
    assert lgG.min() >= win.log_wG_min - 1e-12 and lgG.max() <= top + 1e-12
    empty = L.grid_estimate(lines, 18.0, 9000.0, dv, 1001, T, p, x, axes_window=True, **kw)
    assert (empty.n_G, empty.log_wG_min) == (full.n_G, full.log_wG_min)
