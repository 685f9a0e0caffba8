"""The CPU oracle against golden vectors produced by running the reference's
own functions (tests/golden/make_golden.py)."""
import numpy as np
import pytest

from oracle import ldm_oracle as O

CASES = ["hitran_co_700K", "hitran_co_3000K", "synth_fold", "synth_1atm", "hitran_co_10bar", "synth_self_hot"]
COLS = ["v0", "S_ref", "El", "g_air", "g_self", "n_air", "delta"]


def _case(g, name):
    c = lambda k: float(g[f"{name}/cond_{k}"])
    lines = {k: g[f"{name}/in_{k}"] for k in COLS}
    n_v = int(round((c("wmax") - c("wmin")) / c("wstep"))) + 1
    return lines, c, n_v


@pytest.mark.parametrize("name", CASES)
def test_line_quantities(golden, name):
    lines, c, n_v = _case(golden, name)
    kpos, lgG, lgL, S = O.line_quantities(lines, c("T"), c("p_bar"), c("x"), c("wmin"), c("wstep"),
                                          Qref_Qgas=c("Qr"), molar_mass=c("M"))
    order = np.argsort(kpos, kind="mergesort")   # the reference sorts by shiftwav
    np.testing.assert_allclose(S[order], golden[f"{name}/out_S"], rtol=1e-13)
    np.testing.assert_allclose(np.exp(lgG[order]), 2 * golden[f"{name}/out_hwhm_g"], rtol=1e-13)
    np.testing.assert_allclose(np.exp(lgL[order]), 2 * golden[f"{name}/out_hwhm_l"], rtol=1e-13)
    shift = golden[f"{name}/out_shiftwav"]
    np.testing.assert_allclose(c("wmin") + kpos[order] * c("wstep"), shift, rtol=0, atol=1e-9)


@pytest.mark.parametrize("name", CASES)
def test_cpu_axes(golden, name):
    lines, c, n_v = _case(golden, name)
    _, lgG, lgL, _ = O.line_quantities(lines, c("T"), c("p_bar"), c("x"), c("wmin"), c("wstep"),
                                       molar_mass=c("M"))
    np.testing.assert_allclose(O.cpu_w_axis(np.exp(lgG), c("dxG")), golden[f"{name}/out_wG"], rtol=1e-13)
    np.testing.assert_allclose(O.cpu_w_axis(np.exp(lgL), c("dxL")), golden[f"{name}/out_wL"], rtol=1e-13)


@pytest.mark.parametrize("name", CASES)
def test_lineshape_profiles(golden, name):
    lines, c, n_v = _case(golden, name)
    wG, wL = golden[f"{name}/out_wG"], golden[f"{name}/out_wL"]
    key = f"{name}/out_profiles"
    stride = 1
    if key not in golden:
        key, stride = f"{name}/out_profiles_stride41", 41
    P = golden[key]
    for l in range(len(wG)):
        for m in range(len(wL)):
            mine = O.lineshape_ft(2 * n_v, c("wstep"), wG[l], wL[m])[::stride]
            np.testing.assert_allclose(mine, P[l, m], rtol=1e-12, atol=1e-15)


def test_folding_exercised(golden):
    """At least one golden case adds folding terms (broadening.py:1914-1926)."""
    wG, wL = golden["synth_fold/out_wG"], golden["synth_fold/out_wL"]
    assert O.fold_count(float(golden["synth_fold/cond_wstep"]), wG[0], wL[0]) > 0


@pytest.mark.parametrize("name", CASES)
def test_spectrum(golden, name):
    lines, c, n_v = _case(golden, name)
    kpos, lgG, lgL, S = O.line_quantities(lines, c("T"), c("p_bar"), c("x"), c("wmin"), c("wstep"),
                                          Qref_Qgas=c("Qr"), molar_mass=c("M"))
    wG, wL = golden[f"{name}/out_wG"], golden[f"{name}/out_wL"]
    axes = (np.log(wG[0]), c("dxG"), len(wG), np.log(wL[0]), c("dxL"), len(wL))
    LDM = O.ldm_scatter(kpos, lgG, lgL, S, n_v, axes, n_rows=2 * n_v)
    spec = O.ldm_convolve(LDM, n_v, c("wstep"), axes, 2 * n_v)
    ref = golden[f"{name}/out_sumoflines"]
    assert np.max(np.abs(spec - ref)) <= 1e-10 * np.max(np.abs(ref))


def test_envelope_rule_matches_reference_gpu_params(golden):
    """The oracle's brute-force restatement of radis/gpu/params.py against the
    reference's own outputs (pressure given in the width unit)."""
    rows = golden["grid/rows"]
    dxG, dxL = float(golden["grid/dxG"]), float(golden["grid/dxL"])
    for gi in (0, 1):
        v0 = golden[f"grid{gi}/in_v0"]
        lines = dict(v0=v0, g_air=golden[f"grid{gi}/in_g_air"], g_self=golden[f"grid{gi}/in_g_self"],
                     n_air=golden[f"grid{gi}/in_n_air"])
        for _, T, p, lgmin, NG, llmin, NL in rows[rows[:, 0] == gi]:
            ax = O.envelope_axes(lines, T, p * 1.01325, 0.1, dxG=dxG, dxL=dxL, molar_mass=28.0)
            assert (ax[2], ax[5]) == (NG, NL)
            assert abs(ax[0] - lgmin) < 2e-5 and abs(ax[3] - llmin) < 2e-5
