"""Known-answer checks of the oracle (CPU): cases whose result follows from
the method itself, beside the golden vectors of the reference's own code.

* S(T = Tref) = S_ref (radis/lbl/base.py:2664-2677 at T = Tref).
* A line exactly on a grid node puts all of its intensity in one LDM cell; a
  line half-way between nodes on all three axes puts 1/8 in each of 8 cells
  (weights radis/lbl/broadening.py:2305-2318; node axes with power-of-two
  steps so that the coordinates are exact).
* The spectrum conserves area: the normalised (folded) Voigt FT is 1 at zero
  frequency, so over the whole FFT length sum(abscoeff) dv = sum(I) up to
  rounding, for wide, narrow and folded nodes alike; inside the window the
  loss is the Lorentzian tail beyond it.
* Linearity in the intensities: doubling every S_ref doubles the spectrum
  bit for bit (each operation scales exactly by a power of two).
"""
import numpy as np

from oracle import ldm_oracle as O
from radis_gb300 import synthetic as S

AXES = (-3.0, 0.125, 6, -4.0, 0.25, 7)   # log_wG_min, dxG, N_G, log_wL_min, dxL, N_L


def test_line_strength_at_tref():
    rng = np.random.default_rng(1)
    S_ref = 10 ** rng.uniform(-26, -19, 100)
    El = rng.uniform(0, 20000, 100)
    v0 = rng.uniform(500, 8000, 100)
    np.testing.assert_allclose(O.line_strength_eq(S_ref, El, v0, O.TREF), S_ref, rtol=1e-15)


def test_line_on_a_node_fills_one_cell():
    lg0, dxG, _, ll0, dxL, _ = AXES
    I = np.array([3.0e-20])
    LDM = O.ldm_scatter(np.array([1000.0]), np.array([lg0 + 2 * dxG]), np.array([ll0 + 3 * dxL]), I, 4001, AXES)
    nz = np.argwhere(LDM)
    assert nz.tolist() == [[1000, 2, 3]]
    assert LDM[1000, 2, 3] == I[0]


def test_line_between_nodes_splits_in_eighths():
    lg0, dxG, _, ll0, dxL, _ = AXES
    I = np.array([8.0])
    LDM = O.ldm_scatter(np.array([1000.5]), np.array([lg0 + 2.5 * dxG]), np.array([ll0 + 3.5 * dxL]), I, 4001,
                        AXES)
    nz = sorted(map(tuple, np.argwhere(LDM).tolist()))
    assert nz == [(k, l, m) for k in (1000, 1001) for l in (2, 3) for m in (3, 4)]
    assert all(LDM[c] == 1.0 for c in nz)


def _lines_on_grid(n, seed):
    """n lines at random positions and widths inside the axes."""
    rng = np.random.default_rng(seed)
    lg0, dxG, NG, ll0, dxL, NL = AXES
    kpos = rng.uniform(500, 3500, n)
    lgG = rng.uniform(lg0, lg0 + (NG - 1) * dxG, n)
    lgL = rng.uniform(ll0, ll0 + (NL - 1) * dxL, n)
    return kpos, lgG, lgL, 10 ** rng.uniform(-22, -19, n)


def test_area_conserved_over_the_whole_transform():
    n_ft = 8192
    for dv in (0.001, 0.02):   # 0.02: the narrow nodes fold (FT above 1e-6 at Nyquist)
        kpos, lgG, lgL, I = _lines_on_grid(50, 2)
        LDM = O.ldm_scatter(kpos, lgG, lgL, I, n_ft, AXES)
        out = O.ldm_convolve(LDM, n_ft, dv, AXES, n_ft)
        assert abs(out.sum() * dv / I.sum() - 1) < 1e-12
    wG = O.axis_values(AXES[0], AXES[1], AXES[2])
    wL = O.axis_values(AXES[3], AXES[4], AXES[5])
    assert O.fold_count(0.02, wG[0], wL[0]) > 0 and O.fold_count(0.001, wG[-1], wL[-1]) == 0


def test_area_in_the_window_loses_the_lorentz_tail():
    """One line at the centre of a 4001-point window (dv = 0.001) on the node
    wG = e^-3, wL = e^-4 (HWHM 0.0092 cm-1).  The transform is circular
    (period P = n_ft dv), so the window loses only the mass of the periodised
    profile that lands on the 4191 points after it, 2.0005 to 6.1915 cm-1 from
    the line: sum_k F(6.1915 + k P) - F(2.0005 + k P) with the Lorentzian CDF
    F (2.3e-3; the Gaussian core adds nothing that far out)."""
    n_v, dv, n_ft = 4001, 0.001, 8192
    lg0, _, _, ll0, _, _ = AXES
    LDM = O.ldm_scatter(np.array([2000.0]), np.array([lg0]), np.array([ll0]), np.array([1.0]), n_v, AXES)
    area = O.ldm_convolve(LDM, n_v, dv, AXES, n_ft).sum() * dv
    gamma, P = np.exp(ll0) / 2, n_ft * dv
    k = np.arange(-100000, 100001)
    F = lambda x: np.arctan(x / gamma) / np.pi
    lost = np.sum(F(6.1915 + k * P) - F(2.0005 + k * P))
    assert 0.97 * lost < 1 - area < 1.03 * lost


def test_linear_in_intensity_bit_exact():
    lines = S.co_like(2000)
    lines2 = dict(lines)
    lines2["S_ref"] = lines["S_ref"] * 2
    kpos, lgG, lgL, _ = O.line_quantities(lines, 700.0, 1.01325, 0.1, 1900.0, 0.002, molar_mass=28.0)
    axes = (lgG.min() - 1e-9, 0.1, int(np.ceil((lgG.max() - lgG.min()) / 0.1)) + 2,
            lgL.min() - 1e-9, 0.2, int(np.ceil((lgL.max() - lgL.min()) / 0.2)) + 2)
    a = O.synthesize(lines, 700.0, 1.01325, 0.1, 1900.0, 0.002, 20001, axes, 40960)
    b = O.synthesize(lines2, 700.0, 1.01325, 0.1, 1900.0, 0.002, 20001, axes, 40960)
    assert np.array_equal(b, 2 * a) and np.abs(a).max() > 0
