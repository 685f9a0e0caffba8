"""Skeleton layout, host side (no GPU): the decomposition of the nodes'
lineshape transforms that rg_grid_skeleton returns -- and every plan makes
per spectrum -- checked against the oracle's folded Voigt transforms
(radis/lbl/broadening.py:1896-1926) on the whole DFT grid, and the
projected-rows identity checked end to end in FP64 on a small spectrum."""
import numpy as np
import pytest

from oracle import ldm_oracle as O
from radis_gb300 import _lib as L
from radis_gb300 import synthetic as S


def grid_of(axes, n_ft=0):
    g = L.Grid()
    g.log_wG_min, g.dxG, g.n_G, g.log_wL_min, g.dxL, g.n_L = axes
    g.n_ft = n_ft
    return g


def transforms(axes, n_ft, dv, thresh=1e-6):
    wG = O.axis_values(*axes[:3])
    wL = O.axis_values(*axes[3:])
    return np.array([O.lineshape_ft(n_ft, dv, wG[l], wL[m], thresh)
                     for l in range(len(wG)) for m in range(len(wL))])


# (lines, molar mass, vmin, dv, n_v, T, p, x, grid): a CO2-like 8 x 16 grid,
# a grid with folded copies (widths near the step), a wide H2O-like one
CASES = {
    "co2_8x16": (lambda: S.uniform_lines(100_000, 2000.0, 2400.0, seed=2), 44.0, 2000.0, 0.001, 400001,
                 1500.0, 1.0, 0.1, dict(n_G=8, n_L=16)),
    "folded": (lambda: S.uniform_lines(3000, 2000.0, 2010.0, seed=22), 28.0, 2000.0, 0.02, 501,
               1500.0, 0.01, 0.3, dict(dxG=S.DXG_DEFAULT, dxL=S.DXL_DEFAULT)),
    "h2o_12x24": (lambda: S.uniform_lines(100_000, 500.0, 8000.0, seed=3), 18.0, 500.0, 0.005, 1500001,
                  2000.0, 1.0, 0.2, dict(n_G=12, n_L=24)),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_skeleton_spans_every_transform(native_lib, case):
    make, M, vmin, dv, n_v, T, p, x, grid = CASES[case]
    g = L.grid_estimate(make(), M, vmin, dv, n_v, T, p, x, **grid)
    axes = g.axes()
    tol = 1e-8
    nodes, coef, err = L.grid_skeleton(g, dv, tol=tol)
    n = g.n_G * g.n_L
    R = len(nodes)
    assert 0 < R < n and err <= tol
    assert coef.shape == (R, n)
    # skeleton columns reproduce themselves exactly
    assert np.array_equal(coef[:, nodes], np.eye(R))
    assert np.max(np.abs(coef)) < 4.0
    V = transforms(axes, 2 * n_v, dv)
    full = np.max(np.abs(coef.T @ V[nodes] - V))
    assert full <= 3 * tol, full


def test_skeleton_rank_follows_tolerance(native_lib):
    make, M, vmin, dv, n_v, T, p, x, grid = CASES["co2_8x16"]
    g = L.grid_estimate(make(), M, vmin, dv, n_v, T, p, x, **grid)
    ranks = [len(L.grid_skeleton(g, dv, tol=t)[0]) for t in (1e-4, 1e-6, 1e-8, 1e-10)]
    assert ranks == sorted(ranks) and ranks[0] < ranks[-1]


def test_skeleton_range_error(native_lib):
    make, M, vmin, dv, n_v, T, p, x, grid = CASES["h2o_12x24"]
    g = L.grid_estimate(make(), M, vmin, dv, n_v, T, p, x, **grid)
    with pytest.raises(L.RgError, match="RANGE"):
        L.grid_skeleton(g, dv, tol=1e-8, r_max=4)
    with pytest.raises(L.RgError):
        L.grid_skeleton(g, -1.0)


def test_projected_rows_give_the_reference_spectrum(native_lib):
    """FP64 restatement of the skeleton layout on the oracle's own LDM: rows
    Y_r = sum_n C[r][n] LDM_n transformed with the skeleton nodes' transforms
    give the reference's sum over all nodes within the decomposition's error."""
    import scipy.fft as sfft
    lines = S.uniform_lines(20_000, 2000.0, 2040.0, seed=5)
    M, vmin, dv, n_v, T, p, x = 44.0, 2000.0, 0.001, 40001, 1500.0, 1.0, 0.1
    g = L.grid_estimate(lines, M, vmin, dv, n_v, T, p, x, n_G=8, n_L=16)
    axes = g.axes()
    n_ft = 2 * n_v
    nodes, coef, err = L.grid_skeleton(g, dv)
    kpos, lgG, lgL, Sv = O.line_quantities(lines, T, p, x, vmin, dv, molar_mass=M)
    ldm = O.ldm_scatter(kpos, lgG, lgL, Sv, n_v, axes)          # [n_v][n_G][n_L]
    rows = ldm.reshape(n_v, -1).T                               # node l n_L + m
    ref = O.ldm_convolve(ldm, n_v, dv, axes, n_ft)
    V = transforms(axes, n_ft, dv)
    Y = np.zeros((len(nodes), n_ft))
    Y[:, :n_v] = coef @ rows
    out = sfft.irfft((sfft.rfft(Y, axis=1) * V[nodes]).sum(0), n=n_ft)[:n_v] / dv
    assert np.max(np.abs(out - ref)) <= 1e-7 * np.max(np.abs(ref))


def test_flush_node_order_covers_and_spreads_banks(native_lib):
    """The scatter's tensor-core flush reads a tile's node rows in the order
    of rg_test_flush_order, eight nodes per step: every node appears once
    with its coefficient (repeats carry zero coefficients), and from 32 nodes
    up each A-fragment load (nodes of t = 0..3, or t + 4, at columns g = 0..7
    of a row pitch of 1 mod 32 words) touches 32 distinct banks.  Below 32
    nodes the natural order, padded to a step."""
    for n in range(1, 161):
        nodes, real = L.flush_order(n)
        assert len(nodes) % 8 == 0 and np.all((nodes >= 0) & (nodes < n)), n
        assert sorted(nodes[real].tolist()) == list(range(n)), n
        steps = len(nodes) // 8
        if n < 32:
            assert steps == (n + 7) // 8 and np.array_equal(nodes[real], np.arange(n)), n
            continue
        assert steps <= (n + 7) // 8 + 4, n
        if n % 32 == 0:
            assert steps == n // 8 and real.all(), n
        for pitch in (33, 225, 257, 1025):   # TK + 1, TK a multiple of 32
            for s in range(steps):
                for half in (0, 1):
                    banks = {(int(nodes[8 * s + t + 4 * half]) * pitch + g) % 32 for t in range(4) for g in range(8)}
                    assert len(banks) == 32, (n, pitch, s, half)

