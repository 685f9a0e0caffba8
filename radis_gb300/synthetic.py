"""Seeded synthetic line lists standing in for the line databases of the
benchmark configurations (no network, no HITRAN/HITEMP download).

* ``co_like``   10k lines, v0 ~ U(1900, 2300) cm-1, M = 28
* ``co2_like``  5M lines,  v0 ~ U(2000, 2400) cm-1, M = 44
* ``h2o_like``  100M lines over 500-8000 cm-1 with density peaked near 1600 and
  3700 cm-1 (mixture below), M = 18

Shared distributions: S_ref log-uniform, E_low exponential (capped), g_air ~
U(0.03, 0.08), g_self ~ U(0.05, 0.1) cm-1/atm, n_air ~ U(0.5, 0.8), no pressure
shift.  Columns follow the reference's line-database names
(radis/api/hitranapi.py:82-105): wav->v0, int->S_ref, El, airbrd->g_air,
selbrd->g_self, Tdpair->n_air, Pshft->delta.  v0 is returned sorted.
"""
from __future__ import annotations

import numpy as np

# mixture used for the H2O-like v0 density (weights, log-normal centres and
# log-widths); the remainder is log-uniform over the whole range
H2O_BANDS = ((0.45, 1600.0, 0.06), (0.35, 3700.0, 0.04))
H2O_RANGE = (500.0, 8000.0)


def _common(rng, n, s_lo, s_hi, el_mean, el_cap):
    return dict(
        S_ref=10.0 ** rng.uniform(np.log10(s_lo), np.log10(s_hi), n),
        El=np.minimum(rng.exponential(el_mean, n), el_cap).astype(np.float32),
        g_air=rng.uniform(0.03, 0.08, n).astype(np.float32),
        g_self=rng.uniform(0.05, 0.1, n).astype(np.float32),
        n_air=rng.uniform(0.5, 0.8, n).astype(np.float32),
    )


def uniform_lines(n, lo, hi, seed, s_lo=1e-26, s_hi=1e-19, el_mean=3000.0, el_cap=20000.0,
                  delta=None):
    rng = np.random.default_rng(seed)
    d = dict(v0=np.sort(rng.uniform(lo, hi, n)))
    d.update(_common(rng, n, s_lo, s_hi, el_mean, el_cap))
    if delta is not None:
        d["delta"] = rng.uniform(delta[0], delta[1], n).astype(np.float32)
    return d


def co_like(n=10_000, seed=1):
    """CO-like list of the 10k-line CPU configuration."""
    return uniform_lines(n, 1900.0, 2300.0, seed)


def co2_like(n=5_000_000, seed=2):
    """CO2-like list of the 5M-line GPU configuration."""
    return uniform_lines(n, 2000.0, 2400.0, seed)


def h2o_like(n=100_000_000, seed=3):
    """H2O-like list of the 100M-line scale configuration."""
    rng = np.random.default_rng(seed)
    lo, hi = H2O_RANGE
    which = rng.uniform(0.0, 1.0, n)
    v0 = np.empty(n)
    edge = 0.0
    taken = np.zeros(n, dtype=bool)
    for w, centre, sig in H2O_BANDS:
        sel = (which >= edge) & (which < edge + w)
        v0[sel] = np.exp(rng.normal(np.log(centre), sig, sel.sum()))
        taken |= sel
        edge += w
    rest = ~taken
    v0[rest] = np.exp(rng.uniform(np.log(lo), np.log(hi), rest.sum()))
    v0 = np.clip(v0, lo, hi - 1e-6)
    v0.sort()
    d = dict(v0=v0)
    d.update(_common(rng, n, 1e-30, 1e-18, 5000.0, 40000.0))
    return d


# (lines factory, molar mass, vmin, vmax, wstep, T, p_bar, x, n_G, n_L)
CONFIGS = {
    "co_10k": (co_like, 28.0, 1900.0, 2300.0, 0.002, 700.0, 1.01325, 0.1, None, None),
    "co2_5M": (co2_like, 44.0, 2000.0, 2400.0, 0.001, 1500.0, 1.0, 0.1, 8, 16),
    "h2o_100M": (h2o_like, 18.0, 500.0, 8000.0, 0.005, 2000.0, 1.0, 0.2, 12, 24),
}

# default LDM steps of the reference (radis/lbl/loader.py:452-460,538-543)
DXL_DEFAULT = float(np.log((0.01 / 0.20) ** 0.5 + 1))
DXG_DEFAULT = float(np.log((0.01 / 0.46) ** 0.5 + 1))


def grid_points(vmin, vmax, wstep):
    return int(round((vmax - vmin) / wstep)) + 1
