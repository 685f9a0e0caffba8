"""CPU oracle for tabulated partition functions -- TEST INFRASTRUCTURE ONLY.

Only ``tests/`` may import this module; the library's tables
(``rg_lines_set_partition``, ``radis_gb300.partition``) never call it.

Restates the reference's two tabulators (paths relative to the radis project
root), pinned against golden vectors produced by running them
(``tests/golden/make_golden_partition.py``):

* cubic: ``PartFuncCO2_CDSDtab`` (radis/levels/partfunc_cdsd.py:84-117), an
  interpolating cubic spline ``scipy.interpolate.splrep`` / ``splev`` through
  the table, refused beyond [0.95 Tmin, 1.05 Tmax];
* linear: ``PartFuncExoMol._at`` (radis/levels/partfunc.py:1191-1192),
  ``np.interp`` (clamped to the end values).
"""
from __future__ import annotations

import numpy as np


class OutOfRange(ValueError):
    pass


def cubic_Q(T_tab, Q_tab, T):
    """partfunc_cdsd.py:92 (splrep(T, Q): k = 3, s = 0) and :105-117 (5 %
    extrapolation window, splev)."""
    from scipy.interpolate import splev, splrep

    T_tab = np.asarray(T_tab, dtype=np.float64)
    if not (T_tab.min() * 0.95 <= T <= T_tab.max() * 1.05):
        raise OutOfRange(f"Temperature: {T} is out of bounds {T_tab.min()}-{T_tab.max()}")
    return float(splev(T, splrep(T_tab, np.asarray(Q_tab, dtype=np.float64))))


def cubic_dQ(T_tab, Q_tab, T):
    """dQ/dT of the same spline (splev der=1)."""
    from scipy.interpolate import splev, splrep

    return float(splev(T, splrep(np.asarray(T_tab, np.float64), np.asarray(Q_tab, np.float64)), der=1))


def linear_Q(T_tab, Q_tab, T):
    """partfunc.py:1192."""
    return float(np.interp(T, T_tab, Q_tab))
