"""Tabulated partition functions Q(T) evaluated by the library.

The reference's GPU path takes one Q(T) callable per isotopologue and
evaluates them on the host at every iterate (radis/gpu/params.py:154-155);
its tabulated sources interpolate a (T, Q) table with a cubic spline (CDSD
CO2, radis/levels/partfunc_cdsd.py:84-117) or linearly (ExoMol,
radis/levels/partfunc.py:1191-1192).  ``TabulatedQ`` is such a callable,
evaluated by the library's own interpolation (``rg_partition_eval``), and a
line list can hold the tables itself (``Lines.set_partition``), after which
``q_ratio=None`` means Q(Tref)/Q(T) from them -- no per-spectrum host
callables, and the derivatives get d ln Q / dT from the same spline.
"""
from __future__ import annotations

import numpy as np

from . import _lib as L

# isotopologue columns of the CDSD-4000 table (partfunc_cdsd.py:74)
CDSD_ISOTOPES = {1: "12C16O2", 2: "13C16O2", 3: "16O12C18O", 4: "16O12C17O"}


class TabulatedQ:
    """Q(T) from a table: ``kind`` 'cubic' (splrep/splev spline, refused beyond
    [0.95 Tmin, 1.05 Tmax]) or 'linear' (np.interp)."""

    def __init__(self, T, Q, kind="cubic"):
        self.T = np.ascontiguousarray(T, dtype=np.float64)
        self.Q = np.ascontiguousarray(Q, dtype=np.float64)
        if kind not in L.PARTITION_KINDS:
            raise ValueError(f"kind must be one of {sorted(L.PARTITION_KINDS)}")
        self.kind = kind
        L.partition_eval(self.T, self.Q, kind, float(self.T[0]))   # validates the table
        self.Tmin, self.Tmax = float(self.T[0]), float(self.T[-1])

    def at(self, T):
        """Q at temperature T (the reference's RovibParFuncTabulator.at)."""
        return L.partition_eval(self.T, self.Q, self.kind, float(T))[0]

    def dQ_dT(self, T):
        return L.partition_eval(self.T, self.Q, self.kind, float(T))[1]

    __call__ = at


def load_cdsd_table(path, isotopes=(1, 2, 3, 4)):
    """{isotope number: TabulatedQ} from a CDSD partition-function table
    (whitespace columns 'T(K)' and the isotopologue names, '#' comments), as
    PartFuncCO2_CDSDtab reads it (partfunc_cdsd.py:84-99)."""
    rows = [ln.split() for ln in open(path) if ln.strip() and not ln.lstrip().startswith("#")]
    head = rows[0]
    data = np.array(rows[1:], dtype=np.float64)
    if "T(K)" not in head:
        raise KeyError(f"Missing columns (T(K)) in {path}")
    T = data[:, head.index("T(K)")]
    out = {}
    for iso in isotopes:
        if iso not in CDSD_ISOTOPES:
            raise KeyError(f"Isotope {iso} not defined in CDSD tabulated partition functions")
        out[iso] = TabulatedQ(T, data[:, head.index(CDSD_ISOTOPES[iso])], kind="cubic")
    return out
