"""Tabulated partition functions: the oracle and the library's host
interpolation (rg_partition_eval, radis_gb300.partition) against golden
vectors from the reference's own tabulators (CDSD cubic spline through
radis/db/CO2/partition_functions.txt, ExoMol np.interp;
tests/golden/make_golden_partition.py).

Tolerances: oracle 1e-12 relative (same scipy spline); library 1e-11
relative for Q (its own not-a-knot spline, piecewise-polynomial evaluation
instead of de Boor's), 1e-8 relative for dQ/dT against splev(der=1)."""
import os

import numpy as np
import pytest

from oracle import partition_oracle as PO
from radis_gb300 import _lib as L
from radis_gb300 import partition as P

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_partition.npz"))
ISOS = (1, 2, 3, 4)


@pytest.mark.parametrize("iso", ISOS)
def test_oracle_cdsd(iso):
    T, Q = G["cdsd_T"], G[f"cdsd_Q{iso}"]
    for t, want in zip(G[f"cdsd_T_eval{iso}"], G[f"cdsd_Q_eval{iso}"]):
        assert abs(PO.cubic_Q(T, Q, t) - want) <= 1e-12 * want
    for t in G[f"cdsd_T_refused{iso}"]:
        with pytest.raises(PO.OutOfRange):
            PO.cubic_Q(T, Q, t)


def test_oracle_exomol():
    for t, want in zip(G["exomol_T_eval"], G["exomol_Q_eval"]):
        assert PO.linear_Q(G["exomol_T"], G["exomol_Q"], t) == want


@pytest.mark.parametrize("iso", ISOS)
def test_library_cubic(native_lib, iso):
    T, Q = G["cdsd_T"], G[f"cdsd_Q{iso}"]
    for t, want in zip(G[f"cdsd_T_eval{iso}"], G[f"cdsd_Q_eval{iso}"]):
        q, dq = L.partition_eval(T, Q, "cubic", t)
        assert abs(q - want) <= 1e-11 * want
        d_ref = PO.cubic_dQ(T, Q, t)
        assert abs(dq - d_ref) <= 1e-8 * max(abs(d_ref), 1e-300) + 1e-12 * want
    for t in G[f"cdsd_T_refused{iso}"]:
        with pytest.raises(L.RgError) as e:
            L.partition_eval(T, Q, "cubic", t)
        assert e.value.code == 5   # RG_ERR_RANGE


def test_library_linear(native_lib):
    T, Q = G["exomol_T"], G["exomol_Q"]
    for t, want in zip(G["exomol_T_eval"], G["exomol_Q_eval"]):
        q, dq = L.partition_eval(T, Q, "linear", t)
        assert abs(q - want) <= 1e-14 * want
        if T[0] < t < T[-1] and not np.any(T == t):
            i = np.searchsorted(T, t) - 1
            assert abs(dq - (Q[i + 1] - Q[i]) / (T[i + 1] - T[i])) <= 1e-12 * abs(dq)


def test_library_small_cubic_is_the_cubic_through_four_points(native_lib):
    T = np.array([100.0, 250.0, 300.0, 700.0])
    Q = 2.0 + 0.01 * T - 3e-5 * T ** 2 + 2e-8 * T ** 3
    for t in (95.0, 180.0, 500.0, 735.0):
        want = 2.0 + 0.01 * t - 3e-5 * t ** 2 + 2e-8 * t ** 3
        assert abs(L.partition_eval(T, Q, "cubic", t)[0] - want) <= 1e-12 * want


def test_library_errors(native_lib):
    with pytest.raises(L.RgError):
        L.partition_eval([300.0, 200.0, 400.0, 500.0], [1.0, 2.0, 3.0, 4.0], "cubic", 300.0)   # not increasing
    with pytest.raises(L.RgError):
        L.partition_eval([200.0, 300.0, 400.0], [1.0, 2.0, 3.0], "cubic", 300.0)               # < 4 points
    with pytest.raises(L.RgError):
        L.partition_eval([200.0, 300.0], [1.0, -2.0], "linear", 250.0)                         # Q <= 0
    with pytest.raises(ValueError):
        P.TabulatedQ([200.0, 300.0], [1.0, 2.0], kind="spline")


def test_load_cdsd_table(native_lib, tmp_path):
    path = tmp_path / "partition_functions.txt"
    with open(path, "w") as f:
        f.write("# CDSD-style table\n#\n  T(K)  " + "  ".join(P.CDSD_ISOTOPES[i] for i in ISOS) + "\n")
        for k, t in enumerate(G["cdsd_T"]):
            f.write(f"  {float(t)!r}  " + "  ".join(repr(float(G[f'cdsd_Q{i}'][k])) for i in ISOS) + "\n")
    tabs = P.load_cdsd_table(str(path))
    for iso in ISOS:
        for t, want in zip(G[f"cdsd_T_eval{iso}"], G[f"cdsd_Q_eval{iso}"]):
            assert abs(tabs[iso](t) - want) <= 1e-11 * want
