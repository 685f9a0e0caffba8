"""Generate partition-function golden vectors by RUNNING the reference's own
tabulators (RADIS 0.17.1).

Run where the reference tree is mounted ($RADIS_REFERENCE_ROOT names the radis project root, or ``--ref``);
the tests only read the committed ``golden_partition.npz``.  The methods
are pulled out of their source files with ``ast`` and executed unchanged; the
CDSD tabulator reads its table with ``pandas.read_csv``, which is absent here,
so a minimal stand-in parses the same whitespace table with numpy.

Reference code executed (paths relative to the radis project root):
  radis/levels/partfunc_cdsd.py  PartFuncCO2_CDSDtab.__init__, _inrange, _at
                                 (cubic spline through the CDSD table)
  radis/levels/partfunc.py       PartFuncExoMol.__init__, _at (np.interp)
Table: radis/db/CO2/partition_functions.txt (the reference's CDSD-4000 CO2
partition functions); its columns are stored with the outputs so that the
tests can rebuild the same spline.
"""
from __future__ import annotations

import argparse
import ast
import os
import textwrap

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_REF = os.environ.get("RADIS_REFERENCE_ROOT")  # the radis project root


def _methods(path, cls, names):
    src = open(path).read()
    tree = ast.parse(src)
    node = [n for n in tree.body if isinstance(n, ast.ClassDef) and n.name == cls][0]
    out = {}
    for m in node.body:
        if isinstance(m, ast.FunctionDef) and m.name in names:
            out[m.name] = textwrap.dedent(ast.get_source_segment(src, m))
    missing = set(names) - set(out)
    if missing:
        raise RuntimeError(f"not found in {path}:{cls}: {missing}")
    return out


class _Frame(dict):
    """What PartFuncCO2_CDSDtab uses of a pandas DataFrame: keys() and columns."""


class _PandasStandIn:
    @staticmethod
    def read_csv(path, comment="#", sep=None):
        rows = [ln.split() for ln in open(path) if ln.strip() and not ln.lstrip().startswith(comment)]
        head, body = rows[0], np.array(rows[1:], dtype=np.float64)
        f = _Frame()
        for i, k in enumerate(head):
            f[k] = body[:, i]
        return f


class OutOfBoundError(ValueError):
    pass


def build_class(name, methods, ns):
    body = "\n".join(textwrap.indent(src, "    ") for src in methods.values())
    src = f"class {name}:\n{body}\n"
    exec(compile(src, "<reference>", "exec"), ns)
    return ns[name]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=DEFAULT_REF, required=DEFAULT_REF is None,
                    help="radis project root (default: $RADIS_REFERENCE_ROOT)")
    ap.add_argument("--out", default=os.path.join(HERE, "golden_partition.npz"))
    args = ap.parse_args()
    ns = {"np": np, "pd": _PandasStandIn, "OutOfBoundError": OutOfBoundError}
    cdsd = build_class("PartFuncCO2_CDSDtab",
                       _methods(os.path.join(args.ref, "radis/levels/partfunc_cdsd.py"), "PartFuncCO2_CDSDtab",
                                ["__init__", "_inrange", "_at"]), ns)
    exomol = build_class("PartFuncExoMol",
                         _methods(os.path.join(args.ref, "radis/levels/partfunc.py"), "PartFuncExoMol",
                                  ["_at"]), ns)
    table = os.path.join(args.ref, "radis/db/CO2/partition_functions.txt")
    frame = _PandasStandIn.read_csv(table, comment="#")
    out = {"cdsd_T": frame["T(K)"]}
    T_eval = np.array([290.0, 296.0, 300.0, 450.0, 777.7, 1000.0, 1234.5, 2000.0, 2999.0, 3456.0])
    for iso, col in ((1, "12C16O2"), (2, "13C16O2"), (3, "16O12C18O"), (4, "16O12C17O")):
        pf = cdsd.__new__(cdsd)
        cdsd.__init__(pf, iso, table)
        out[f"cdsd_Q{iso}"] = frame[col]
        lo, hi = pf.Tmin * 0.95, pf.Tmax * 1.05
        T = np.concatenate([T_eval[(T_eval >= lo) & (T_eval <= hi)], [lo * 1.0000001, hi * 0.9999999]])
        out[f"cdsd_T_eval{iso}"] = T
        out[f"cdsd_Q_eval{iso}"] = np.array([float(pf._at(t)) for t in T])
        bad = []
        for t in (lo * 0.999, hi * 1.001):
            try:
                pf._at(t)
            except OutOfBoundError:
                bad.append(t)
        out[f"cdsd_T_refused{iso}"] = np.array(bad)
    rng = np.random.default_rng(21)
    Tt = np.sort(rng.uniform(100.0, 5000.0, 40))
    Qt = 10.0 * (Tt / 296.0) ** 1.7 * (1.0 + 0.05 * rng.normal(size=40))
    pe = exomol.__new__(exomol)
    pe.T_range, pe.Q_range = Tt, Qt
    T = np.concatenate([[50.0, 100.0], rng.uniform(Tt[0], Tt[-1], 20), [Tt[5], 6000.0]])
    out["exomol_T"], out["exomol_Q"], out["exomol_T_eval"] = Tt, Qt, T
    out["exomol_Q_eval"] = np.array([float(pe._at(t)) for t in T])
    np.savez_compressed(args.out, **out)
    print("wrote", args.out, len(out), "arrays")


if __name__ == "__main__":
    main()
