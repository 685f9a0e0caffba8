"""Generate HITRAN-160 parse golden vectors by RUNNING the reference's own
parser (RADIS 0.17.1) on synthetic .par files committed beside this script.

Run where the reference tree is mounted ($RADIS_REFERENCE_ROOT names the radis project root, or ``--ref``);
the tests only read the committed ``hitran_*.par`` files and
``golden_hitran.npz``.  The ``radis`` package cannot be imported here
(pandas, astropy, numba, hapi are absent), so the parse functions are pulled
out of their source files with ``ast`` and executed unchanged, with a minimal
pandas stand-in for the DataFrame that ``_ndarray2df`` builds.

Reference code executed (paths relative to the radis project root):
  radis/api/hitranapi.py   columns_2004 (the HITRAN-2004 column table)
  radis/api/cdsdapi.py     columns_cdsdhitemp (the CDSD-HITEMP column table)
  radis/api/tools.py       _get_linereturnformat, _ndarray2df, _read_hitran_file,
                           _create_dtype, _format_dtype, _cast_to_dtype
(parse_hitran_file, tools.py:25-78, chains these; its only other work is the
optional vaex conversion.)

Fixtures (seeded; written by radis_gb300.hitran.write_hitran160):
  hitran_co_lf.par    300 CO-like records, "\\n" line ends, isotopologues 1-3,
                      intensities down to 1e-120 (three-digit exponents),
                      negative and positive pressure shifts
  hitran_co2_crlf.par 200 CO2-like records, "\\r\\n" line ends, isotopologues
                      1-9 and the HITEMP labels '0', 'A', 'B' (10, 11, 12)
  hitemp_co2_cdsd.par 150 CO2-like records in the 127-character CDSD-HITEMP
                      layout (radis/api/cdsdapi.py:47-85): the HITRAN-160
                      fields up to Pshft, then Tdpsel and the CDSD quantum
                      numbers; parsed by the reference with columns_cdsdhitemp
"""
from __future__ import annotations

import argparse
import ast
import os
import sys
from collections import OrderedDict

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
DEFAULT_REF = os.environ.get("RADIS_REFERENCE_ROOT")  # the radis project root
COLS = {"id": "id", "iso": "iso", "wav": "v0", "int": "S_ref", "A": "A", "airbrd": "g_air",
        "selbrd": "g_self", "El": "El", "Tdpair": "n_air", "Pshft": "delta", "gp": "gp", "gpp": "gpp"}


def _lines(rng, n, mol):
    v0 = np.sort(rng.uniform(1900.0, 2400.0, n))
    s = 10 ** rng.uniform(-30, -18, n)
    s[rng.choice(n, 8, replace=False)] = 10 ** rng.uniform(-120, -101, 8)
    iso = rng.integers(1, 4, n) if mol == "CO" else rng.integers(1, 13, n)
    return {"v0": v0, "S_ref": s, "A": 10 ** rng.uniform(-3, 2, n), "g_air": rng.uniform(0.03, 0.09, n),
            "g_self": rng.uniform(0.05, 0.11, n), "El": np.minimum(rng.exponential(3000.0, n), 40000.0),
            "n_air": rng.uniform(0.5, 0.8, n), "delta": rng.uniform(-0.008, 0.004, n), "iso": iso,
            "gp": rng.integers(1, 200, n).astype(float), "gpp": rng.integers(1, 200, n).astype(float)}


def write_fixtures():
    sys.path.insert(0, ROOT)
    from radis_gb300.hitran import write_hitran160
    rng = np.random.default_rng(20250614)
    p1 = os.path.join(HERE, "hitran_co_lf.par")
    write_hitran160(p1, _lines(rng, 300, "CO"), mol_id=5)
    p2 = os.path.join(HERE, "hitran_co2_crlf.par")
    write_hitran160(p2, _lines(rng, 200, "CO2"), mol_id=2)
    with open(p2, "rb") as f:
        b = f.read()
    with open(p2, "wb") as f:
        f.write(b.replace(b"\n", b"\r\n"))
    p3 = os.path.join(HERE, "hitemp_co2_cdsd.par")
    tmp = p3 + ".tmp"
    lines3 = _lines(rng, 150, "CO2")
    write_hitran160(tmp, lines3, mol_id=2)
    with open(tmp) as f:
        recs = [r.rstrip("\n")[:67] for r in f]
    os.remove(tmp)
    nself = rng.uniform(0.5, 0.8, len(recs))
    with open(p3, "w") as f:
        for i, r in enumerate(recs):
            j = int(rng.integers(0, 60))
            tail = (f"{nself[i]:5.2f}" + "  1" + " 2" + " 2" + " 1" + "1" + "       0" + " 0" + " 0" + " 0" + "1"
                    + "  3" + " 1" + f"{i % 9999:4d}" + "  0" + " 1" + "   1" + "  R" + f"{j:3d}" + "e" + "  750")
            rec = r + tail
            assert len(rec) == 127, len(rec)
            f.write(rec + "\n")
    return {"CO": p1, "CO2": p2, "CO2-CDSD": p3}


class _Str:
    def __init__(self, s):
        self.s = s

    def decode(self, enc):
        return _Series(np.array([x.decode(enc) for x in self.s.a], dtype=object))

    def strip(self):
        return _Series(np.array([x.strip() for x in self.s.a], dtype=object))


class _Series:
    def __init__(self, a):
        self.a = np.asarray(a)

    @property
    def str(self):
        return _Str(self)

    def replace(self, mapping):
        return _Series(np.array([mapping.get(x, x) for x in self.a], dtype=object))

    def astype(self, t):
        return _Series(self.a.astype(t))


class _DataFrame:
    """What _ndarray2df touches of a pandas DataFrame."""

    def __init__(self, data, columns):
        self.c = OrderedDict((k, np.asarray(data[k])) for k in columns)

    def __getitem__(self, k):
        return _Series(self.c[k])

    def __setitem__(self, k, v):
        self.c[k] = v.a if isinstance(v, _Series) else np.asarray(v)

    def __delitem__(self, k):
        del self.c[k]

    def __contains__(self, k):
        return k in self.c

    def __getattr__(self, k):   # df.branch (tools.py:148)
        if k == "c":
            raise AttributeError(k)
        try:
            return _Series(self.c[k])
        except KeyError:
            raise AttributeError(k) from None


def _reference(ref):
    api = os.path.join(ref, "radis", "api")
    src = open(os.path.join(api, "hitranapi.py")).read()
    ns = {"OrderedDict": OrderedDict}
    for node in ast.parse(src).body:
        if isinstance(node, ast.Assign) and any(getattr(t, "id", None) == "columns_2004" for t in node.targets):
            exec(compile(ast.Module([node], []), "hitranapi.py", "exec"), ns)
    src = open(os.path.join(api, "cdsdapi.py")).read()
    for node in ast.parse(src).body:
        if isinstance(node, ast.Assign) and any(getattr(t, "id", None) == "columns_cdsdhitemp"
                                                for t in node.targets):
            exec(compile(ast.Module([node], []), "cdsdapi.py", "exec"), ns)
    src = open(os.path.join(api, "tools.py")).read()
    names = {"_get_linereturnformat", "_ndarray2df", "_read_hitran_file", "_create_dtype", "_format_dtype",
             "_cast_to_dtype"}
    pd = type("pd", (), {"DataFrame": _DataFrame})
    basics = type("m", (), {"to_str": staticmethod(lambda b: b.decode() if isinstance(b, bytes) else str(b))})
    sys.modules.setdefault("radis", type(sys)("radis"))
    sys.modules.setdefault("radis.misc", type(sys)("radis.misc"))
    sys.modules["radis.misc.basics"] = basics
    ns.update({"np": np, "pd": pd})
    for node in ast.parse(src).body:
        if isinstance(node, ast.FunctionDef) and node.name in names:
            exec(compile(ast.Module([node], []), "tools.py", "exec"), ns)
    return ns


def parse_with_reference(ns, path, molecule, table="columns_2004"):
    """parse_hitran_file (tools.py:25-78) minus its vaex branch."""
    cols = ns[table]
    data = ns["_read_hitran_file"](path, cols, count=1, linereturnformat="a2")
    lr = ns["_get_linereturnformat"](data, cols, path)
    data = ns["_read_hitran_file"](path, cols, -1, lr)
    df = ns["_ndarray2df"](data, cols, lr, molecule=molecule)
    return {COLS[k]: np.asarray(df.c[k].astype(np.int64 if k in ("id", "iso") else np.float64))
            for k in COLS if k in df}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=DEFAULT_REF, required=DEFAULT_REF is None,
                    help="radis project root (default: $RADIS_REFERENCE_ROOT)")
    args = ap.parse_args()
    files = write_fixtures()
    ns = _reference(args.ref)
    out = {}
    for mol, path in files.items():
        tag = os.path.basename(path)[:-4]
        table = "columns_cdsdhitemp" if mol == "CO2-CDSD" else "columns_2004"
        for k, v in parse_with_reference(ns, path, mol.split("-")[0], table).items():
            out[f"{tag}__{k}"] = v
    np.savez_compressed(os.path.join(HERE, "golden_hitran.npz"), **out)
    print("wrote", sorted(out)[:4], "...", len(out), "arrays")


if __name__ == "__main__":
    main()
