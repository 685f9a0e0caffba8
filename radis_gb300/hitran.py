"""HITRAN-2004 160-character line records: reader and writer.

Column widths follow radis/api/hitranapi.py:82-105 (id a2, iso a1, wav a12,
int a10, A a10, airbrd a5, selbrd a5, El a10, Tdpair a4, Pshft a8, then the
quantum-number/reference fields, gp a7, gpp a7).  The reader keeps the
columns the equilibrium synthesis needs and returns them under the names the
rest of this package uses (v0, S_ref, A, g_air, g_self, El, n_air, delta, id,
iso, gp, gpp); iso is the HITRAN isotopologue number (1-based).
"""
from __future__ import annotations

import numpy as np

# (name, width) in record order; None = field skipped by the reader
_FIELDS = [("id", 2), ("iso", 1), ("v0", 12), ("S_ref", 10), ("A", 10), ("g_air", 5),
           ("g_self", 5), ("El", 10), ("n_air", 4), ("delta", 8), (None, 15), (None, 15),
           (None, 15), (None, 15), (None, 6), (None, 12), (None, 1), ("gp", 7), ("gpp", 7)]
RECORD = sum(w for _, w in _FIELDS)   # 160


def _iso_code(c: str) -> int:
    # HITRAN writes isotopologue 10, 11, ... as '0', 'A', 'B', ...
    if c.isdigit():
        return 10 if c == "0" else int(c)
    return 11 + ord(c.upper()) - ord("A")


def read_hitran160(path) -> dict:
    """Parse a .par file into numpy columns (float64; id/iso int64)."""
    cols = {n: [] for n, _ in _FIELDS if n}
    with open(path, "r") as f:
        for line in f:
            line = line.rstrip("\r\n")
            if len(line) < 67:
                continue
            pos = 0
            for name, w in _FIELDS:
                fld = line[pos:pos + w]
                pos += w
                if not name:
                    continue
                if name == "iso":
                    cols[name].append(_iso_code(fld.strip() or "1"))
                elif name == "id":
                    cols[name].append(int(fld))
                else:
                    fld = fld.strip()
                    cols[name].append(float(fld) if fld else np.nan)
    return {k: np.asarray(v, dtype=np.int64 if k in ("id", "iso") else np.float64)
            for k, v in cols.items()}


def _fmt_e(v, w, prec):
    s = f"{v:{w}.{prec}E}"
    while len(s) > w and prec > 0:   # three-digit exponents: drop mantissa digits
        prec -= 1
        s = f"{v:{w}.{prec}E}"
    return s


def _fmt_w(v):
    """Width field a5 ('.0567' style: HITRAN drops the leading zero)."""
    s = f"{v:6.4f}"
    if s.startswith(" 0"):
        s = s[2:]
    elif s.startswith("0"):
        s = s[1:]
    return s[:5].rjust(5)


def _fmt_shift(v):
    """Pressure-shift field a8 ('-.002750' style)."""
    s = f"{v:.6f}"
    if s.startswith("0."):
        s = s[1:]
    elif s.startswith("-0."):
        s = "-" + s[2:]
    return s.rjust(8)[:8]


def write_hitran160(path, lines: dict, mol_id: int = 5):
    """Write columns as 160-character HITRAN records; fields this package does
    not use are blank.  ``lines`` needs v0, S_ref, g_air, g_self, El, n_air and
    may hold A, delta, iso (HITRAN number, 1-based), gp, gpp."""
    n = len(lines["v0"])
    iso = np.asarray(lines.get("iso", np.ones(n, dtype=int)))
    A = np.asarray(lines.get("A", np.zeros(n)))
    delta = np.asarray(lines.get("delta", np.zeros(n)))
    gp = np.asarray(lines.get("gp", np.zeros(n)))
    gpp = np.asarray(lines.get("gpp", np.zeros(n)))
    blank = " " * (15 * 4 + 6 + 12 + 1)
    with open(path, "w") as f:
        for i in range(n):
            rec = (f"{mol_id:2d}{int(iso[i]) % 10:1d}{lines['v0'][i]:12.6f}"
                   f"{_fmt_e(lines['S_ref'][i], 10, 3)}{_fmt_e(A[i], 10, 3)}"
                   f"{_fmt_w(lines['g_air'][i])}{_fmt_w(lines['g_self'][i])}"
                   f"{lines['El'][i]:10.4f}{lines['n_air'][i]:4.2f}{_fmt_shift(delta[i])}"
                   f"{blank}{gp[i]:7.1f}{gpp[i]:7.1f}")
            if len(rec) != RECORD:
                raise ValueError(f"record {i} has {len(rec)} characters")
            f.write(rec + "\n")
