"""CPU restatement of the reference's HITRAN-160 column parse -- TEST
INFRASTRUCTURE ONLY (only ``tests/`` import it; the product reader is the
library's ``rg_hitran_parse``).

The reference reads a .par file as fixed-size byte records (numpy.fromfile
with the column widths of radis/api/hitranapi.py:82-105; parse_hitran_file,
radis/api/tools.py:25-78) and casts every numeric field to float
(_ndarray2df / _cast_to_dtype, tools.py:111-151, 214-247); for CO2 the
isotopologue labels '0', 'A', 'B' become 10, 11, 12 (tools.py:141-143).  This
restatement splits the text into lines (Python's universal newlines: "\\n",
"\\r\\n", "\\r"), slices the same fields out of each line and converts each with
float(); it is pinned against the reference's own parse of committed
synthetic files (tests/golden/make_golden_hitran.py).

Extensions over the reference, shared with the library's parser: records
shorter than 67 characters (the end of the Pshft field) are skipped, fields
past the end of a shorter record are empty, empty numeric fields read as NaN,
a blank isotopologue reads as 1, and the labels '0', 'A'.. 'Z' map to 10, 11..
36 for every molecule.
"""
from __future__ import annotations

import io

import numpy as np

# (name, offset, width) of the fields read (hitranapi.py:82-105)
FIELDS = [("id", 0, 2), ("iso", 2, 1), ("v0", 3, 12), ("S_ref", 15, 10), ("A", 25, 10),
          ("g_air", 35, 5), ("g_self", 40, 5), ("El", 45, 10), ("n_air", 55, 4), ("delta", 59, 8),
          ("gp", 146, 7), ("gpp", 153, 7)]
MIN_RECORD = 67
_BLANKS = " \t\v\f"


def _float(fld: str) -> float:
    fld = fld.strip(_BLANKS)
    if not fld:
        return float("nan")
    if "_" in fld or "(" in fld:   # float() takes digit groups; numpy's cast does not
        raise ValueError(fld)
    return float(fld)


def _int(fld: str) -> int:
    fld = fld.strip(_BLANKS)
    if "_" in fld:
        raise ValueError(fld)
    return int(fld)


def _iso(fld: str) -> int:
    fld = fld.strip(_BLANKS)
    if not fld:
        return 1
    if len(fld) == 1:
        c = fld
        if "1" <= c <= "9":
            return ord(c) - ord("0")
        if c == "0":
            return 10
        if "A" <= c.upper() <= "Z":
            return 11 + ord(c.upper()) - ord("A")
    raise ValueError(fld)


def read_hitran160(text: bytes) -> dict:
    """Columns of the records in ``text`` (id/iso int64, the rest float64)."""
    cols = {name: [] for name, _, _ in FIELDS}
    for ln, line in enumerate(io.StringIO(text.decode("ascii"), newline=None), start=1):
        line = line.rstrip("\n")
        if len(line) < MIN_RECORD:
            continue
        for name, off, w in FIELDS:
            fld = line[off:off + w]
            try:
                v = _int(fld) if name == "id" else _iso(fld) if name == "iso" else _float(fld)
            except ValueError:
                raise ValueError(f"line {ln}, field {name}: {fld.strip(_BLANKS)!r} does not convert") from None
            cols[name].append(v)
    return {k: np.asarray(v, dtype=np.int64 if k in ("id", "iso") else np.float64) for k, v in cols.items()}


# Fixed-size records, as the reference reads them: the whole file as one
# structured array of byte fields (160 characters + a 1- or 2-byte line
# return, detected from the first record; tools.py:61-67, 81-108, 153-178),
# each field cast with numpy (tools.py:111-151).  Used as the timed CPU
# baseline of the ingestion path; every record must be complete.
_WIDTHS = [("id", 2), ("iso", 1), ("v0", 12), ("S_ref", 10), ("A", 10), ("g_air", 5), ("g_self", 5),
           ("El", 10), ("n_air", 4), ("delta", 8), ("globu", 15), ("globl", 15), ("locu", 15), ("locl", 15),
           ("ierr", 6), ("iref", 12), ("lmix", 1), ("gp", 7), ("gpp", 7)]


def read_fixed_records(text: bytes) -> dict:
    first = text[:162]
    if first[160:162] == b"\r\n":
        lr = 2
    elif first[160:161] in (b"\n", b"\r"):
        lr = 1
    else:
        raise ValueError("not a file of 160-character records")
    dt = np.dtype([(k, f"S{w}") for k, w in _WIDTHS] + [("_lr", f"S{lr}")])
    if len(text) % dt.itemsize:
        raise ValueError("the file is not a whole number of records")
    rec = np.frombuffer(text, dtype=dt)
    out = {"id": rec["id"].astype(np.int64)}
    iso = rec["iso"]
    code = np.zeros(len(rec), dtype=np.int64)
    for c in np.unique(iso):
        code[iso == c] = _iso(c.decode("ascii"))
    out["iso"] = code
    for k in ("v0", "S_ref", "A", "g_air", "g_self", "El", "n_air", "delta", "gp", "gpp"):
        out[k] = rec[k].astype(np.float64)
    return out
