"""HITRAN-2004 160-character line records: native reader, columnar cache, writer.

Column widths follow radis/api/hitranapi.py:82-105 (id a2, iso a1, wav a12,
int a10, A a10, airbrd a5, selbrd a5, El a10, Tdpair a4, Pshft a8, then the
quantum-number/reference fields, gp a7, gpp a7).  Records are parsed by the
library's multi-threaded C++ parser (``rg_hitran_parse``); the columns the
equilibrium synthesis needs come back under the names the rest of this
package uses (v0, S_ref, A, g_air, g_self, El, n_air, delta, id, iso, gp,
gpp); iso is the HITRAN isotopologue number (1-based; HITEMP's '0', 'A', 'B'
labels read as 10, 11, 12).

``load_hitran`` adds the reference's cache behaviour (hit2df,
radis/api/hitranapi.py:182-380, with load_h5_cache_file,
radis/api/cache_files.py:58-196): the parsed columns are written next to the
file (or into ``cache_directory_path``) on first access and memory-mapped on
later ones.  The cache is a flat columnar file: an 8-byte magic, an 8-byte
header length, a JSON header (format version, the source file's size and
modification time, the line count, wavenumber range and column table) and
the raw little-endian columns at 64-byte aligned offsets.
"""
from __future__ import annotations

import json
import mmap
import os
import threading
import warnings

import numpy as np

from . import _lib

# (name, width) in record order; None = field skipped by the reader
_FIELDS = [("id", 2), ("iso", 1), ("v0", 12), ("S_ref", 10), ("A", 10), ("g_air", 5),
           ("g_self", 5), ("El", 10), ("n_air", 4), ("delta", 8), (None, 15), (None, 15),
           (None, 15), (None, 15), (None, 6), (None, 12), (None, 1), ("gp", 7), ("gpp", 7)]
RECORD = sum(w for _, w in _FIELDS)   # 160

CACHE_MAGIC = b"RGHITC01"
CACHE_VERSION = 1
CACHE_SUFFIX = ".rgcache"


class DeprecatedFileWarning(UserWarning):
    """A cache file that does not match its source (radis/misc/warning.py)."""


class IrrelevantFileWarning(UserWarning):
    """A cache file whose lines lie outside the requested range; raised, as by
    the reference's load_h5_cache_file, so that callers skip the file."""


def read_hitran160(path, threads: int = 0) -> dict:
    """Parse a .par file into numpy columns (float64; id/iso int64) with the
    library's parser over a read-only memory map of the file; threads <= 0:
    one per host core."""
    if os.path.getsize(path) == 0:
        return _lib.hitran_parse(np.zeros(0, dtype=np.uint8), threads=threads)
    with open(path, "rb") as f, mmap.mmap(f.fileno(), 0, access=mmap.ACCESS_READ) as m:
        buf = np.frombuffer(m, dtype=np.uint8)
        try:
            return _lib.hitran_parse(buf, threads=threads)
        finally:
            del buf   # the map closes only once no view of it is left


def cache_file(path, cache_directory_path=None):
    """Cache file of a .par file: <dir>/<name>.rgcache, dir = the file's own
    directory unless ``cache_directory_path`` is given (hitranapi.py:283-291)."""
    d = cache_directory_path or os.path.dirname(os.path.abspath(path))
    return os.path.join(d, os.path.basename(path) + CACHE_SUFFIX)


def _source_meta(path):
    st = os.stat(path)
    return {"source_size": int(st.st_size), "source_mtime_ns": int(st.st_mtime_ns)}


def write_cache(fcache, cols: dict, meta: dict):
    """Write columns and metadata (atomically: a temporary file renamed)."""
    n = len(next(iter(cols.values()))) if cols else 0
    table, off = [], 0
    for k, a in cols.items():
        a = np.ascontiguousarray(a)
        table.append({"name": k, "dtype": a.dtype.newbyteorder("<").str, "offset": off, "count": int(a.size)})
        off += (a.nbytes + 63) // 64 * 64
    v0 = cols.get("v0")
    header = dict(meta, version=CACHE_VERSION, n=int(n), columns=table,
                  wavenum_min=float(np.min(v0)) if v0 is not None and n else None,
                  wavenum_max=float(np.max(v0)) if v0 is not None and n else None)
    hb = json.dumps(header).encode()
    data0 = (16 + len(hb) + 63) // 64 * 64
    tmp = fcache + f".tmp{os.getpid()}.{threading.get_ident()}"
    with open(tmp, "wb") as f:
        f.write(CACHE_MAGIC + len(hb).to_bytes(8, "little") + hb)
        for t, a in zip(table, cols.values()):
            f.seek(data0 + t["offset"])
            f.write(np.ascontiguousarray(a, dtype=np.dtype(t["dtype"])).tobytes())
        f.truncate(data0 + off)
    os.replace(tmp, fcache)
    return header


def read_cache_header(fcache) -> dict:
    with open(fcache, "rb") as f:
        head = f.read(16)
        if len(head) != 16 or head[:8] != CACHE_MAGIC:
            raise DeprecatedFileWarning(f"{fcache} is not a line cache file of this format")
        hb = f.read(int.from_bytes(head[8:], "little"))
    h = json.loads(hb)
    h["_data0"] = (16 + len(hb) + 63) // 64 * 64
    return h


def read_cache(fcache, columns=None) -> dict:
    """Memory-mapped read-only columns of a cache file."""
    h = read_cache_header(fcache)
    out = {}
    for t in h["columns"]:
        if columns is not None and t["name"] not in columns:
            continue
        dt = np.dtype(t["dtype"])
        if t["count"] == 0:
            out[t["name"]] = np.zeros(0, dtype=dt)
        else:
            out[t["name"]] = np.memmap(fcache, dtype=dt, mode="r", offset=h["_data0"] + t["offset"],
                                       shape=(t["count"],))
    return out


def load_hitran(path, cache=True, load_wavenum_min=None, load_wavenum_max=None, cache_directory_path=None,
                threads: int = 0, columns=None, verbose=False) -> dict:
    """HITRAN-160 file -> columns, through the columnar cache.

    ``cache`` as in hit2df / load_h5_cache_file (cache_files.py:76-85): False
    parses the file; True uses the cache file, generating it when absent and
    regenerating it when it no longer matches its source (size, modification
    time or format version); 'regen' deletes it first; 'force' requires a valid
    cache file (ValueError when absent, DeprecatedFileWarning raised when it
    does not match).  With an existing cache, ``load_wavenum_min`` /
    ``load_wavenum_max`` raise IrrelevantFileWarning when the cached lines lie
    entirely outside [min, max] (cache_files.py:157-174), without reading the
    columns.  A cache that cannot be written (read-only directory) is skipped
    with a warning."""
    if cache not in (True, False, "regen", "force"):
        raise ValueError(f"cache must be True, False, 'regen' or 'force', not {cache!r}")
    if load_wavenum_min is not None and load_wavenum_max is not None and not load_wavenum_min < load_wavenum_max:
        raise ValueError("load_wavenum_min must be below load_wavenum_max")
    if not cache:
        return read_hitran160(path, threads=threads) if columns is None else \
            _select(read_hitran160(path, threads=threads), columns)
    fcache = cache_file(path, cache_directory_path)
    if cache == "regen" and os.path.exists(fcache):
        os.remove(fcache)
        if verbose:
            print(f"Deleted cache file: {fcache}")
    if os.path.exists(fcache):
        try:
            h = read_cache_header(fcache)
            src = _source_meta(path)
            if h.get("version") != CACHE_VERSION or any(h.get(k) != v for k, v in src.items()):
                raise DeprecatedFileWarning(f"{fcache} does not match {path} (size, modification time or version)")
        except (DeprecatedFileWarning, ValueError, OSError) as err:
            if cache == "force":
                raise
            if verbose:
                print(f"{err}: deleting {fcache}")
            os.remove(fcache)
        else:
            lo, hi = h.get("wavenum_min"), h.get("wavenum_max")
            if lo is not None and ((load_wavenum_min is not None and hi < load_wavenum_min) or
                                   (load_wavenum_max is not None and lo > load_wavenum_max)):
                raise IrrelevantFileWarning(f"{fcache}: lines in [{lo}, {hi}] cm-1, outside the requested range")
            return read_cache(fcache, columns)
    elif cache == "force":
        raise ValueError(f"Cache file {fcache} doesnt exist")
    meta = _source_meta(path)
    cols = read_hitran160(path, threads=threads)
    try:
        write_cache(fcache, cols, meta)
        if verbose:
            print(f"Generated cache file {fcache}")
    except OSError as err:
        warnings.warn(f"cache file {fcache} not written: {err}")
    return cols if columns is None else _select(cols, columns)


def _select(cols, columns):
    return {k: v for k, v in cols.items() if k in columns}


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


def _iso_char(i: int) -> str:
    """HITRAN isotopologue label: 1-9, '0' for 10, 'A', 'B', ... from 11."""
    if 1 <= i <= 9:
        return str(i)
    if i == 10:
        return "0"
    if 11 <= i <= 36:
        return chr(ord("A") + i - 11)
    raise ValueError(f"isotopologue {i} has no HITRAN label")


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
            rec = (f"{mol_id:2d}{_iso_char(int(iso[i]))}{lines['v0'][i]:12.6f}"
                   f"{_fmt_e(lines['S_ref'][i], 10, 3)}{_fmt_e(A[i], 10, 3)}"
                   f"{_fmt_w(lines['g_air'][i])}{_fmt_w(lines['g_self'][i])}"
                   f"{lines['El'][i]:10.4f}{lines['n_air'][i]:4.2f}{_fmt_shift(delta[i])}"
                   f"{blank}{gp[i]:7.1f}{gpp[i]:7.1f}")
            if len(rec) != RECORD:
                raise ValueError(f"record {i} has {len(rec)} characters")
            f.write(rec + "\n")
