"""HITRAN-160 ingestion on the CPU: the library's parser (rg_hitran_parse,
radis_gb300.hitran) and the oracle against the reference's own parse of the
committed synthetic fixtures (tests/golden/make_golden_hitran.py: two
HITRAN-160 files, and a CDSD-HITEMP CO2 file whose first ten columns are the
HITRAN ones), the parser
against the oracle on edge cases and across thread-chunk boundaries, and the
columnar cache (hit2df / load_h5_cache_file rules: cache True, False,
'regen', 'force'; deprecation by source size / modification time; relevance
by wavenumber range).  Integer and float columns are compared bit for bit."""
import os
import time

import numpy as np
import pytest

from oracle import hitran_oracle as HO
from radis_gb300 import _lib as L
from radis_gb300 import hitran as H

HERE = os.path.dirname(__file__)
G = np.load(os.path.join(HERE, "golden", "golden_hitran.npz"))
FIXTURES = ("hitran_co_lf", "hitran_co2_crlf", "hitemp_co2_cdsd")


def _golden(tag):
    """The reference's parse of a fixture: every HITRAN column, or for the
    127-character CDSD-HITEMP records the ten it shares with HITRAN-160."""
    return {k.split("__")[1]: G[k] for k in G.files if k.startswith(tag + "__")}


def _check_fixture(tag, got):
    want = _golden(tag)
    _assert_cols({k: got[k] for k in want}, want)
    if tag.startswith("hitemp"):   # no gp/gpp in CDSD records: the fields lie past their end
        assert np.isnan(got["gp"]).all() and np.isnan(got["gpp"]).all()


def _same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if a.dtype != b.dtype or a.shape != b.shape:
        return False
    if a.dtype == np.float64:
        return np.array_equal(a.view(np.int64), b.view(np.int64))
    return np.array_equal(a, b)


def _assert_cols(got, want):
    assert set(got) == set(want)
    for k in want:
        assert _same(got[k], want[k]), k


@pytest.mark.parametrize("tag", FIXTURES)
def test_oracle_matches_reference(tag):
    _check_fixture(tag, HO.read_hitran160(open(os.path.join(HERE, "golden", tag + ".par"), "rb").read()))


@pytest.mark.parametrize("tag", FIXTURES[:2])
def test_fixed_record_oracle_matches_reference(tag):
    """The numpy fixed-record restatement timed as the CPU baseline."""
    o = HO.read_fixed_records(open(os.path.join(HERE, "golden", tag + ".par"), "rb").read())
    _assert_cols(o, {k: G[f"{tag}__{k}"] for k in o})


@pytest.mark.parametrize("tag", FIXTURES)
@pytest.mark.parametrize("threads", [1, 4])
def test_native_matches_reference(native_lib, tag, threads):
    _check_fixture(tag, H.read_hitran160(os.path.join(HERE, "golden", tag + ".par"), threads=threads))


WIDTHS = {"id": 2, "iso": 1, "v0": 12, "S": 10, "A": 10, "ga": 5, "gs": 5, "El": 10, "na": 4, "d": 8}


def _rec(v0="2000.123456", s=" 1.234E-20", iso="1", tail=True, **kw):
    """One record; every field right-aligned in its width."""
    f = {"id": "5", "iso": iso, "v0": v0, "S": s, "A": "1.000E+00", "ga": ".0600", "gs": ".0800",
         "El": "100.0000", "na": "0.70", "d": "-.002000"}
    f.update(kw)
    for k, w in WIDTHS.items():
        assert len(f[k]) <= w, (k, f[k])
    r = "".join(f[k].rjust(w) for k, w in WIDTHS.items())
    if tail:
        r += " " * 79 + "   12.0" + "   10.0"
    return r


EDGE_TEXTS = {
    "empty": b"",
    "newlines only": b"\n\r\n\r\n\n",
    "no final newline": (_rec() + "\n" + _rec(v0="2001.5")).encode(),
    "crlf and lone cr": (_rec() + "\r\n" + _rec(v0="2002") + "\r" + _rec(v0="2003") + "\r\r\n").encode(),
    "short lines skipped": ("short\n" + _rec() + "\n" + "x" * 66 + "\n" + _rec(v0="2004") + "\n").encode(),
    "record without quanta tail": (_rec(tail=False) + "\n" + _rec(tail=False)[:100] + "\n").encode(),
    "blank fields are NaN": _rec(s="", A="          ", d="        ").encode() + b"\n",
    "signs, inf, nan": (_rec(v0="+2000.5", s="+1.000E+10") + "\n" + _rec(s="       inf", A="      -NaN") +
                        "\n" + _rec(s=" -infinity") + "\n").encode(),
    "out of range exponents": (_rec(s=" 1.00E+999", A=" 1.00E-999") + "\n" +
                               _rec(s="-9.99E+400", A="-1.00E-400") + "\n").encode(),
    "subnormal": _rec(s=" 4.94E-324", A=" 2.47E-324").encode() + b"\n",
    "isotopologue labels": "\n".join(_rec(iso=c) for c in "1290ABab Z").encode(),
    "tabs around fields": _rec(s="\t1.5E-20\t ", v0="\t2000.25\t").encode() + b"\n",
}


@pytest.mark.parametrize("name", sorted(EDGE_TEXTS))
def test_native_matches_oracle_edge_cases(native_lib, name):
    text = EDGE_TEXTS[name]
    _assert_cols(L.hitran_parse(np.frombuffer(text, dtype=np.uint8)), HO.read_hitran160(text))


BAD = {
    "letters in a number": (_rec(v0="2000.12x456"), 1, "wav"),
    "two signs": (_rec(s="+-1.0E-20"), 1, "int"),
    "digit groups": (_rec(A="1_000.0"), 1, "A"),
    "nan payload": (_rec(A="nan(7)"), 1, "A"),
    "blank id": (_rec(id="  "), 1, "id"),
    "label that is not an isotopologue": (_rec(iso="#"), 1, "iso"),
}


@pytest.mark.parametrize("name", sorted(BAD))
def test_bad_field_reports_line_and_field(native_lib, name):
    rec, _, field = BAD[name]
    text = (_rec() + "\n" + "short\n" + rec + "\n").encode()
    with pytest.raises(L.RgError, match=f"line 3, field {field}:"):
        L.hitran_parse(np.frombuffer(text, dtype=np.uint8))
    with pytest.raises(ValueError, match="line 3"):
        HO.read_hitran160(text)


def _big_text(n, seed):
    """n records with random line ends (LF / CRLF / CR) and short lines."""
    rng = np.random.default_rng(seed)
    v0 = np.sort(rng.uniform(500, 8000, n))
    s = 10 ** rng.uniform(-30, -18, n)
    ends = rng.choice([b"\n", b"\r\n", b"\r"], n)
    out = []
    for i in range(n):
        out.append(_rec(v0=f"{v0[i]:12.6f}", s=f"{s[i]:10.3E}", iso="123"[i % 3]).encode() + ends[i])
        if i % 997 == 0:
            out.append(b"# comment" + ends[i])
    return b"".join(out)


def test_thread_chunks_match_single_thread(native_lib):
    text = _big_text(30000, 5)   # ~4.9 MB: up to 5 chunks at 1 MB per thread
    buf = np.frombuffer(text, dtype=np.uint8)
    one = L.hitran_parse(buf, threads=1)
    for t in (2, 3, 4, 16):
        _assert_cols(L.hitran_parse(buf, threads=t), one)
    _assert_cols(one, HO.read_hitran160(text))


def test_column_subset(native_lib):
    text = EDGE_TEXTS["crlf and lone cr"]
    sub = L.hitran_parse(np.frombuffer(text, dtype=np.uint8), columns=("v0", "iso"))
    assert set(sub) == {"v0", "iso"}
    _assert_cols(sub, {k: HO.read_hitran160(text)[k] for k in sub})


def _par(tmp_path, n=400, seed=1, name="lines.par"):
    rng = np.random.default_rng(seed)
    lines = {"v0": np.sort(rng.uniform(2000, 2300, n)), "S_ref": 10 ** rng.uniform(-26, -19, n),
             "g_air": rng.uniform(0.03, 0.08, n), "g_self": rng.uniform(0.05, 0.1, n),
             "El": rng.uniform(0, 5000, n), "n_air": rng.uniform(0.5, 0.8, n),
             "delta": rng.uniform(-0.005, 0.0, n), "iso": rng.integers(1, 4, n)}
    p = tmp_path / name
    H.write_hitran160(p, lines)
    return str(p)


def test_cache_generate_then_memory_map(native_lib, tmp_path):
    p = _par(tmp_path)
    fc = H.cache_file(p)
    assert not os.path.exists(fc)
    first = H.load_hitran(p)
    assert os.path.exists(fc)
    second = H.load_hitran(p)
    assert all(isinstance(v, np.memmap) for v in second.values())
    _assert_cols({k: np.asarray(v) for k, v in second.items()}, first)
    _assert_cols(first, H.read_hitran160(p))
    h = H.read_cache_header(fc)
    assert h["n"] == 400 and h["wavenum_min"] == float(first["v0"].min())
    assert all(t["offset"] % 64 == 0 for t in h["columns"]) and h["_data0"] % 64 == 0


def test_cache_false_writes_nothing(native_lib, tmp_path):
    p = _par(tmp_path)
    _assert_cols(H.load_hitran(p, cache=False), H.read_hitran160(p))
    assert not os.path.exists(H.cache_file(p))


def test_cache_regenerated_when_source_changes(native_lib, tmp_path):
    p = _par(tmp_path, seed=1)
    H.load_hitran(p)
    st = os.stat(p)
    _par(tmp_path, seed=2)                                       # new content, same size
    os.utime(p, ns=(st.st_atime_ns, st.st_mtime_ns + 10**9))     # and a later time
    with pytest.raises(H.DeprecatedFileWarning):
        H.load_hitran(p, cache="force")
    got = H.load_hitran(p)
    _assert_cols({k: np.asarray(v) for k, v in got.items()}, H.read_hitran160(p))
    assert H.read_cache_header(H.cache_file(p))["source_mtime_ns"] == os.stat(p).st_mtime_ns


def test_cache_regen_and_force(native_lib, tmp_path):
    p = _par(tmp_path)
    with pytest.raises(ValueError, match="doesnt exist"):
        H.load_hitran(p, cache="force")
    H.load_hitran(p)
    t0 = os.stat(H.cache_file(p)).st_mtime_ns
    time.sleep(0.01)
    H.load_hitran(p, cache="regen")
    assert os.stat(H.cache_file(p)).st_mtime_ns != t0
    assert isinstance(H.load_hitran(p, cache="force")["v0"], np.memmap)
    with pytest.raises(ValueError):
        H.load_hitran(p, cache="sometimes")


def test_cache_corrupt_file(native_lib, tmp_path):
    p = _par(tmp_path)
    with open(H.cache_file(p), "wb") as f:
        f.write(b"not a cache file at all")
    with pytest.raises(H.DeprecatedFileWarning):
        H.load_hitran(p, cache="force")
    _assert_cols(H.load_hitran(p), H.read_hitran160(p))


def test_cache_relevance(native_lib, tmp_path):
    p = _par(tmp_path)   # lines in [2000, 2300]
    H.load_hitran(p)
    with pytest.raises(H.IrrelevantFileWarning):
        H.load_hitran(p, load_wavenum_min=2400, load_wavenum_max=2500)
    with pytest.raises(H.IrrelevantFileWarning):
        H.load_hitran(p, load_wavenum_max=1900)
    assert len(H.load_hitran(p, load_wavenum_min=2200, load_wavenum_max=2500)["v0"]) == 400


def test_cache_directory(native_lib, tmp_path):
    d = tmp_path / "cache"
    d.mkdir()
    p = _par(tmp_path)
    H.load_hitran(p, cache_directory_path=str(d))
    assert os.path.exists(os.path.join(str(d), "lines.par" + H.CACHE_SUFFIX))
    assert not os.path.exists(H.cache_file(p))


def test_factory_load_databank_uses_cache(native_lib, tmp_path):
    from radis_gb300 import SpectrumFactory
    p = _par(tmp_path)
    sf = SpectrumFactory(wavenum_min=2050, wavenum_max=2250, wstep=0.01, molecule="CO", isotope="1,2")
    sf.load_databank(p)
    assert os.path.exists(H.cache_file(p))
    ref = HO.read_hitran160(open(p, "rb").read())
    keep = np.isin(ref["iso"], [1, 2])
    lo = sf.params.wavenum_min_calc - sf.params.neighbour_lines
    hi = sf.wavenumber_calc[-1] + sf.params.neighbour_lines
    keep &= (ref["v0"] >= lo) & (ref["v0"] <= hi)
    for k in ("v0", "S_ref", "El", "iso"):
        assert _same(np.asarray(sf.df0[k]), ref[k][keep]), k
    sf2 = SpectrumFactory(wavenum_min=2050, wavenum_max=2250, wstep=0.01, molecule="CO")
    sf2.load_databank(p, db_use_cached=False)
    assert len(sf2.df0["v0"]) == int(((ref["v0"] >= lo) & (ref["v0"] <= hi)).sum())


def _decimal_strings(n, seed):
    """Decimal fields of at most 12 characters on both sides of the exact fast
    path's limits (15 significant digits, |power of ten| <= 22)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        kind = rng.integers(0, 6)
        if kind == 0:     # fixed point, 1-11 digits
            d = int(rng.integers(1, 12))
            f = int(rng.integers(0, d + 1))
            s = "".join(str(x) for x in rng.integers(0, 10, d))
            s = s[:d - f] + "." + s[d - f:] if f else s
        elif kind == 1:   # leading / trailing zeros
            s = "0" * int(rng.integers(0, 4)) + "." + "0" * int(rng.integers(0, 5)) + str(rng.integers(1, 10 ** 5))
        elif kind == 2:   # mantissa + exponent near the fast path's limits
            s = f"{rng.integers(1, 10**6)}E{rng.integers(-30, 31):+d}"
        elif kind == 3:   # HITRAN intensity style
            s = f"{rng.uniform(1, 10):.3f}E{rng.integers(-40, 5):+03d}"
        elif kind == 4:   # 14-17 significant digits (around the 15-digit limit)
            s = str(rng.integers(10 ** 13, 10 ** 16))[: int(rng.integers(10, 12))]
            s = s[:3] + "." + s[3:]
        else:             # exponent without a sign, lower case
            s = f"{rng.integers(1, 999)}.{rng.integers(0, 99)}e{rng.integers(0, 25)}"
        if rng.integers(0, 3) == 0:
            s = ("-" if rng.integers(0, 2) else "+") + s
        out.append(s[:12])
    return out


def test_decimal_conversion_matches_float(native_lib):
    """Every field value equals Python's float() of its text, bit for bit, on
    both sides of the exact fast path's limits."""
    vals = _decimal_strings(20000, 9)
    text = "".join(_rec(v0=v) + "\n" for v in vals).encode()
    got = L.hitran_parse(np.frombuffer(text, dtype=np.uint8), columns=("v0",))["v0"]
    want = np.array([float(v) for v in vals])
    assert _same(got, want)
