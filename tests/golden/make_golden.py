"""Generate golden vectors by RUNNING the reference's own code (RADIS 0.17.1).

Run in a container where the reference tree is mounted ($RADIS_REFERENCE_ROOT names the radis project root, or
``--ref``); the GPU tests never run this script, they only read the committed
``golden_ldm.npz``.  The full ``radis`` package cannot be imported here (pandas,
astropy, numba, hapi are absent), so the few reference functions on the LDM
path are pulled out of their source files with ``ast`` and executed unchanged
in a namespace that provides the module-level names they use, with a minimal
stand-in for the factory ``self`` they read attributes from.  Nothing from the
reference is copied into this repository: only its outputs are stored.

Reference code executed (paths relative to the radis project root):
  radis/lbl/broadening.py   doppler_broadening_HWHM, pressure_broadening_HWHM,
                            gaussian_FT, lorentzian_FT, voigt_FT,
                            BroadenFactory._calc_lineshape_LDM,
                            BroadenFactory._get_indices,
                            BroadenFactory._apply_lineshape_LDM
  radis/lbl/base.py         BaseFactory.calc_linestrength_eq, calc_lineshift
  radis/misc/arrays.py      numpy_add_at
  radis/phys/constants.py   (module executed for its constants)
  radis/gpu/params.py, radis/gpu/structs.py (imported by path: numpy/scipy/ctypes only)
Line inputs: radis/test/files/hitran_co_3iso_2000_2300cm.par (reference test
fixture, parsed here with the HITRAN-160 column widths of
radis/api/hitranapi.py:82-105) and seeded synthetic CO-like lines.
"""
from __future__ import annotations

import argparse
import ast
import importlib.util
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_REF = os.environ.get("RADIS_REFERENCE_ROOT")  # the radis project root


def _extract(path, names, cls=None):
    """Return {name: source} for top-level functions (or methods of ``cls``)."""
    src = open(path).read()
    tree = ast.parse(src)
    out = {}
    body = tree.body
    if cls is not None:
        body = [n for n in tree.body if isinstance(n, ast.ClassDef) and n.name == cls][0].body
    for node in body:
        if isinstance(node, ast.FunctionDef) and node.name in names:
            seg = ast.get_source_segment(src, node)
            # methods are indented inside the class: dedent to top level
            lines = seg.splitlines()
            out[node.name] = "\n".join(lines)
    missing = set(names) - set(out)
    if missing:
        raise RuntimeError(f"not found in {path}: {missing}")
    return out


def _load_module_by_path(name, path):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


class _Obj(types.SimpleNamespace):
    pass


class _Profiler:
    def start(self, *a, **k):
        pass

    def stop(self, *a, **k):
        pass


class _Col(np.ndarray):
    """ndarray with a ``.values`` attribute (pandas-Series stand-in)."""

    @property
    def values(self):
        return np.asarray(self)


class _DF:
    """Tiny column store exposing what the executed reference methods touch."""

    def __init__(self, cols, attrs=None):
        self._c = {k: np.asarray(v, dtype=np.float64) for k, v in cols.items()}
        self.attrs = dict(attrs or {})

    @property
    def columns(self):
        return list(self._c)

    def __contains__(self, k):
        return k in self._c

    def __len__(self):
        return len(next(iter(self._c.values())))

    def __getitem__(self, k):
        return self._c[k].view(_Col)

    def __setitem__(self, k, v):
        self._c[k] = np.asarray(v, dtype=np.float64)

    def __getattr__(self, k):
        if k.startswith("_"):
            raise AttributeError(k)
        try:
            return self._c[k].view(_Col)
        except KeyError:
            raise AttributeError(k)

    def sort_values(self, key, kind="mergesort", inplace=True):
        order = np.argsort(self._c[key], kind=kind)
        for k in self._c:
            self._c[k] = self._c[k][order]


def parse_hitran160(path):
    """HITRAN-2004 160-char records (radis/api/hitranapi.py:82-105 widths)."""
    widths = [("id", 2), ("iso", 1), ("wav", 12), ("int", 10), ("A", 10),
              ("airbrd", 5), ("selbrd", 5), ("El", 10), ("Tdpair", 4), ("Pshft", 8)]
    cols = {k: [] for k, _ in widths}
    for line in open(path):
        if len(line.rstrip("\n")) < 67:
            continue
        pos = 0
        for k, w in widths:
            cols[k].append(float(line[pos:pos + w]))
            pos += w
    return {k: np.array(v) for k, v in cols.items()}


def build_reference(ref):
    rp = lambda *p: os.path.join(ref, "radis", *p)
    consts = {}
    exec(compile(open(rp("phys", "constants.py")).read(), "constants.py", "exec"), consts)
    ns = dict(np=np, exp=np.exp, ln=np.log, pi=np.pi, sqrt=np.sqrt, zeros=np.zeros,
              zeros_like=np.zeros_like, arange=np.arange, sin=np.sin)
    for k in ("Na", "c_CGS", "k_b_CGS", "hc_k", "h_CGS"):
        ns[k] = consts[k]
    fns = _extract(rp("lbl", "broadening.py"),
                   ["doppler_broadening_HWHM", "pressure_broadening_HWHM",
                    "gaussian_FT", "lorentzian_FT", "voigt_FT"])
    fns.update(_extract(rp("misc", "arrays.py"), ["numpy_add_at"]))
    for src in fns.values():
        exec(src, ns)
    meths = _extract(rp("lbl", "broadening.py"),
                     ["_calc_lineshape_LDM", "_get_indices", "_apply_lineshape_LDM"],
                     cls="BroadenFactory")
    meths.update(_extract(rp("lbl", "base.py"), ["calc_linestrength_eq", "calc_lineshift"],
                          cls="BaseFactory"))
    import textwrap
    for name, src in meths.items():
        exec(textwrap.dedent(src), ns)
    gpu_structs = _load_module_by_path("ref_gpu_structs", rp("gpu", "structs.py"))
    gpu_params = _load_module_by_path("ref_gpu_params", rp("gpu", "params.py"))
    return ns, consts, gpu_params, gpu_structs


def make_self(ns, wmin, wmax, wstep, dxG, dxL, pressure, Tref=296.0):
    s = _Obj()
    s.profiler = _Profiler()
    s.params = _Obj(dxG=dxG, dxL=dxL, broadening_method="fft", wstep=wstep,
                    folding_thresh=1e-6, sparse_ldm=False)
    s.dataframe_type = "pandas"
    n = int(round((wmax - wmin) / wstep)) + 1
    s.wavenumber_calc = wmin + wstep * np.arange(n)
    s.wavenumber = s.wavenumber_calc
    s.woutrange = (0, n)
    s.misc = _Obj()
    s.verbose = 0
    s.input = _Obj(Tref=Tref, pressure=pressure, isatom=False)
    s.molparam = _Obj(terrestrial_abundances=True)
    s.warn = lambda *a, **k: None
    s._get_indices = types.MethodType(ns["_get_indices"], s)
    return s


def run_case(ns, lines, *, T, p_bar, x, wmin, wmax, wstep, dxG, dxL, M, Qr, Tref=296.0):
    """Run the reference CPU fft-LDM chain on ``lines`` and return its outputs."""
    s = make_self(ns, wmin, wmax, wstep, dxG, dxL, p_bar, Tref)
    df = _DF({"wav": lines["v0"], "int": lines["S_ref"], "El": lines["El"],
              "airbrd": lines["g_air"], "selbrd": lines["g_self"],
              "Tdpair": lines["n_air"], "Pshft": lines["delta"]})
    s.df1 = df
    s.Qref_Qgas_ratio = lambda df1, Tgas, Tref_: Qr
    ns["calc_linestrength_eq"](s, T)
    ns["calc_lineshift"](s)              # sorts df1 by shiftwav (mergesort)
    p_atm = p_bar / 1.01325
    hwhm_l = ns["pressure_broadening_HWHM"](df.airbrd, df.selbrd, df.Tdpair, None, p_atm,
                                            x, T, Tref, {"air": 1 - x}, {})
    hwhm_g = ns["doppler_broadening_HWHM"](df.wav, M, T)
    df["hwhm_lorentz"] = hwhm_l
    df["hwhm_gauss"] = hwhm_g
    prof, wL, wG, wL_dat, wG_dat = ns["_calc_lineshape_LDM"](s, df)
    wav_out, sumoflines = ns["_apply_lineshape_LDM"](s, df.S.values, prof, df.shiftwav.values,
                                                     wL, wG, wL_dat, wG_dat, None)
    NG, NL = len(wG), len(wL)
    prof_arr = np.array([[prof[l][m] for m in range(NL)] for l in range(NG)])
    return dict(v0_sorted=df.wav.values, S=df.S.values, shiftwav=df.shiftwav.values,
                hwhm_l=np.asarray(hwhm_l), hwhm_g=np.asarray(hwhm_g), wL=wL, wG=wG,
                profiles=prof_arr, sumoflines=np.asarray(sumoflines))


def synthetic_co(n, seed, lo=2000.0, hi=2010.0):
    """CO-like synthetic lines (distributions of the 10k-line CO-like list)."""
    rng = np.random.default_rng(seed)
    return dict(v0=np.sort(rng.uniform(lo, hi, n)),
                S_ref=10 ** rng.uniform(-26, -19, n),
                El=np.minimum(rng.exponential(3000.0, n), 20000.0),
                g_air=rng.uniform(0.03, 0.08, n), g_self=rng.uniform(0.05, 0.1, n),
                n_air=rng.uniform(0.5, 0.8, n), delta=rng.uniform(-0.005, 0.0, n))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=DEFAULT_REF, required=DEFAULT_REF is None,
                    help="radis project root (default: $RADIS_REFERENCE_ROOT)")
    ap.add_argument("--out", default=os.path.join(HERE, "golden_ldm.npz"))
    a = ap.parse_args()
    ns, consts, gpu_params, gpu_structs = build_reference(a.ref)
    fx = parse_hitran160(os.path.join(a.ref, "radis", "test", "files",
                                      "hitran_co_3iso_2000_2300cm.par"))
    iso1 = fx["iso"] == 1
    hit = dict(v0=fx["wav"][iso1], S_ref=fx["int"][iso1], El=fx["El"][iso1],
               g_air=fx["airbrd"][iso1], g_self=fx["selbrd"][iso1],
               n_air=fx["Tdpair"][iso1], delta=fx["Pshft"][iso1])
    dxL = np.log((0.01 / 0.20) ** 0.5 + 1)   # loader.py:452-460,538-543 defaults
    dxG = np.log((0.01 / 0.46) ** 0.5 + 1)
    cases = {
        # name: (lines, T, p_bar, x, wmin, wmax, wstep, M, Qr)
        "hitran_co_700K": (hit, 700.0, 1.01325, 0.1, 2050.0, 2150.0, 0.01, 28.0, 0.37),
        "hitran_co_3000K": (hit, 3000.0, 1.0, 0.5, 2100.0, 2200.0, 0.02, 28.0, 0.083),
        # low pressure + coarse step: Gaussian width ~ wstep, folding terms active
        "synth_fold": (synthetic_co(400, 11), 1500.0, 0.01, 0.3, 2000.0, 2010.0, 0.02,
                       28.0, 0.2),
        "synth_1atm": (synthetic_co(300, 12), 296.0, 1.01325, 0.05, 2000.0, 2010.0, 0.005,
                       28.0, 1.0),
        # high pressure: Lorentzian-dominated profiles, shifts of ~0.02 cm-1
        "hitran_co_10bar": (hit, 1000.0, 10.0, 0.5, 2050.0, 2150.0, 0.01, 28.0, 0.2),
        # pure self-broadening (x = 1: no air term) on a fine step, hot
        "synth_self_hot": (synthetic_co(500, 14), 2500.0, 1.01325, 1.0, 2000.0, 2010.0, 0.002,
                           28.0, 0.05),
    }
    out = {}
    for name, (lines, T, p, x, wmin, wmax, wstep, M, Qr) in cases.items():
        # the CPU path clamps out-of-window lines onto the edge bins (np.interp,
        # broadening.py:2151-2154) while the GPU path drops them; the factory only
        # hands it lines inside the calculation window, so keep those
        sel = (lines["v0"] > wmin + 0.5) & (lines["v0"] < wmax - 0.5)
        lines = {k: np.asarray(v)[sel] for k, v in lines.items()}
        r = run_case(ns, lines, T=T, p_bar=p, x=x, wmin=wmin, wmax=wmax, wstep=wstep,
                     dxG=dxG, dxL=dxL, M=M, Qr=Qr)
        for k, v in lines.items():
            out[f"{name}/in_{k}"] = np.asarray(v)
        for k, v in dict(T=T, p_bar=p, x=x, wmin=wmin, wmax=wmax, wstep=wstep, M=M, Qr=Qr,
                         dxG=dxG, dxL=dxL).items():
            out[f"{name}/cond_{k}"] = np.float64(v)
        for k, v in r.items():
            if k == "profiles" and v.size > 200_000:
                # keep the fixture small: every 41st rfft bin of each node profile
                out[f"{name}/out_profiles_stride41"] = v[:, :, ::41]
                continue
            out[f"{name}/out_{k}"] = v
        print(name, "lines", len(lines["v0"]), "NG", len(r["wG"]), "NL", len(r["wL"]),
              "peak", r["sumoflines"].max())

    # --- reference GPU grid-parameter rule (radis/gpu/params.py) ---------------
    rng = np.random.default_rng(5)
    grid_rows = []
    for gi, lines in enumerate((hit, synthetic_co(2000, 13, 1900.0, 2300.0))):
        na = np.asarray(lines["n_air"], np.float32)
        gamma_arr = np.stack([np.asarray(lines["g_self"], np.float32),
                              np.asarray(lines["g_air"], np.float32)])
        Mm_arr = np.array([0.0, 28.0])
        kc, cc, NA_ = gpu_params.k, gpu_params.c, 6.02214076e23
        log_c2Mm = np.array([0.0] + [0.5 * np.log(8 * kc * np.log(2) / (cc ** 2 * m * 1e-3 / NA_))
                                     for m in Mm_arr[1:]])
        iso = np.ones(len(lines["v0"]), dtype=np.int64)
        log_2vMm = np.log(lines["v0"]) + log_c2Mm.take(iso)
        gpu_params.init_G_params(log_2vMm.astype(np.float32))
        gpu_params.init_L_params(na, gamma_arr)
        gpu_params.init_Q([lambda T: 1.0, lambda T: 1.0])
        for T in (300.0, 700.0, 1500.0, 3000.0, 250.0):
            for p in (0.1, 1.0, 5.0):
                init_h = gpu_structs.initData_t()
                iter_h = gpu_structs.iterData_t()
                init_h.dxG = dxG
                init_h.dxL = dxL
                gpu_params.set_pTQ(p, T, 0.1, iter_h)
                gpu_params.set_G_params(init_h, iter_h)
                gpu_params.set_L_params(init_h, iter_h)
                grid_rows.append([gi, T, p, iter_h.log_wG_min, iter_h.N_G,
                                  iter_h.log_wL_min, iter_h.N_L])
        out[f"grid{gi}/in_v0"] = np.asarray(lines["v0"])
        out[f"grid{gi}/in_n_air"] = na
        out[f"grid{gi}/in_g_self"] = gamma_arr[0]
        out[f"grid{gi}/in_g_air"] = gamma_arr[1]
    out["grid/rows"] = np.array(grid_rows)
    out["grid/dxG"] = np.float64(dxG)
    out["grid/dxL"] = np.float64(dxL)
    np.savez_compressed(a.out, **out)
    print("wrote", a.out, os.path.getsize(a.out), "bytes")


if __name__ == "__main__":
    main()
