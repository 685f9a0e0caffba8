"""Generate slit golden vectors by RUNNING the reference's own code (RADIS 0.17.1).

Run in a container where the reference tree is mounted ($RADIS_REFERENCE_ROOT names the radis project root, or
``--ref``); the tests only read the committed ``golden_slit.npz``.  The
``radis`` package cannot be imported here (pandas, astropy, numba, hapi are
absent), so the slit functions are pulled out of their source file with
``ast`` and executed unchanged in a namespace that provides the module-level
names they use.  Only their outputs are stored in this repository.

Reference code executed (paths relative to the radis project root):
  radis/tools/slit.py    triangular_slit, trapezoidal_slit, gaussian_slit,
                         normalize_slit, remove_boundary, get_FWHM,
                         convolve_with_slit
  radis/misc/arrays.py   evenly_distributed, evenly_distributed_fast, anynan
Spectra: seeded synthetic transmittance-like arrays on even grids.
"""
from __future__ import annotations

import argparse
import ast
import os
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_REF = os.environ.get("RADIS_REFERENCE_ROOT")  # the radis project root


def _extract(path, names):
    src = open(path).read()
    tree = ast.parse(src)
    out = {}
    for node in tree.body:
        if isinstance(node, ast.FunctionDef) and node.name in names:
            out[node.name] = ast.get_source_segment(src, node)
    missing = set(names) - set(out)
    if missing:
        raise RuntimeError(f"not found in {path}: {missing}")
    return out


def reference_namespace(ref):
    ns = {"np": np, "exp": np.exp, "ln": np.log, "sqrt": np.sqrt, "warn": warnings.warn,
          "plot_slit": lambda *a, **k: None}

    def _no_resample(*a, **k):
        raise RuntimeError("resampling is not exercised")

    ns["resample_even"] = _no_resample
    arrays = _extract(os.path.join(ref, "radis/misc/arrays.py"),
                      ["evenly_distributed", "evenly_distributed_fast", "anynan"])
    slit = _extract(os.path.join(ref, "radis/tools/slit.py"),
                    ["triangular_slit", "trapezoidal_slit", "gaussian_slit", "normalize_slit",
                     "remove_boundary", "get_FWHM", "convolve_with_slit"])
    for src in list(arrays.values()) + list(slit.values()):
        exec(compile(src, "<reference>", "exec"), ns)
    return ns


def spectrum(n, w0, wstep, seed):
    """Seeded transmittance-like spectrum: exp(-sum of Lorentzian lines)."""
    rng = np.random.default_rng(seed)
    w = w0 + wstep * np.arange(n)
    k = np.zeros(n)
    for c, s, g in zip(rng.uniform(w[0], w[-1], 60), rng.uniform(0.1, 3.0, 60), rng.uniform(0.01, 0.2, 60)):
        k += s * g / np.pi / ((w - c) ** 2 + g * g)
    return w, np.exp(-k)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=DEFAULT_REF, required=DEFAULT_REF is None,
                    help="radis project root (default: $RADIS_REFERENCE_ROOT)")
    ap.add_argument("--out", default=os.path.join(HERE, "golden_slit.npz"))
    args = ap.parse_args()
    R = reference_namespace(args.ref)
    out = {}
    # slit generators (FWHM / base in the same unit as wstep)
    tri = [(0.5, 0.01, "area", 0.0, 1.0), (0.1, 0.001, "area", 0.0, 1.0), (0.35, 0.002, "area", 2000.0, 1.0),
           (1.0, 0.001, "max", 0.0, 2.5), (0.07, 0.01, "area", 0.0, 1.0)]
    for i, (fwhm, ws, nb, c, sc) in enumerate(tri):
        w, I = R["triangular_slit"](fwhm, ws, center=c, norm_by=nb, scale=sc)
        out[f"tri{i}_args"] = np.array([fwhm, ws, c, sc, 1.0 if nb == "area" else 0.0])
        out[f"tri{i}_w"], out[f"tri{i}_I"] = w, I
    trap = [(0.2, 0.6, 0.01, "area"), (0.05, 0.15, 0.001, "area"), (0.31, 0.3, 0.002, "area"),
            (0.1, 0.5, 0.01, "max")]
    for i, (top, base, ws, nb) in enumerate(trap):
        w, I = R["trapezoidal_slit"](top, base, ws, norm_by=nb)
        out[f"trap{i}_args"] = np.array([top, base, ws, 1.0 if nb == "area" else 0.0])
        out[f"trap{i}_w"], out[f"trap{i}_I"] = w, I
    gau = [(0.5, 0.01, 4), (0.1, 0.001, 4), (0.3, 0.002, 3), (0.25, 0.01, 4)]
    for i, (fwhm, ws, cr) in enumerate(gau):
        w, I = R["gaussian_slit"](fwhm, ws, calc_range=cr)
        out[f"gau{i}_args"] = np.array([fwhm, ws, cr])
        out[f"gau{i}_w"], out[f"gau{i}_I"] = w, I
    # convolution: on-grid slits (valid and same) and a slit sampled on a
    # different step (spline interpolation, k = 1 and k = 3)
    w, I = spectrum(4001, 2000.0, 0.01, seed=11)
    out["spec_w"], out["spec_I"] = w, I
    cases = [("tri", R["triangular_slit"](0.5, 0.01), "valid", 1),
             ("trisame", R["triangular_slit"](0.5, 0.01), "same", 1),
             ("trap", R["trapezoidal_slit"](0.2, 0.6, 0.01), "valid", 1),
             ("gau", R["gaussian_slit"](0.3, 0.01), "valid", 1),
             ("fine1", R["gaussian_slit"](0.3, 0.004), "valid", 1),
             ("fine3", R["triangular_slit"](0.4, 0.004), "valid", 3)]
    for name, (ws, Is), mode, k in cases:
        wc, Ic = R["convolve_with_slit"](w, I, ws, Is, mode=mode, k=k, verbose=False)
        out[f"conv_{name}_slit_w"], out[f"conv_{name}_slit_I"] = ws, Is
        out[f"conv_{name}_mode"] = np.array([0 if mode == "same" else 1, k])
        out[f"conv_{name}_I"] = Ic
    np.savez_compressed(args.out, **out)
    print("wrote", args.out, len(out), "arrays")


if __name__ == "__main__":
    main()
