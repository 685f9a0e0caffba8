"""Generate air-wavelength golden vectors by RUNNING the reference's own
functions (RADIS 0.17.1): air_index_dispersion, vacuum2air and air2vacuum of
radis/phys/air.py:16-119, pulled out of the source with ``ast`` and executed
unchanged.  Run where the reference tree is mounted ($RADIS_REFERENCE_ROOT names the radis project root, or
``--ref``); the tests only read the committed ``golden_units.npz``."""
from __future__ import annotations

import argparse
import ast
import os
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_REF = os.environ.get("RADIS_REFERENCE_ROOT")  # the radis project root


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=DEFAULT_REF, required=DEFAULT_REF is None,
                    help="radis project root (default: $RADIS_REFERENCE_ROOT)")
    args = ap.parse_args()
    src = open(os.path.join(args.ref, "radis", "phys", "air.py")).read()
    ns = {"np": np}
    for node in ast.parse(src).body:
        if isinstance(node, ast.FunctionDef) and node.name in ("air_index_dispersion", "vacuum2air", "air2vacuum"):
            exec(compile(ast.Module([node], []), "air.py", "exec"), ns)
    # vacuum wavelengths (nm): the infrared bands of the benchmarks, the visible, and
    # a few below the 300 nm validity limit (index 1 there)
    nm = np.concatenate([1e7 / np.linspace(500.0, 8000.0, 2001), np.linspace(300.0, 1000.0, 701),
                         np.array([150.0, 250.0, 299.9])])
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        air = ns["vacuum2air"](nm)
        n = ns["air_index_dispersion"](nm * 1e-3)
        vac_of_air = ns["air2vacuum"](nm)      # the same numbers taken as air wavelengths
    np.savez_compressed(os.path.join(HERE, "golden_units.npz"), vac_nm=nm, air_nm=air, index=n,
                        air2vac_nm=vac_of_air)
    print("wrote", len(nm), "wavelengths")


if __name__ == "__main__":
    main()
