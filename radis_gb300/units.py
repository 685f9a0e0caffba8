"""Wave units, propagation media and spectral-quantity units for
``Spectrum.get`` (host side).

* Air wavelengths: the refractive index of standard air by Ciddor's
  dispersion relation (P. E. Ciddor, Appl. Opt. 35, 1566 (1996)), as
  radis/phys/air.py:16-63 uses it: n = 1 + 0.05792105 / (238.0185 - s^2)
  + 0.00167917 / (57.362 - s^2), s = 1 / lambda in um, and n = 1 below its
  300 nm validity limit; lambda_air = lambda_vac / n(lambda_vac)
  (vacuum2air, air.py:66-90).
* Radiance per wavelength <-> per wavenumber: L_nu = L_lambda |d lambda /
  d nu| = L_lambda 1e7 / nu^2 for nm and cm-1 (radis/phys/units.py:
  convert_rad2cm / convert_rad2nm, used by convert_universal :333-396);
  other unit changes are products of SI prefix factors.
"""
from __future__ import annotations

import warnings

import numpy as np

_POWER = {"W": 1.0, "kW": 1e3, "mW": 1e-3, "µW": 1e-6, "uW": 1e-6, "nW": 1e-9}
_AREA = {"m2": 1.0, "cm2": 1e-4, "mm2": 1e-6}
_PER_LENGTH = {"m": 1.0, "cm": 1e-2, "mm": 1e-3, "µm": 1e-6, "um": 1e-6, "nm": 1e-9}   # metres
_PER_WAVENUMBER = {"m-1": 1.0, "cm-1": 1e2}                                           # 1/m
_WAVEUNITS = {"cm-1": "cm-1", "cm_1": "cm-1", "wavenumber": "cm-1", "nm": "nm", "wavelength": "nm",
              "nm_air": "nm", "nm_vac": "nm_vac", "nm_vacuum": "nm_vac", "wavelength_vacuum": "nm_vac"}


def air_index(lbd_um):
    """Refractive index of standard air at vacuum wavelength ``lbd_um`` (um)."""
    lbd = np.asarray(lbd_um, dtype=np.float64)
    s2 = lbd ** -2.0
    n = 1.0 + 0.05792105 / (238.0185 - s2) + 0.00167917 / (57.362 - s2)
    low = lbd < 0.3
    if np.any(low):
        warnings.warn("air index used below its 300 nm validity limit (n = 1 there)")
        n = np.where(low, 1.0, n)
    return n


def vacuum2air(nm):
    """Wavelength in air of vacuum wavelength ``nm``."""
    nm = np.asarray(nm, dtype=np.float64)
    return nm / air_index(nm * 1e-3)


def cast_waveunit(wunit: str) -> str:
    """'cm-1', 'nm' (in the spectrum's medium) or 'nm_vac'."""
    try:
        return _WAVEUNITS[wunit]
    except KeyError:
        raise ValueError(f"unknown wave unit {wunit!r}: use 'cm-1', 'nm', 'nm_air' or 'nm_vac'") from None


def _radiance_unit(u: str):
    """(SI factor, 'nm' | 'cm-1') of a radiance unit such as 'mW/cm2/sr/nm':
    one power over an area, a solid angle and a wavelength or wavenumber
    interval, in any order."""
    parts = [p.strip() for p in u.split("/")]
    if len(parts) != 4 or parts[0] not in _POWER or "sr" not in parts[1:]:
        raise ValueError(f"radiance unit {u!r} not understood (e.g. 'mW/cm2/sr/nm')")
    f, kind, area = _POWER[parts[0]], None, None
    for p in parts[1:]:
        if p == "sr":
            continue
        if p in _AREA and area is None:
            area = _AREA[p]
        elif p in _PER_WAVENUMBER and kind is None:
            f /= _PER_WAVENUMBER[p]
            kind = "cm-1"
        elif p in _PER_LENGTH and kind is None:
            f /= _PER_LENGTH[p]
            kind = "nm"
        else:
            raise ValueError(f"radiance unit {u!r} not understood")
    if area is None or kind is None:
        raise ValueError(f"radiance unit {u!r} not understood")
    return f / area, kind


def convert_radiance(I, from_unit: str, to_unit: str, wavenumber):
    """Radiance in ``from_unit`` to ``to_unit``; per-wavelength <-> per-
    wavenumber changes use the vacuum wavenumber ``wavenumber`` (cm-1)."""
    if from_unit == to_unit:
        return np.asarray(I)
    f0, k0 = _radiance_unit(from_unit)
    f1, k1 = _radiance_unit(to_unit)
    si = np.asarray(I, dtype=np.float64) * f0          # W/m2/sr per m, or per m-1
    if k0 != k1:
        nu = np.asarray(wavenumber, dtype=np.float64) * 1e2          # 1/m
        si = si / nu ** 2 if k0 == "nm" else si * nu ** 2            # |d lambda / d nu| = 1 / nu^2 (SI)
    return si / f1


def convert_per_length(I, from_unit: str, to_unit: str):
    """A coefficient per unit length (abscoeff: 'cm-1' <-> 'm-1')."""
    if from_unit == to_unit:
        return np.asarray(I)
    try:
        return np.asarray(I, dtype=np.float64) * _PER_WAVENUMBER[from_unit] / _PER_WAVENUMBER[to_unit]
    except KeyError:
        raise ValueError(f"cannot convert {from_unit!r} to {to_unit!r}") from None


def air2vacuum(nm):
    """Vacuum wavelength of air wavelength ``nm``: lambda n(lambda), the index
    evaluated at the air wavelength (radis/phys/air.py:93-119, which notes
    the approximation: the index varies little over the shift)."""
    nm = np.asarray(nm, dtype=np.float64)
    return air_index(nm * 1e-3) * nm


def nm2cm(nm):
    """Vacuum wavelength (nm) -> wavenumber (cm-1)."""
    return 1e7 / np.asarray(nm, dtype=np.float64)


def nm_air2cm(nm):
    """Air wavelength (nm) -> vacuum wavenumber (cm-1)."""
    return nm2cm(air2vacuum(nm))


_RANGE_UNITS = {"cm-1": ("cm-1", 1.0), "1/cm": ("cm-1", 1.0), "m-1": ("cm-1", 1e-2), "1/m": ("cm-1", 1e-2),
                "nm": ("nm", 1.0), "nm_air": ("nm", 1.0), "nm_vac": ("nm", 1.0), "nm_vacuum": ("nm", 1.0),
                "um": ("nm", 1e3), "µm": ("nm", 1e3), "m": ("nm", 1e9)}


def get_wavenumber_range(wmin=None, wmax=None, wunit=None, wavenum_min=None, wavenum_max=None,
                         wavelength_min=None, wavelength_max=None, medium="air"):
    """(wavenum_min, wavenum_max, input_wunit) from exactly one of: wmin/wmax
    in ``wunit`` (default cm-1; wavelength units in ``medium``, or 'nm_air' /
    'nm_vac'), wavenum_min/wavenum_max (cm-1), wavelength_min/wavelength_max
    (nm in ``medium``).  Wavelengths in air go through air2vacuum
    (radis/lbl/base.py get_wavenumber_range; input_wunit is 'cm-1', 'nm' or
    'nm_vac', the default output unit of the spectra)."""
    if medium not in ("air", "vacuum"):
        raise NotImplementedError(f"unknown propagating medium {medium!r}: use 'air' or 'vacuum'")
    given = [wmin is not None and wmax is not None, wavenum_min is not None and wavenum_max is not None,
             wavelength_min is not None and wavelength_max is not None]
    if sum(given) != 1:
        raise ValueError("pass exactly one range: wmin/wmax (with wunit), wavenum_min/wavenum_max (cm-1) "
                         "or wavelength_min/wavelength_max (nm)")
    if wunit is not None and not given[0]:
        raise ValueError("wunit goes with wmin/wmax")
    if given[0]:
        wu = "cm-1" if wunit is None else wunit
        if wu not in _RANGE_UNITS:
            raise ValueError(f"unknown range unit {wu!r}")
        kind, f = _RANGE_UNITS[wu]
        if wu in ("nm_vac", "nm_vacuum"):
            medium = "vacuum"
        elif wu == "nm_air":
            medium = "air"
        if kind == "cm-1":
            wavenum_min, wavenum_max = float(wmin) * f, float(wmax) * f
        else:
            wavelength_min, wavelength_max = float(wmin) * f, float(wmax) * f
    if wavenum_min is not None:
        lo, hi, unit = float(wavenum_min), float(wavenum_max), "cm-1"
    else:
        a, b = float(wavelength_min), float(wavelength_max)
        if not a < b:
            raise ValueError("wavelength_min must be below wavelength_max")
        conv = nm_air2cm if medium == "air" else nm2cm
        lo, hi = float(conv(b)), float(conv(a))
        unit = "nm" if medium == "air" else "nm_vac"
    if not lo < hi:
        raise ValueError("the range is empty: give min < max")
    return lo, hi, unit
