"""SpectrumFactory front end of the GPU equilibrium synthesis.

Mirrors the part of radis/lbl/factory.py the GPU path uses: the factory
inputs and parameters (factory.py:415-440, 625-720), the wavenumber grid
(factory.py:1953-2044, 2560-2617), ``eq_spectrum_gpu`` (factory.py:1027-1391)
and ``calc_spectrum(..., mode='gpu')`` (radis/lbl/calc.py:37, 1016-1028).
Line databases come from HITRAN-160 files (radis_gb300.hitran) or column
dicts; partition functions are callables Q(T) per isotopologue (the
reference's TIPS tables need hapi, which is not part of this path).
"""
from __future__ import annotations

import time
import types

import numpy as np

from . import __version__
from .gpu import gpuApp
from .spectrum import DEFAULT_UNITS, Spectrum
from .units import get_wavenumber_range

# default LDM steps (radis/lbl/loader.py:452-460, 538-543)
DXL_DEFAULT = float(np.log((0.01 / 0.20) ** 0.5 + 1))
DXG_DEFAULT = float(np.log((0.01 / 0.46) ** 0.5 + 1))

# HITRAN molecule ids and isotopologue molar masses (g/mol) of the species
# the benchmarks use; other species need molar_mass= explicitly
MOLECULE_ID = {"H2O": 1, "CO2": 2, "CO": 5}
MOLAR_MASS = {
    ("H2O", 1): 18.010565, ("H2O", 2): 20.014811, ("H2O", 3): 19.01478,
    ("CO2", 1): 43.98983, ("CO2", 2): 44.993185, ("CO2", 3): 45.994076,
    ("CO", 1): 27.994915, ("CO", 2): 28.99827, ("CO", 3): 29.999161,
}


class SpectrumFactory:
    """Subset of radis.lbl.factory.SpectrumFactory for eq_spectrum_gpu."""

    def __init__(self, wmin=None, wmax=None, wunit=None, wavenum_min=None, wavenum_max=None,
                 wavelength_min=None, wavelength_max=None, Tref=296.0, pressure=1.01325, mole_fraction=1.0,
                 path_length=1.0, wstep=0.01, isotope="all", medium="air", neighbour_lines=0.0,
                 folding_thresh=1e-6, broadening_method="voigt_poly", verbose=0, warnings=None,
                 species=None, molecule=None, dxG=None, dxL=None, n_G=None, n_L=None, molar_mass=None,
                 partition_functions=None, **kwargs):
        """Arguments in the reference's order (radis/lbl/factory.py:419-470).
        The range is one of wmin/wmax (``wunit``, cm-1 by default),
        wavenum_min/wavenum_max (cm-1) or wavelength_min/wavelength_max (nm in
        ``medium``); it also sets the spectra's default output unit.
        ``broadening_method`` is recorded only: eq_spectrum_gpu always runs
        the LDM with the FFT, as the reference's does.  ``molecule`` is an
        alias of ``species``."""
        if species is not None and molecule is not None and species != molecule:
            raise ValueError("species and molecule (an alias) differ")
        molecule = species if species is not None else molecule
        wavenum_min, wavenum_max, input_wunit = get_wavenumber_range(
            wmin, wmax, wunit, wavenum_min, wavenum_max, wavelength_min, wavelength_max, medium)
        self.input_wunit = input_wunit
        self.input = types.SimpleNamespace(
            wavenum_min=float(wavenum_min), wavenum_max=float(wavenum_max), molecule=molecule,
            isotope=isotope, pressure=float(pressure), mole_fraction=float(mole_fraction),
            path_length=float(path_length), Tref=float(Tref), Tgas=None, self_absorption=True,
            isatom=False, medium=medium)
        self.params = types.SimpleNamespace(
            wstep=float(wstep), dxG=float(dxG or DXG_DEFAULT), dxL=float(dxL or DXL_DEFAULT),
            n_G=n_G, n_L=n_L, broadening_method=broadening_method,
            folding_thresh=float(folding_thresh), neighbour_lines=float(neighbour_lines),
            optimization="simple")
        self.verbose = verbose
        self.units = dict(DEFAULT_UNITS)
        self._molar_mass = molar_mass
        self._Q = partition_functions
        self.df0 = None
        self._generate_wavenumber_arrays()

    # --- wavenumber grid (factory.py:2560-2617) ---------------------------------
    def _generate_wavenumber_arrays(self):
        ws = self.params.wstep
        n_out = int(round((self.input.wavenum_max - self.input.wavenum_min) / ws)) + 1
        m = int(np.ceil(self.params.neighbour_lines / ws)) if self.params.neighbour_lines else 0
        self.params.wavenum_min_calc = self.input.wavenum_min - m * ws
        self.wavenumber_calc = self.params.wavenum_min_calc + ws * np.arange(n_out + 2 * m)
        self.woutrange = (m, m + n_out)
        self.wavenumber = self.wavenumber_calc[m:m + n_out]

    # --- line databases -----------------------------------------------------------
    def load_databank(self, path=None, format="hitran", db_use_cached=True, **kwargs):
        """Load a HITRAN-160 file (radis/lbl/loader.py:1715 load_databank):
        parsed by the library's parser and cached as columns beside the file
        (``db_use_cached``: True, False, 'regen' or 'force', as hit2df's
        ``cache``, radis/api/hitranapi.py:182-380)."""
        if format not in ("hitran", "hitran160", "par"):
            raise NotImplementedError(f"format {format!r}: only HITRAN-160 files are read here")
        from .hitran import load_hitran
        d = load_hitran(path, cache=db_use_cached if db_use_cached is not None else True)
        return self.load_lines(d)

    def load_lines(self, lines: dict):
        """Use a column dict (v0, S_ref, El, g_air, g_self, n_air, optional
        delta, iso (HITRAN 1-based), id)."""
        d = {k: np.asarray(v) for k, v in lines.items() if v is not None}
        n = len(d["v0"])
        if "iso" not in d:
            d["iso"] = np.ones(n, dtype=np.int64)
        iso_sel = self.input.isotope
        if iso_sel not in (None, "all"):
            wanted = [int(i) for i in str(iso_sel).split(",")]
            keep = np.isin(d["iso"], wanted)
            d = {k: v[keep] for k, v in d.items()}
        lo = self.params.wavenum_min_calc - self.params.neighbour_lines
        hi = self.wavenumber_calc[-1] + self.params.neighbour_lines
        keep = (d["v0"] >= lo) & (d["v0"] <= hi)
        self.df0 = {k: v[keep] for k, v in d.items()}
        return self

    def _isotope_tables(self, iso_set):
        mol = self.input.molecule
        n_slots = int(max(iso_set)) + 1
        Mm = np.zeros(n_slots)
        for i in iso_set:
            if self._molar_mass is not None:
                mm = self._molar_mass
                Mm[i] = float(mm[i] if isinstance(mm, dict) else mm)
            elif (mol, int(i)) in MOLAR_MASS:
                Mm[i] = MOLAR_MASS[(mol, int(i))]
            else:
                raise ValueError(f"no molar mass for {mol} isotopologue {i}: pass molar_mass=")
        Q = []
        for i in range(n_slots):
            q = None
            if self._Q is not None:
                q = self._Q.get(i) if isinstance(self._Q, dict) else self._Q
            Q.append(q if q is not None else (lambda T: 1.0))
        return Mm, Q

    # --- eq_spectrum_gpu (factory.py:1027-1391) -----------------------------------
    def eq_spectrum_gpu(self, Tgas, mole_fraction=None, diluent=None, path_length=None,
                        pressure=None, name=None, backend="vulkan", device_id=0, exit_gpu=False,
                        verbose=None) -> Spectrum:
        if self.df0 is None:
            raise ValueError("load a line database first (load_databank / load_lines)")
        if path_length is not None:
            self.input.path_length = float(path_length)
        if mole_fraction is not None:
            self.input.mole_fraction = float(mole_fraction)
        if pressure is not None:
            self.input.pressure = float(pressure)
        try:
            Tgas = float(Tgas)
        except (TypeError, ValueError):
            raise ValueError("Tgas should be float.")
        self.input.Tgas = Tgas
        verbose = self.verbose if verbose is None else verbose
        t0 = time.perf_counter()
        d = self.df0
        iso = d["iso"].astype(np.int64)
        iso_set = sorted(set(iso.tolist()))
        Mm, Q = self._isotope_tables(iso_set)
        app = gpuApp(self.params.wavenum_min_calc, len(self.wavenumber_calc), self.params.wstep,
                     self.params.dxG, self.params.dxL, d["v0"], d.get("delta", np.zeros(len(iso))),
                     d["n_air"], None, d["El"], np.stack([d["g_self"], d["g_air"]]), iso, Mm, Q,
                     verbose=verbose, device_id=device_id, S_ref=d["S_ref"],
                     n_G=self.params.n_G, n_L=self.params.n_L,
                     folding_thresh=self.params.folding_thresh)
        # abscoeff and the post-processing of factory.py:1284-1297 from the device
        # (fused into the last kernel), cropped to the output range
        quant, times = app.iterate_quantities(self.input.pressure, Tgas, self.input.mole_fraction,
                                              self.input.path_length, verbose=verbose)
        n_L, n_G = app.get_griddims()
        w0, w1 = self.woutrange
        abscoeff, a, e, t, r = (quant[k][w0:w1] for k in gpuApp.QUANTITIES)
        conditions = dict(
            Tgas=Tgas, Trot=Tgas, Tvib=Tgas, pressure=self.input.pressure,
            pressure_mbar=self.input.pressure * 1e3, mole_fraction=self.input.mole_fraction,
            path_length=self.input.path_length, wavenum_min=self.input.wavenum_min,
            wavenum_max=self.input.wavenum_max, wstep=self.params.wstep,
            molecule=self.input.molecule, isotope=self.input.isotope, Tref=self.input.Tref,
            dxG=self.params.dxG, dxL=self.params.dxL, broadening_method=self.params.broadening_method,
            folding_thresh=self.params.folding_thresh,
            calculation_time=time.perf_counter() - t0, lines_calculated=int(len(iso)),
            thermal_equilibrium=True, diluents=diluent if diluent is not None else {"air": 1 - self.input.mole_fraction},
            radis_version=f"radis_gb300 {__version__}", gpu_backend=app.backend,
            spectral_points=len(self.wavenumber), add_at_used="gpu-backend", NwL=n_L, NwG=n_G,
            gpu_times=times, default_output_unit=self.input_wunit, medium=self.input.medium)
        s = Spectrum(quantities=dict(wavenumber=self.wavenumber, abscoeff=abscoeff, absorbance=a,
                                     emissivity_noslit=e, transmittance_noslit=t,
                                     radiance_noslit=r),
                     units=self.units, conditions=conditions, gpu_app=None if exit_gpu else app,
                     name=name)
        s._woutrange = self.woutrange
        if exit_gpu:
            app.free()
        return s


def calc_spectrum(wmin=None, wmax=None, wunit=None, Tgas=None, Tvib=None, Trot=None, Telec=None,
                  pressure=1.01325, species=None, isotope="all", mole_fraction=1.0, diluent=None,
                  path_length=1.0, databank=None, medium="air", wstep=0.01, name=None, mode="gpu",
                  verbose=0, return_factory=False, **kwargs):
    """One-molecule front end, arguments in the reference's order
    (radis/lbl/calc.py:37-75; mode dispatch :1016-1028).  Equilibrium only
    (Tvib / Trot / Telec absent or equal to Tgas); ``databank``: path of a
    HITRAN-160 file or a column dict; ``molecule=`` is accepted as an alias
    of ``species``; ``wavenum_min=`` / ``wavelength_min=`` ranges pass
    through to the factory."""
    if mode != "gpu":
        raise NotImplementedError("radis_gb300 implements mode='gpu' only")
    for t in (Tvib, Trot, Telec):
        if t is not None and t != Tgas:
            raise NotImplementedError("non-equilibrium temperatures: the GPU path is equilibrium only")
    sf = SpectrumFactory(wmin=wmin, wmax=wmax, wunit=wunit, wstep=wstep, species=species, isotope=isotope,
                         pressure=pressure, mole_fraction=mole_fraction, path_length=path_length, medium=medium,
                         verbose=verbose, **kwargs)
    if isinstance(databank, dict):
        sf.load_lines(databank)
    else:
        sf.load_databank(databank)
    s = sf.eq_spectrum_gpu(Tgas, diluent=diluent, name=name)
    return (s, sf) if return_factory else s
