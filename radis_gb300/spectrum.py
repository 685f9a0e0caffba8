"""Spectrum container returned by the GPU synthesis.

Keeps the reference's output contract for this path
(radis/lbl/factory.py:1284-1376): quantities wavenumber, abscoeff,
absorbance, emissivity_noslit, transmittance_noslit, radiance_noslit; the
conditions keys the GPU path sets; ``recalc_gpu`` (radis/spectrum/spectrum.py:
6438-6572) to re-run the resident GPU application at new conditions; and
``exit_gpu`` (spectrum.py:6574-6577).  Derived quantities are computed on the
host from abscoeff exactly as the reference does.
"""
from __future__ import annotations

import warnings

import numpy as np

from . import units as U

# radis/phys/constants.py:22,33,38
_H = 6.62607015e-34
_C = 2.99792458e8
_KB = 1.3806490e-23

DEFAULT_UNITS = {
    "wavenumber": "cm-1",
    "abscoeff": "cm-1",
    "absorbance": "",
    "emissivity_noslit": "",
    "transmittance_noslit": "",
    "radiance_noslit": "mW/cm2/sr/nm",
}


class GPUInitWarning(UserWarning):
    """No GPU application attached (radis/misc/warning.py:68)."""


def planck_nm(lambda_nm, T):
    """Black-body radiance in mW/cm2/sr/nm (radis/phys/blackbody.py:35-74)."""
    lbd = np.asarray(lambda_nm, dtype=np.float64) * 1e-9
    return 2 * _H * _C ** 2 / lbd ** 5 / np.expm1(_H * _C / (lbd * _KB * T)) * 1e-10


def derived_quantities(wavenumber, abscoeff, path_length, Tgas):
    """absorbance, emissivity, transmittance, radiance (factory.py:1284-1297,
    radis/spectrum/equations.py:21-44 with unit mW/sr/cm2/nm)."""
    absorbance = abscoeff * path_length
    emissivity = -np.expm1(-absorbance)
    transmittance = 1 - emissivity
    radiance = emissivity * planck_nm(1e7 / np.asarray(wavenumber, np.float64), Tgas)
    return absorbance, emissivity, transmittance, radiance


class Spectrum:
    """Minimal Spectrum: ``get(var)`` -> (wavenumber, values)."""

    def __init__(self, quantities, units=None, conditions=None, cond_units=None, gpu_app=None,
                 name=None, lines=None, **_):
        self._q = {k: np.asarray(v) for k, v in quantities.items()}
        self.units = dict(DEFAULT_UNITS if units is None else units)
        self.conditions = dict(conditions or {})
        self.cond_units = dict(cond_units or {})
        self.gpu_app = gpu_app
        self.name = name
        self.lines = lines
        self._woutrange = None

    @property
    def c(self):
        return self.conditions

    def get_vars(self):
        return [k for k in self._q if k != "wavenumber"]

    def get(self, var, wunit="default", Iunit="default", copy=True):
        """(wave axis, values) of ``var`` (radis/spectrum/spectrum.py:1183-1420).

        ``wunit``: 'cm-1'; 'nm' (wavelength in the spectrum's medium,
        ``conditions['medium']``, air by default); 'nm_air'; 'nm_vac';
        'default' (``conditions['default_output_unit']``, else cm-1).
        ``Iunit``: 'default' is the stored unit, with radiance switched to
        per nm or per cm-1 to match ``wunit``; radiance converts between
        W/mW/uW, cm2/m2 and per nm/um/cm-1 units, abscoeff between cm-1 and
        m-1; unitless quantities take '' or '1'."""
        if var not in self._q:
            self._update(var)
        if wunit == "default":
            wunit = self.conditions.get("default_output_unit", "cm-1")
        force_air = wunit == "nm_air"
        wu = U.cast_waveunit(wunit)
        nu = self._q["wavenumber"]
        if wu == "cm-1":
            w = nu
        else:
            w = 1e7 / np.asarray(nu, dtype=np.float64)    # vacuum wavelength
            medium = "air" if force_air else self.conditions.get("medium", "air")
            if wu == "nm" and medium == "air":
                w = U.vacuum2air(w)
            elif wu == "nm" and medium != "vacuum":
                raise NotImplementedError(f"unknown propagating medium {medium!r}")
        v = self._q[var]
        unit0 = self.units.get(var, "")
        radiance = var in ("radiance", "radiance_noslit")
        if Iunit == "default":
            Iunit = unit0
            if radiance:
                Iunit = unit0.replace("/cm-1", "/nm") if wu != "cm-1" else unit0.replace("/nm", "/cm-1")
        if Iunit != unit0:
            if radiance:
                v = U.convert_radiance(v, unit0, Iunit, nu)
            elif unit0 in ("", "1") and Iunit in ("", "1"):
                pass
            elif unit0 in ("", "1") or Iunit in ("", "1"):
                raise ValueError(f"{var} is dimensionless: Iunit must be '' or '1', not {Iunit!r}")
            else:
                v = U.convert_per_length(v, unit0, Iunit)
        return (np.array(w, copy=True), np.array(v, copy=True)) if copy else (w, v)

    def _update(self, var):
        if "abscoeff" not in self._q:
            raise KeyError(var)
        a, e, t, r = derived_quantities(self._q["wavenumber"], self._q["abscoeff"],
                                        self.conditions["path_length"], self.conditions["Tgas"])
        self._q.update(absorbance=a, emissivity_noslit=e, transmittance_noslit=t, radiance_noslit=r)
        if var not in self._q:
            raise KeyError(var)

    def get_wavenumber(self, copy=True):
        """Vacuum wavenumber (cm-1)."""
        w = self._q["wavenumber"]
        return np.array(w, copy=True) if copy else w

    def get_wavelength(self, medium="air", copy=True):
        """Wavelength (nm) in ``medium`` (spectrum.py:1421-1460)."""
        if medium not in ("air", "vacuum"):
            raise NotImplementedError(f"unknown propagating medium {medium!r}")
        w = 1e7 / np.asarray(self._q["wavenumber"], dtype=np.float64)
        return U.vacuum2air(w) if medium == "air" else w

    def get_waveunit(self):
        """'cm-1': the spectral axis is stored as wavenumbers."""
        return "cm-1"

    def crop(self, wmin=None, wmax=None, wunit="default", inplace=True):
        """Keep the points inside [wmin, wmax] given in ``wunit`` ('cm-1';
        'nm' in the spectrum's medium, 'nm_air', 'nm_vac'; 'default' = the
        default output unit) (radis/spectrum/operations.py crop)."""
        if wunit == "default":
            wunit = self.conditions.get("default_output_unit", "cm-1")
        wu = U.cast_waveunit(wunit)
        medium = "air" if wunit == "nm_air" else self.conditions.get("medium", "air")
        if wu == "cm-1":
            axis = self._q["wavenumber"]
        else:
            axis = self.get_wavelength(medium="vacuum" if wu == "nm_vac" else medium, copy=False)
        sel = np.ones(len(axis), dtype=bool)
        if wmin is not None:
            sel &= axis >= wmin
        if wmax is not None:
            sel &= axis <= wmax
        s = self if inplace else Spectrum(dict(self._q), self.units, self.conditions, self.cond_units,
                                          name=self.name)
        for k in s._q:
            s._q[k] = s._q[k][sel]
        return s

    def recalc_gpu(self, var="abscoeff", wunit="default", Iunit="default", pressure=None, Tgas=None,
                   mole_fraction=None, path_length=None, slit_function=None, verbose=False):
        """Re-run the resident GPU application at new conditions and return
        ``var`` (spectrum.py:6438-6572).  abscoeff and the quantities derived
        from it (absorbance, emissivity, transmittance, radiance) all come from
        the GPU, the post-processing fused into the spectrum's last kernel.
        With ``slit_function`` the slit is applied on the GPU (``apply_slit``)
        and a convolved quantity (transmittance, radiance, emissivity) is
        returned."""
        if self.gpu_app is None:
            warnings.warn("no GPU application attached to this Spectrum (exit_gpu was "
                          "called or exit_gpu=True was used)", GPUInitWarning)
            return None
        c = self.conditions
        if pressure is not None:
            c["pressure"] = pressure
        if Tgas is not None:
            c["Tgas"] = Tgas
        if mole_fraction is not None:
            c["mole_fraction"] = mole_fraction
        if path_length is not None:
            c["path_length"] = path_length
        quant, times = self.gpu_app.iterate_quantities(c["pressure"], c["Tgas"], c["mole_fraction"],
                                                       c["path_length"], verbose=verbose)
        w0, w1 = self._woutrange or (0, len(quant["abscoeff"]))
        for k in list(self._q):
            if k != "wavenumber":
                del self._q[k]
        for k, v in quant.items():
            self._q[k] = v[w0:w1]
        n_L, n_G = self.gpu_app.get_griddims()
        c.update(NwL=n_L, NwG=n_G, gpu_times=times)
        if slit_function is not None:
            # the reference stores the slit and leaves its application as a TODO
            # (spectrum.py:6527-6534); here the GPU slit applies it
            c["slit_function"] = slit_function
            self.apply_slit(slit_function, shape=c.get("slit_shape", "triangular"))
            if var in self._q:
                return self.get(var, wunit=wunit, Iunit=Iunit)[1]
        key = {"transmittance": "transmittance_noslit", "radiance": "radiance_noslit",
               "emissivity": "emissivity_noslit"}.get(var, var)
        return self.get(key, wunit=wunit, Iunit=Iunit)[1]

    def apply_slit(self, slit_function, unit="cm-1", shape="triangular", center_wavespace=None, norm_by="area",
                   mode="valid", store=True, slit_dispersion=None, assert_evenly_spaced=True, verbose=False,
                   inplace=True, calc_range=4):
        """Convolve every ``*_noslit`` quantity with the instrument slit and
        store it without the suffix (radis/spectrum/spectrum.py:3127-3579),
        the convolution on the GPU (``radis_gb300.slit``).  ``slit_function``:
        FWHM (``shape`` 'triangular' or 'gaussian'), (top, base) for
        'trapezoidal', or sampled (w, I) arrays; given in the spectrum's
        wavespace (cm-1).  Slit dispersion is not provided."""
        import torch

        from . import slit as S

        if slit_dispersion is not None:
            raise NotImplementedError("slit dispersion is not provided")
        if "abscoeff" in self._q and "transmittance_noslit" not in self._q:
            self._update("transmittance_noslit")
        varlist = [k for k in self.get_vars() if k.endswith("_noslit")]
        if not varlist:
            raise AssertionError("No spectral arrays to apply slit on. Spectral arrays to be convolved "
                                 f"should end with _noslit. Available arrays in Spectrum : {self.get_vars()}")
        w = np.asarray(self._q["wavenumber"], dtype=np.float64)
        wstep = np.abs(np.diff(w)).min()
        if assert_evenly_spaced and not np.allclose(np.diff(w), np.diff(w).mean(), atol=wstep * 1e-3):
            raise ValueError("Spectrum is not evenly spaced. Cannot apply slit function.")
        if center_wavespace is None:
            center_wavespace = w[len(w) // 2]
        w_slit, I_slit = S.get_slit_function(slit_function, unit=unit, norm_by=norm_by, shape=shape,
                                             center_wavespace=center_wavespace, return_unit="cm-1",
                                             wstep=wstep, calc_range=calc_range)
        taps = S.slit_on_grid(w_slit, I_slit, wstep)
        s = self if inplace else Spectrum(dict(self._q), self.units, self.conditions, self.cond_units,
                                          name=self.name)
        dev = torch.device("cuda", getattr(getattr(self.gpu_app, "ctx", None), "device", 0) or 0)
        ctx = getattr(self.gpu_app, "ctx", None)
        for qns in varlist:
            I_dev = torch.as_tensor(np.asarray(self._q[qns], dtype=np.float32), device=dev)
            out = S.convolve_device(I_dev, taps, wstep, mode=mode, ctx=ctx)
            s._q[qns[:-7]] = out.cpu().numpy()
            s.units[qns[:-7]] = self.units.get(qns, "")
        s.conditions.update(slit_function=slit_function, slit_unit=unit, slit_shape=shape, norm_by=norm_by,
                            slit_dispersion=slit_dispersion)
        return s

    def exit_gpu(self):
        """Release the GPU application (spectrum.py:6574-6577)."""
        if self.gpu_app is not None:
            self.gpu_app.free()
            self.gpu_app = None
