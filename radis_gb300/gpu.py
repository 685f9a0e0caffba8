"""Drop-in replacement of the reference's GPU application object.

``gpuApp`` has the constructor, ``iterate``, ``get_griddims`` and
``__del__``/``free`` contract of radis/gpu/gpu.py:35-380, so that
``SpectrumFactory.eq_spectrum_gpu`` (which imports it lazily,
radis/lbl/factory.py:1230-1231) can use it unchanged.  Underneath it drives the
sm_103a kernels through the C ABI (include/radis_gb300.h); there is no CPU
fallback.

Behavioural differences from the reference, each deliberate (same choices as
the CPU path the results are checked against):
* pressure enters the Lorentzian widths and the line shift in atm
  (bar / 1.01325), as radis/lbl/broadening.py:1063 and base.py:2351 do; the
  reference's shader uses bar (params.py:144, cmdFillLDM.comp:95);
* the Voigt profiles include the CPU path's folding correction
  (broadening.py:1914-1926);
* the intensity is carried as S(T_ref) and Q(T_ref)/Q(T), which is
  algebraically the reference's Einstein-A form (cmdFillLDM.comp:126).
"""
from __future__ import annotations

import numpy as np

from . import _lib as L

C2 = 6.62607015e-34 * 2.99792458e8 / 1.3806490e-23 * 100.0   # hc/k, cm K
TREF = 296.0
STAGES = ("scatter", "fft_col", "fft_row+voigt", "ifft_row", "ifft_col")
QUANTITIES = ("abscoeff", "absorbance", "emissivity_noslit", "transmittance_noslit", "radiance_noslit")


class gpuApp:
    """See radis/gpu/gpu.py:35-97 for the argument meaning.

    v0, da (Pshft, cm-1/atm), na (Tdpair), S0 (Einstein-A intensity factor,
    radis/lbl/base.py:2380-2447), El, gamma_arr[2, N] = (self, air), iso (index
    into Mm_arr), Mm_arr (g/mol, Mm_arr[0] unused), Q_intp_list (callables
    Q_i(T), one per slot of Mm_arr)."""

    def __init__(self, vmin, Nv, dv, dxG, dxL, v0, da, na, S0, El, gamma_arr, iso, Mm_arr,
                 Q_intp_list, verbose=0, device_id=0, S_ref=None, n_G=None, n_L=None,
                 folding_thresh=1e-6):
        """Extra keywords (not in the reference): ``S_ref`` gives HITRAN
        intensities at 296 K instead of S0; ``n_G``/``n_L`` fix the node counts
        instead of the dxG/dxL spacing; ``folding_thresh`` as in the CPU path
        (radis/lbl/factory.py:437)."""
        self.backend = "gb300-cuda"
        self.verbose = verbose
        self._freed = True
        if isinstance(device_id, str):
            device_id = 0   # device names are not matched: single-GPU build
        gamma_arr = np.asarray(gamma_arr)
        if gamma_arr.ndim != 2 or gamma_arr.shape[0] < 2:
            raise ValueError("gamma_arr must be (2, N): self then air broadening")
        iso = np.asarray(iso).astype(np.int64)
        Mm = np.asarray(Mm_arr, dtype=np.float64).copy()
        if len(Mm) > 16:
            raise ValueError("at most 16 isotopologue slots")
        Mm[~(Mm > 0)] = 1.0          # unused slots (Mm_arr[0] is always 0)
        self._Q = list(Q_intp_list)
        if len(self._Q) != len(Mm):
            raise ValueError("Q_intp_list needs one callable per slot of Mm_arr")
        self._Qref = np.array([float(q(TREF)) for q in self._Q], dtype=np.float64)
        v0 = np.asarray(v0, dtype=np.float64)
        El64 = np.asarray(El, dtype=np.float64)
        # S0 -> S(T_ref) giving the same per-line intensity
        # N x S0 (exp(-c2 El/T) - exp(-c2 (El+v0)/T)) / Q(T)  (cmdFillLDM.comp:126)
        if S_ref is None:
            S_ref = (np.asarray(S0, dtype=np.float64) * np.exp(-C2 * El64 / TREF)
                     * (-np.expm1(-C2 * v0 / TREF)) / self._Qref[iso])
        da = np.asarray(da, np.float32)
        lines = dict(v0=v0, S_ref=S_ref, El=np.asarray(El, np.float32),
                     g_self=np.asarray(gamma_arr[0], np.float32),
                     g_air=np.asarray(gamma_arr[-1], np.float32),
                     n_air=np.asarray(na, np.float32), delta=da if np.any(da) else None,
                     iso=iso.astype(np.uint8))
        lines = L.sort_lines(lines)   # the tile scatter needs ascending v0
        self.ctx = L.Context(int(device_id))
        self.lines = L.Lines(self.ctx, lines, Mm, t_ref=TREF)
        self.plan = L.Plan(self.lines, vmin, dv, int(Nv), dxG=dxG, dxL=dxL, n_G=n_G, n_L=n_L,
                           folding_thresh=folding_thresh)
        # tables the library can evaluate itself: Q(Tref)/Q(T) per spectrum
        # without calling back into Python
        from .partition import TabulatedQ
        self._q_in_lib = all(isinstance(q, TabulatedQ) for q in self._Q)
        if self._q_in_lib:
            for i, q in enumerate(self._Q):
                self.lines.set_partition(i, q.T, q.Q, q.kind)
        self._freed = False
        self.Nv, self.vmin, self.dv = int(Nv), float(vmin), float(dv)
        self._griddims = (0, 0)
        self.last_info = None

    QUANTITIES = QUANTITIES

    def q_ratio(self, T):
        return np.array([self._Qref[i] / float(q(T)) for i, q in enumerate(self._Q)])

    def iterate(self, p, T, mole_fraction, verbose=0, l=1.0, slit_FWHM=0.0):
        """Absorption coefficient (cm-1, float32 when representable) on the
        plan's grid and a dict of stage times (ms).  p in bar, T in K.  ``l``
        and ``slit_FWHM`` are accepted and unused, as in the reference
        (gpu.py:308-311)."""
        if self._freed:
            raise RuntimeError("gpuApp was freed (exit_gpu)")
        q = None if self._q_in_lib else self.q_ratio(T)
        out, info = self.plan.synthesize_host(T, p, mole_fraction, q_ratio=q, timing=True)
        g = info.grid
        self._griddims = (g.n_L, g.n_G)
        self.last_info = info
        times = {n: float(info.stage_ms[i]) for i, n in enumerate(STAGES)}
        times["total"] = float(info.stage_ms[5])
        if info.log_scale != 0.0:
            out = out.astype(np.float64) * np.exp(info.log_scale)
        if verbose >= 1 or self.verbose >= 2:
            print(f"gpuApp: N_G={g.n_G} N_L={g.n_L} n_ft={g.n_ft} total {times['total']:.3f} ms")
        return out, times

    def iterate_quantities(self, p, T, mole_fraction, path_length, verbose=0):
        """The spectral quantities of eq_spectrum_gpu on the plan's grid, with
        the post-processing of radis/lbl/factory.py:1284-1297 fused into the
        last kernel: ({abscoeff, absorbance, emissivity_noslit,
        transmittance_noslit, radiance_noslit}, stage times).  float32 arrays
        (float64 for abscoeff/absorbance when the spectrum exceeds FP32)."""
        if self._freed:
            raise RuntimeError("gpuApp was freed (exit_gpu)")
        q = None if self._q_in_lib else self.q_ratio(T)
        out, info = self.plan.synthesize_quantities_host(T, p, mole_fraction, path_length, q_ratio=q,
                                                         timing=True)
        g = info.grid
        self._griddims = (g.n_L, g.n_G)
        self.last_info = info
        times = {n: float(info.stage_ms[i]) for i, n in enumerate(STAGES)}
        times["total"] = float(info.stage_ms[5])
        if info.log_scale != 0.0:
            for k in ("abscoeff", "absorbance"):
                out[k] = out[k].astype(np.float64) * np.exp(info.log_scale)
        if verbose >= 1 or self.verbose >= 2:
            print(f"gpuApp: N_G={g.n_G} N_L={g.n_L} n_ft={g.n_ft} total {times['total']:.3f} ms")
        return out, times

    def get_griddims(self):
        """(N_L, N_G) of the last iterate (radis/gpu/gpu.py:372-374)."""
        return self._griddims

    def free(self):
        """Release the device objects; safe to call twice (gpu.py:376-380)."""
        if self._freed:
            return
        self.plan.close()
        self.lines.close()
        self.ctx.close()
        self._freed = True

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
