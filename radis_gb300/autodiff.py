"""Derivatives of the synthesised spectrum with respect to (T, p, x).

The reference has no derivatives; this module differentiates the same FP32
LDM synthesis the plans compute, through the library's hand-written kernels:

* ``absorbance(plan, T, p, x, ...)`` is a ``torch.autograd.Function``: its
  forward is ``rg_synthesize`` (absorbance = abscoeff x path length, on the
  plan's grid) and its backward is ``rg_backward``, the adjoint of the
  synthesis (FFT of the upstream gradient, Voigt multiply and inverse FFT per
  node pair, gather at every line's eight LDM cells, per-line chain rule).
* ``jacobian(plan, T, p, x, ...)`` returns abscoeff and its three forward-mode
  derivative spectra from ``rg_jvp`` (tangent scatter + the ordinary FFT
  stages).

The LDM node axes are held at the values the conditions give: the axes are a
discretisation choice of the method (radis/gpu/params.py:89-117), so the
derivative is that of the discrete synthesis on a fixed grid.  Partition
functions enter as Q(Tref)/Q(T) per isotopologue (radis/lbl/base.py:2664-2677);
their temperature derivative is taken on the host by central differences of
the given callables.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import _lib as L

TREF = 296.0


def _q_terms(Q, T, n_iso):
    """(q_ratio, d ln q_ratio / dT) per isotopologue for callables Q_i(T), or
    (None, None) when Q is None (ratio 1)."""
    if Q is None:
        return None, None
    Qs = list(Q) if isinstance(Q, (list, tuple)) else [Q] * n_iso
    if len(Qs) != n_iso:
        raise ValueError(f"need {n_iso} partition functions, got {len(Qs)}")
    h = 1e-3 * T
    q = np.array([float(f(TREF)) / float(f(T)) for f in Qs])
    dlnq = np.array([-(math.log(float(f(T + h))) - math.log(float(f(T - h)))) / (2 * h) for f in Qs])
    return q, dlnq


def _stream(dev):
    """torch's current stream as a cudaStream_t for the C ABI, where NULL
    would select the library context's own stream: torch's default stream
    (handle 0) is passed as cudaStreamLegacy (1)."""
    return torch.cuda.current_stream(dev).cuda_stream or 1


class _Absorbance(torch.autograd.Function):
    @staticmethod
    def forward(ctx, T, p_bar, x, plan, path_length, Q):
        Tv, pv, xv = float(T), float(p_bar), float(x)
        q, dlnq = _q_terms(Q, Tv, plan.lines.n_iso)
        dev = torch.device("cuda", plan.lines.ctx.device)
        out = torch.empty(plan.n_v, dtype=torch.float32, device=dev)
        info = plan.synthesize_device(Tv, pv, xv, out.data_ptr(), _stream(dev), q_ratio=q)
        ctx.plan, ctx.cond, ctx.path_length = plan, (Tv, pv, xv, q, dlnq), float(path_length)
        ctx.dtypes = [(t.dtype, t.device) if torch.is_tensor(t) else (torch.float64, torch.device("cpu"))
                      for t in (T, p_bar, x)]
        scale = math.exp(info.log_scale) * float(path_length)
        return out * scale if scale != 1.0 else out

    @staticmethod
    def backward(ctx, grad):
        Tv, pv, xv, q, dlnq = ctx.cond
        g = grad.contiguous().to(torch.float32) * ctx.path_length   # dL/d abscoeff
        d = ctx.plan.backward(Tv, pv, xv, g.data_ptr(), q_ratio=q, dlnq_dT=dlnq,
                              stream_ptr=_stream(g.device))
        outs = [torch.tensor(float(d[i]), dtype=dt, device=dv) for i, (dt, dv) in enumerate(ctx.dtypes)]
        return outs[0], outs[1], outs[2], None, None, None


def absorbance(plan: L.Plan, T, p_bar, x, path_length: float = 1.0, Q=None) -> torch.Tensor:
    """Absorbance (abscoeff x path_length, float32 on the plan's device) on the
    plan's grid, differentiable in T [K], p_bar [bar] and x (0-d tensors with
    requires_grad).  ``Q``: partition function callable(s) Q_i(T), one per
    isotopologue of the line list, or None for Q(Tref)/Q(T) = 1."""
    return _Absorbance.apply(T, p_bar, x, plan, path_length, Q)


def jacobian(plan: L.Plan, T: float, p_bar: float, x: float, Q=None):
    """Forward mode: (abscoeff, d abscoeff/dT, d/dp_bar, d/dx) as float32
    tensors of n_v on the plan's device (true units: cm-1, cm-1/K, cm-1/bar,
    cm-1)."""
    q, dlnq = _q_terms(Q, float(T), plan.lines.n_iso)
    dev = torch.device("cuda", plan.lines.ctx.device)
    st = _stream(dev)
    a = torch.empty(plan.n_v, dtype=torch.float32, device=dev)
    info = plan.synthesize_device(T, p_bar, x, a.data_ptr(), st, q_ratio=q)
    d = torch.empty((3, plan.n_v), dtype=torch.float32, device=dev)
    dinfo = plan.jvp(T, p_bar, x, d.data_ptr(), q_ratio=q, dlnq_dT=dlnq, stream_ptr=st)
    sa, sd = math.exp(info.log_scale), math.exp(dinfo.log_scale)
    if sa != 1.0:
        a = a * sa
    if sd != 1.0:
        d = d * sd
    return a, d[0], d[1], d[2]
