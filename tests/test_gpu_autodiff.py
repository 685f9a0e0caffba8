"""Derivatives of the spectrum with respect to (T, p, x) through the C ABI
(rg_backward: adjoint / reverse mode; rg_jvp: tangent / forward mode) and the
torch.autograd.Function on top, checked against central finite differences
of the FP64 CPU oracle on the same fixed LDM node axes and FFT length.

Tolerances (stated here, used below):
* derivative spectra: max |dA_gpu - dA_fd| <= 1e-3 * max |dA_fd| per parameter;
* gradient-vector products: |g.dA_gpu - g.dA_fd| <= 1e-3 * sum |g| |dA_fd|;
* adjoint against tangent (both GPU): <= 2e-4 of sum |g| |dA|.
The finite-difference steps are 1e-5 of each parameter: the FP64 round-off
of the difference is ~1e-11 relative, and few lines cross an LDM cell edge
within the step (the weights are piecewise linear in the coordinates).
"""
import os

import numpy as np
import pytest

from oracle import ldm_oracle as O
from radis_gb300 import _lib as L
from radis_gb300 import synthetic as S

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

WORKERS = os.cpu_count() or 1
REL_H = 1e-5
TREF = 296.0


@pytest.fixture(scope="module")
def ctx(native_lib):
    c = L.Context(0)
    yield c
    c.close()


def power_Q(k):
    return lambda T: (T / TREF) ** k


CASES = {
    # CO-like lines with pressure shifts, 20 001 points
    "shift": dict(lines=lambda: S.uniform_lines(4000, 2000.0, 2040.0, seed=41, delta=(-0.01, 0.01)),
                  M=28.0, Q=None, grid=(2000.0, 0.002, 20001), cond=(900.0, 2.0, 0.3)),
    # three isotopologues with Q(T) = (T/Tref)^k
    "isotopes": dict(lines=lambda: dict(S.uniform_lines(6000, 2000.0, 2030.0, seed=42),
                                        iso=np.random.default_rng(43).integers(0, 3, 6000).astype(np.uint8)),
                     M=np.array([28.0, 29.0, 30.0]), Q=[power_Q(1.0), power_Q(1.5), power_Q(2.5)],
                     grid=(2000.0, 0.001, 30001), cond=(1500.0, 0.8, 0.1)),
    # low pressure, coarse step: folded Voigt terms active
    "folding": dict(lines=lambda: S.uniform_lines(2000, 2000.0, 2010.0, seed=44),
                    M=28.0, Q=None, grid=(2000.0, 0.02, 501), cond=(1500.0, 0.02, 0.3)),
}


def q_of(Q, T, n_iso):
    if Q is None:
        return 1.0
    return np.array([f(TREF) / f(T) for f in Q])


def oracle_A(case, lines, T, p, x, axes, n_ft):
    vmin, dv, n_v = case["grid"]
    n_iso = len(np.atleast_1d(case["M"]))
    return O.synthesize(lines, T, p, x, vmin, dv, n_v, axes, n_ft, Qref_Qgas=q_of(case["Q"], T, n_iso),
                        molar_mass=case["M"], fft_workers=WORKERS)


def fd_columns(case, lines, axes, n_ft):
    T, p, x = case["cond"]
    cols = []
    for i in range(3):
        th = [T, p, x]
        h = REL_H * th[i]
        up, dn = list(th), list(th)
        up[i] += h
        dn[i] -= h
        cols.append((oracle_A(case, lines, *up, axes, n_ft) - oracle_A(case, lines, *dn, axes, n_ft)) / (2 * h))
    return cols


_FD = {}


# every case with the FFT-stage layout the planner picks (skeleton rows where
# the grid allows: the adjoint then expands skeleton rows in the gather, the
# tangent projects its LDM) and with node rows (layout 1)
@pytest.fixture(scope="module", params=[(name, lay) for name in sorted(CASES) for lay in (0, 1)],
                ids=lambda p: f"{p[0]}-layout{p[1]}")
def setup(request, ctx):
    name, layout = request.param
    case = CASES[name]
    lines = case["lines"]()
    vmin, dv, n_v = case["grid"]
    ln = L.Lines(ctx, lines, case["M"])
    plan = L.Plan(ln, vmin, dv, n_v, dxG=S.DXG_DEFAULT, dxL=S.DXL_DEFAULT, layout=layout)
    T, p, x = case["cond"]
    g = plan.grid(T, p, x)
    if name not in _FD:   # the oracle's columns do not depend on the layout
        _FD[name] = (fd_columns(case, lines, g.axes(), g.n_ft), oracle_A(case, lines, T, p, x, g.axes(), g.n_ft))
    fd, ref = _FD[name]
    yield name, case, plan, fd, ref
    plan.close()
    ln.close()


def test_skeleton_rows_in_some_case(ctx):
    """At least one case's grid takes the skeleton layout under the planner's
    choice, so the skeleton adjoint and tangent paths run in the tests above."""
    used = []
    for name, case in CASES.items():
        lines = case["lines"]()
        vmin, dv, n_v = case["grid"]
        ln = L.Lines(ctx, lines, case["M"])
        plan = L.Plan(ln, vmin, dv, n_v, dxG=S.DXG_DEFAULT, dxL=S.DXL_DEFAULT)
        _, info = plan.synthesize_host(*case["cond"], q_ratio=q_of(case["Q"], case["cond"][0], 0))
        used.append(int(info.layout))
        plan.close()
        ln.close()
    assert any(u in (3, 4) for u in used), used


def test_jvp_matches_fd(setup):
    from radis_gb300.autodiff import jacobian
    name, case, plan, fd, ref = setup
    T, p, x = case["cond"]
    a, dT, dp, dx = jacobian(plan, T, p, x, Q=case["Q"])
    a = a.double().cpu().numpy()
    assert np.max(np.abs(a - ref)) <= 1e-4 * np.max(np.abs(ref))
    for got, want in zip((dT, dp, dx), fd):
        got = got.double().cpu().numpy()
        assert np.max(np.abs(got - want)) <= 1e-3 * np.max(np.abs(want)), name


def test_backward_matches_fd(setup):
    name, case, plan, fd, ref = setup
    T, p, x = case["cond"]
    from radis_gb300.autodiff import _q_terms
    q, dlnq = _q_terms(case["Q"], T, plan.lines.n_iso)
    rng = np.random.default_rng(7)
    for g in (rng.uniform(0.5, 1.5, plan.n_v), rng.normal(size=plan.n_v)):
        gd = torch.tensor(g, dtype=torch.float32, device="cuda")
        got = plan.backward(T, p, x, gd.data_ptr(), q_ratio=q, dlnq_dT=dlnq)
        g64 = gd.double().cpu().numpy()
        for i in range(3):
            want = float(np.dot(g64, fd[i]))
            scale = float(np.dot(np.abs(g64), np.abs(fd[i])))
            assert abs(got[i] - want) <= 1e-3 * scale, (name, i, got[i], want)


def test_backward_equals_g_dot_jvp(setup):
    from radis_gb300.autodiff import _q_terms, jacobian
    name, case, plan, fd, ref = setup
    T, p, x = case["cond"]
    q, dlnq = _q_terms(case["Q"], T, plan.lines.n_iso)
    _, dT, dp, dx = jacobian(plan, T, p, x, Q=case["Q"])
    g = torch.tensor(np.random.default_rng(8).normal(size=plan.n_v), dtype=torch.float32, device="cuda")
    got = plan.backward(T, p, x, g.data_ptr(), q_ratio=q, dlnq_dT=dlnq)
    for i, col in enumerate((dT, dp, dx)):
        want = float(torch.dot(g.double(), col.double()))
        scale = float(torch.dot(g.double().abs(), col.double().abs()))
        assert abs(got[i] - want) <= 2e-4 * scale, (name, i)


def test_autograd_function(setup):
    from radis_gb300.autodiff import absorbance
    name, case, plan, fd, ref = setup
    T0, p0, x0 = case["cond"]
    Lp = 2.5
    T = torch.tensor(T0, dtype=torch.float64, requires_grad=True)
    p = torch.tensor(p0, dtype=torch.float64, requires_grad=True)
    x = torch.tensor(x0, dtype=torch.float64, requires_grad=True)
    A = absorbance(plan, T, p, x, path_length=Lp, Q=case["Q"])
    assert A.shape == (plan.n_v,) and A.is_cuda
    assert np.max(np.abs(A.detach().double().cpu().numpy() - Lp * ref)) <= 1e-4 * Lp * np.max(np.abs(ref))
    w = torch.tensor(np.random.default_rng(9).uniform(0.0, 1.0, plan.n_v), dtype=torch.float32, device="cuda")
    (A * w).sum().backward()
    w64 = w.double().cpu().numpy()
    for t, col in zip((T, p, x), fd):
        want = Lp * float(np.dot(w64, col))
        scale = Lp * float(np.dot(np.abs(w64), np.abs(col)))
        assert t.grad is not None and t.grad.dtype == torch.float64
        assert abs(float(t.grad) - want) <= 1e-3 * scale, name
