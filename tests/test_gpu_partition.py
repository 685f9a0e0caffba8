"""Partition-function tables held by a line list (rg_lines_set_partition):
with q_ratio = NULL the library takes Q(Tref)/Q(T) from the tables, and the
adjoint takes d ln(Q(Tref)/Q(T))/dT from them.  Checked against the same
ratios passed explicitly (identical results), against the FP64 oracle
(1e-4 of the peak, as every spectrum test), and through gpuApp with
TabulatedQ callables.  Tables: the CDSD CO2 columns of the golden file
(the reference's radis/db/CO2/partition_functions.txt)."""
import os

import numpy as np
import pytest

from oracle import ldm_oracle as O
from radis_gb300 import _lib as L
from radis_gb300 import synthetic as S
from radis_gb300.partition import TabulatedQ

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_partition.npz"))
TABS = [TabulatedQ(G["cdsd_T"], G[f"cdsd_Q{i}"], kind="cubic") for i in (1, 2, 3)]


@pytest.fixture(scope="module")
def ctx(native_lib):
    c = L.Context(0)
    yield c
    c.close()


def _lines():
    d = S.uniform_lines(6000, 2000.0, 2030.0, seed=42)
    d["iso"] = np.random.default_rng(43).integers(0, 3, 6000).astype(np.uint8)
    return d


def test_tables_drive_q_ratio_and_its_derivative(ctx):
    lines = _lines()
    M = np.array([44.0, 45.0, 46.0])
    ln = L.Lines(ctx, lines, M)
    plan = L.Plan(ln, 2000.0, 0.001, 30001, dxG=S.DXG_DEFAULT, dxL=S.DXL_DEFAULT)
    T, p, x = 1500.0, 0.8, 0.1
    q = np.array([t(296.0) / t(T) for t in TABS])
    dlnq = np.array([-t.dQ_dT(T) / t(T) for t in TABS])
    a_explicit, _ = plan.synthesize_host(T, p, x, q_ratio=q)
    a_one, _ = plan.synthesize_host(T, p, x)          # no tables yet: ratio 1
    for i, t in enumerate(TABS):
        ln.set_partition(i, t.T, t.Q, "cubic")
    a_tab, info = plan.synthesize_host(T, p, x)       # ratio from the tables
    assert np.array_equal(a_tab, a_explicit)
    assert not np.array_equal(a_one, a_explicit)
    g = plan.grid(T, p, x)
    ref = O.synthesize(lines, T, p, x, 2000.0, 0.001, 30001, g.axes(), g.n_ft, Qref_Qgas=q, molar_mass=M,
                       fft_workers=os.cpu_count() or 1)
    got = a_tab.astype(np.float64) * np.exp(info.log_scale)
    assert np.max(np.abs(got - ref)) <= 1e-4 * np.max(np.abs(ref))
    w = torch.tensor(np.random.default_rng(3).normal(size=30001), dtype=torch.float32, device="cuda")
    d_tab = plan.backward(T, p, x, w.data_ptr())
    d_exp = plan.backward(T, p, x, w.data_ptr(), q_ratio=q, dlnq_dT=dlnq)
    # the adjoint's FP64 cross-block sums are atomic: equal up to summation order
    assert np.allclose(d_tab, d_exp, rtol=1e-10, atol=0.0)
    with pytest.raises(L.RgError) as e:     # beyond 1.05 x the table's 6000 K
        plan.synthesize_host(7000.0, p, x)
    assert e.value.code == 5
    plan.close()
    ln.close()


def test_gpuapp_with_tabulated_q(native_lib):
    from radis_gb300.gpu import gpuApp

    lines = _lines()
    n = len(lines["v0"])
    iso = lines["iso"].astype(np.int64) + 1          # gpuApp slots: Mm_arr[0] unused
    Mm = np.array([0.0, 44.0, 45.0, 46.0])
    tabs = [TABS[0]] + TABS
    args = (2000.0, 30001, 0.001, S.DXG_DEFAULT, S.DXL_DEFAULT, lines["v0"], np.zeros(n, np.float32),
            lines["n_air"], None, lines["El"], np.vstack([lines["g_self"], lines["g_air"]]), iso, Mm)
    app_tab = gpuApp(*args, tabs, S_ref=lines["S_ref"])
    app_fn = gpuApp(*args, [lambda T, t=t: t(T) for t in tabs], S_ref=lines["S_ref"])
    try:
        assert app_tab._q_in_lib and not app_fn._q_in_lib
        a, _ = app_tab.iterate(0.8, 1500.0, 0.1)
        b, _ = app_fn.iterate(0.8, 1500.0, 0.1)
        assert np.array_equal(a, b)
    finally:
        app_tab.free()
        app_fn.free()
