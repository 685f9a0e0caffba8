"""The continuous-batching server (rg_server_*): each result is the same alone
and in the mix, admission under a memory budget, and request errors."""
import numpy as np
import pytest

from radis_gb300 import _lib as L
from radis_gb300 import synthetic as S

# a hard per-test limit that also ends a test blocked inside a native call
pytestmark = [pytest.mark.gpu, pytest.mark.timeout(240, method="thread")]
TOL = 1e-4


@pytest.fixture(scope="module")
def env(native_lib):
    ctx = L.Context(0)
    co = L.Lines(ctx, S.co_like(), 28.0)
    co2 = L.Lines(ctx, S.uniform_lines(500_000, 2000.0, 2400.0, seed=52), 44.0)
    yield ctx, co, co2
    ctx.close()


def mix(co, co2, n=24, seed=7):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        lines, lo, hi = (co, 1900.0, 2300.0) if i % 2 else (co2, 2000.0, 2400.0)
        dv = float(rng.choice([0.001, 0.002, 0.005, 0.01]))
        width = float(np.exp(rng.uniform(np.log(5.0), np.log(hi - lo))))
        vmin = float(np.round(rng.uniform(lo, hi - width) / dv) * dv)
        n_v = int(width / dv) + 1
        T = float(np.exp(rng.uniform(np.log(300), np.log(3000))))
        p = float(np.exp(rng.uniform(np.log(0.1), np.log(10))))
        x = float(np.exp(rng.uniform(np.log(0.01), np.log(1.0))))
        reqs.append((lines, vmin, dv, n_v, T, p, x))
    return reqs


def alone(r):
    lines, vmin, dv, n_v, T, p, x = r
    plan = L.Plan(lines, vmin, dv, n_v, dxG=S.DXG_DEFAULT, dxL=S.DXL_DEFAULT)
    out, info = plan.synthesize_host(T, p, x)
    plan.close()
    return out.astype(np.float64) * np.exp(info.log_scale)


def test_same_alone_and_in_the_mix(env):
    ctx, co, co2 = env
    reqs = mix(co, co2)
    srv = L.Server(ctx, slots=6, mem_budget=8 << 30)
    tickets = [srv.submit(*r, dxG=S.DXG_DEFAULT, dxL=S.DXL_DEFAULT) for r in reqs]
    for r, t in zip(reqs, tickets):
        out, info, (ts, t0, t1) = srv.wait(t, timeout_ms=60000)
        assert ts <= t0 <= t1
        got = out.astype(np.float64) * np.exp(info.log_scale)
        ref = alone(r)
        assert np.max(np.abs(got - ref)) <= TOL * max(np.max(np.abs(ref)), 1e-300)
    st = srv.stats()
    assert st.completed == len(reqs) and st.failed == 0 and st.in_flight == 0
    srv.close()


def test_page_locked_request_buffers(env):
    """Page-locked request buffers are written by the last kernel directly;
    pageable ones through the slot's staging buffer: the same spectra, and the
    worker copies only the pageable ones."""
    import torch
    ctx, co, co2 = env
    reqs = mix(co, co2, n=12, seed=11)
    srv = L.Server(ctx, slots=4, mem_budget=8 << 30)
    pinned = [torch.full((r[3],), np.nan, dtype=torch.float32, pin_memory=True).numpy() for r in reqs]
    tickets = [srv.submit(*r, out=(pinned[i] if i % 2 else None), dxG=S.DXG_DEFAULT, dxL=S.DXL_DEFAULT)
               for i, r in enumerate(reqs)]
    for i, (r, t) in enumerate(zip(reqs, tickets)):
        out, info, _ = srv.wait(t, timeout_ms=60000)
        if i % 2:
            assert out is pinned[i]
        got = out.astype(np.float64) * np.exp(info.log_scale)
        ref = alone(r)
        assert np.all(np.isfinite(got))
        assert np.max(np.abs(got - ref)) <= TOL * max(np.max(np.abs(ref)), 1e-300)
    st = srv.stats()
    assert st.completed == len(reqs) and st.failed == 0
    srv.close()
    # all page-locked: the worker copies nothing
    srv = L.Server(ctx, slots=4, mem_budget=8 << 30)
    tickets = [srv.submit(*r, out=pinned[i], dxG=S.DXG_DEFAULT, dxL=S.DXL_DEFAULT) for i, r in enumerate(reqs)]
    for t in tickets:
        srv.wait(t, timeout_ms=60000)
    assert srv.stats().host_copy_ms == 0.0
    srv.close()


def test_budget_admission_and_errors(env):
    ctx, co, co2 = env
    # a budget that fits one mid-size request at a time: the queue drains in order
    srv = L.Server(ctx, slots=4, mem_budget=400 << 20)
    reqs = [(co2, 2000.0 + 20 * i, 0.001, 20001, 800.0 + 50 * i, 1.0, 0.1) for i in range(6)]
    tickets = [srv.submit(*r, n_G=6, n_L=10) for r in reqs]
    for r, t in zip(reqs, tickets):
        out, info, _ = srv.wait(t, timeout_ms=60000)
        lines, vmin, dv, n_v, T, p, x = r
        plan = L.Plan(lines, vmin, dv, n_v, n_G=6, n_L=10)
        ref, ri = plan.synthesize_host(T, p, x)
        plan.close()
        assert np.max(np.abs(out - ref)) <= TOL * np.max(np.abs(ref))
    assert srv.stats().device_bytes <= 400 << 20
    # larger than the whole budget: fails with RG_ERR_OOM, the server keeps running
    t = srv.submit(co2, 2000.0, 0.001, 400001, 1000.0, 1.0, 0.1, n_G=16, n_L=32)
    with pytest.raises(L.RgError) as e:
        srv.wait(t, timeout_ms=60000)
    assert e.value.code == 3
    t = srv.submit(co, 1900.0, 0.01, 1001, 500.0, 1.0, 0.1, dxG=S.DXG_DEFAULT, dxL=S.DXL_DEFAULT)
    srv.wait(t, timeout_ms=60000)
    # malformed requests are rejected at submission
    with pytest.raises(L.RgError):
        srv.submit(co, 1900.0, -0.01, 1001, 500.0, 1.0, 0.1, dxG=0.1, dxL=0.1)
    with pytest.raises(L.RgError):
        srv.submit(co, 1900.0, 0.01, 1001, 500.0, 1.0, 0.1)   # no node policy
    srv.close()
