"""bench.py's launch contract on the CPU.

* The reference arm under torchrun with two ranks (127.0.0.1, gloo-free: the
  arm needs no process group): rank 0 alone times the reference algorithm on
  the host cores and prints one JSON line carrying impl, cpu_baseline and an
  e2e object with zero copy bytes; the other rank exits 0 without work.
* The kernel-launch claim (gpu_launches = kernels per spectrum x steps) for
  the plain, merged, merged-with-narrow-rows and skeleton FFT layouts.
* The multi-rank timing reduction of the GPU arm (max over ranks) on two
  gloo ranks.
* The host-only ingestion mode (--ingest-only) on a small file.
* The reference arm runs without this library: after a whole run in one
  process no module of the package is imported and libradisgb.so is not
  mapped; its config equals the GPU arm's description of the workload.
* The oracle's node-axis rule (used by the reference arm) equals the
  library's hull-based grid on the bench workloads' kind of list.
"""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_reference_arm_two_ranks():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py",
           "--impl", "reference", "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    out = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(out) == 1, r.stdout[-2000:]
    d = json.loads(out[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    sys.path.insert(0, ROOT)
    import bench
    assert d["config"] == bench.workload_desc("co2_5M", 5_000_000, 400001, 28)


def test_reference_arm_loads_nothing_of_the_library():
    code = (
        "import sys, runpy\n"
        "sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0']\n"
        "try:\n"
        "    runpy.run_path('bench.py', run_name='__main__')\n"
        "except SystemExit as e:\n"
        "    assert not e.code, e.code\n"
        "mods = [m for m in sys.modules if m == 'radis_gb300' or m.startswith('radis_gb300.')]\n"
        "assert not mods, mods\n"
        "assert 'libradisgb' not in open('/proc/self/maps').read()\n"
        "print('REFERENCE_ARM_CLEAN')\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    assert "REFERENCE_ARM_CLEAN" in r.stdout


def test_oracle_axes_equal_library_grid(native_lib):
    """The reference arm takes its node axes from the oracle's brute-force
    envelope rule; the GPU arm from the library's hulls: the same axes."""
    sys.path.insert(0, ROOT)
    from oracle import ldm_oracle as O
    from radis_gb300 import _lib as L
    from radis_gb300 import synthetic as S
    for lines, M, vmin, dv, n_v, T, p, x, nG, nL in (
            (S.co2_like(200_000, seed=9), 44.0, 2000.0, 0.001, 400001, 1500.0, 1.0, 0.1, 8, 16),
            (S.h2o_like(300_000, seed=9), 18.0, 500.0, 0.005, 1500001, 2000.0, 1.0, 0.2, 12, 24)):
        g = L.grid_estimate(lines, M, vmin, dv, n_v, T, p, x, n_G=nG, n_L=nL)
        ax = O.envelope_axes(lines, T, p, x, NG=nG, NL=nL, molar_mass=M)
        assert (ax[2], ax[5]) == (g.n_G, g.n_L)
        for a, b in zip((ax[0], ax[1], ax[3], ax[4]), (g.log_wG_min, g.dxG, g.log_wL_min, g.dxL)):
            assert abs(a - b) <= 1e-12 * max(1.0, abs(b))


def test_kernels_per_step():
    sys.path.insert(0, ROOT)
    import bench

    class Info:
        def __init__(self, merged_rows, fft_rows, layout=None):
            self.merged_rows, self.fft_rows = merged_rows, fft_rows
            self.layout = layout if layout is not None else (2 if merged_rows else 1)

    # up to 32 FFT rows the inverse row DFT runs inside the row kernel
    assert bench.kernels_per_step(Info(0, 128)) == 5     # plain layout
    assert bench.kernels_per_step(Info(0, 12, 3)) == 5   # skeleton rows: the projection in addition
    assert bench.kernels_per_step(Info(0, 12, 4)) == 4   # projected in the scatter's flush
    assert bench.kernels_per_step(Info(0, 40, 3)) == 6   # more rows: separate inverse row DFT
    assert bench.kernels_per_step(Info(16, 16)) == 5     # CO2 5M: all Gaussian nodes wide
    assert bench.kernels_per_step(Info(24, 216)) == 7    # H2O 100M: merged + narrow-node rows
    assert bench.kernels_per_step(Info(7, 8)) == 5       # odd n_L padded with a zero row
    assert bench.kernels_per_step(Info(7, 16)) == 6


def _max_worker(rank, port, q):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=2)
    try:
        q.put((rank, bench.max_over_ranks(1.5 + rank, 2, "cpu"), bench.max_over_ranks(7.0, 1, "cpu")))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo_two_ranks():
    """The multi-rank timing reduction of bench.py (the slowest rank's time)
    on two gloo ranks: every rank gets the max; one rank is a no-op."""
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_max_worker, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert got == [(0, 2.5, 7.0), (1, 2.5, 7.0)]


def test_ingest_mode():
    """bench.py --ingest-only: the host-side HITRAN-160 ingestion line (no GPU)."""
    r = subprocess.run([sys.executable, "bench.py", "--ingest-only", "--ingest-records", "20000"], cwd=ROOT,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    d = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])
    assert d["records"] == 20000 and d["bytes"] == 20000 * 161 and d["bit_exact_vs_baseline"] is True
    assert d["value"] > 0 and d["cpu_baseline"]["kind"] == "port" and d["cache"]["cached_load_ms"] > 0
