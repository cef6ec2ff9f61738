"""The N > 1 path of bench.py on CPU: two ranks over gloo.

Each rank is an independent replica (no data-path collective); the only
cross-rank operation is the max over ranks of the timed region, from which
the whole-job throughput is formed.  The reference arm runs on rank 0 only;
the other ranks exit 0 without work or output."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, times, queue):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sys.path.insert(0, ROOT)
        import bench

        env = bench.dist_env()
        rate, slowest = bench.whole_job_rate(times[rank], 3, world, dist)
        queue.put((rank, env, rate, slowest))
    finally:
        dist.destroy_process_group()


def test_whole_job_rate_over_two_gloo_ranks():
    import torch.multiprocessing as mp

    sys.path.insert(0, ROOT)
    import bench

    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    times = [2.0, 3.5]  # seconds of the timed region on ranks 0 and 1
    procs = [ctx.Process(target=_worker, args=(r, 2, port, times, queue)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(queue.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, env, rate, slowest in results:
        assert env == (rank, 2, rank)
        assert slowest == 3.5  # the slowest rank's time, on every rank
        assert rate == pytest.approx(2 * 3 * bench.UNITS_PER_STEP / 3.5)


def test_single_rank_rate_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench

    rate, slowest = bench.whole_job_rate(250.0, 4, 1, None, per_second=1e3)
    assert slowest == 250.0
    assert rate == pytest.approx(4 * bench.UNITS_PER_STEP / 0.25)


def test_reference_arm_other_ranks_exit_quietly(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("LOCAL_RANK", "1")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1",
                                      "--warmup", "0"])
    assert bench.main() == 0
    assert capsys.readouterr().out == ""


def test_cpu_oracle_problems_rate():
    """The bench's CPU reference points: the oracle on a list of problems, one
    per host thread; the rate counts every problem's N * M * T."""
    import numpy as np

    sys.path.insert(0, ROOT)
    import bench

    rng = np.random.default_rng(5)
    probs = []
    for N, M in ((300, 3), (512, 4)):
        U = rng.uniform(0.1, 3.0, size=(N, M)).astype(np.float32)
        f = rng.normal(0, 1.5, size=(N, 3)).astype(np.float32)
        probs.append((N, M, 4, U, [(f, 2.0, 1), (f[:, :2].copy(), np.eye(M, dtype=np.float32), 1)]))
    rate, dt, n = bench.cpu_oracle_problems(probs, 2)
    assert n == 2 and dt > 0
    assert rate == pytest.approx((300 * 3 * 4 + 512 * 4 * 4) / 1e6 / dt)


def test_cpu_arms_follow_the_host_variant(monkeypatch):
    """The CPU arms run the lattice path the reference compiles on the host:
    SSE on x86-64, scalar elsewhere (aarch64)."""
    import platform

    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import bench
    import oracle as O

    monkeypatch.setattr(platform, "machine", lambda: "aarch64")
    assert bench.host_variant(O) == O.VARIANT_SCALAR and "scalar" in bench.host_variant_name()
    monkeypatch.setattr(platform, "machine", lambda: "x86_64")
    assert bench.host_variant(O) == O.VARIANT_SSE and "SSE" in bench.host_variant_name()


def test_cpu_single_core_point():
    """One solve of the bench workload on one thread, build and iterations apart."""
    sys.path.insert(0, ROOT)
    import bench
    from pydensecrf_gb300 import synthetic as S

    r = bench.cpu_single_core(S.plain_vga(0))
    assert r["cores"] == 1 and r["kind"] == "port" and r["build_ms"] > 0 and r["iteration_ms"] > 0
    total_s = (r["build_ms"] + bench.T * r["iteration_ms"]) / 1e3
    assert r["value"] == pytest.approx(bench.UNITS_PER_STEP / total_s, rel=0.01)


def test_reference_arm_line(monkeypatch, capsys):
    """The reference arm's JSON line on one rank: the contract's keys, the
    CPU sample described, and an e2e entry with no host-device traffic."""
    import json

    sys.path.insert(0, ROOT)
    import bench

    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"])
    assert bench.main() == 0
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["metric"] == bench.METRIC and line["config"]["workload"] == bench.WORKLOAD
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_solve_accuracy_figures():
    """The bench's accuracy entry: given the oracle's own float marginals
    (M x N, as the API returns them) the float error is 0, and the float64
    error is the oracle's own, well inside the 1e-4 inference tolerance."""
    import numpy as np

    sys.path.insert(0, ROOT)
    import bench
    from pydensecrf_gb300 import synthetic as S

    cfg = S.plain_vga(0)
    O = bench._oracle()
    c = O.OracleCRF(bench.W * bench.H, bench.M, O.VARIANT_SSE)
    c.set_unary(np.ascontiguousarray(cfg["U"].T))
    c.add_pairwise(O.features_gaussian_2d(bench.W, bench.H, 3.0, 3.0), 3.0)
    c.add_pairwise(O.features_bilateral_2d(cfg["img"], 80, 80, 13, 13, 13), 10.0)
    r = bench.solve_accuracy(cfg, np.ascontiguousarray(c.inference(bench.T).T))
    assert r["max_abs_vs_oracle"] == 0.0 and r["argmax_agreement_vs_oracle"] == 1.0
    assert r["max_abs_vs_fp64"] == r["oracle_vs_fp64"] < 1e-4
