"""bench.py's reference arm on the host (no GPU): one JSON line with the
keys of the benchmark line, timing the oracle on a bounded sample."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_json_line(built):
    env = dict(os.environ, RANK="0")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ["impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"]:
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "evals/s"
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert "workload" in d["config"]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.max_over_ranks(10.0 + rank, world, "cpu")  # rank 1 is the slower one
    q.put((rank, ms, bench.job_rate(world, 100, ms)))
    dist.barrier()
    dist.destroy_process_group()


def test_multi_rank_timing_takes_the_slowest_rank():
    """world_size 2 over gloo: both ranks see the slower rank's time, and the
    job rate counts both ranks' work (replicas, weak scaling)."""
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [11.0, 11.0]
    assert all(abs(o[2] - 2 * 100 / 0.011) < 1e-6 for o in out)


def test_cpu_chain_step_runs_the_oracle_chain(built):
    """The CPU chain-step baseline on a small membrane: HMC moves and
    parallel flip sweeps of the oracle, a finite rate and a valid
    acceptance."""
    sys.path.insert(0, ROOT)
    import bench
    from trimem_gb300 import meshgen
    from trimem_gb300.workloads import workload_params

    p, f = meshgen.jittered_icosphere(2, seed=0)
    prm = dict(workload_params(p, f, kappa_b=20.0), cont_lambda=0.0)
    out = bench.cpu_chain_step({"x": p, "faces": f, "prm": prm}, n_steps=2, n_leapfrog=3, dt=1e-6)
    assert out["steps"] == 2 and out["steps_per_s"] > 0
    assert 0.0 <= out["acceptance"] <= 1.0 and out["flips_accepted_per_sweep"] >= 0
    assert out["kind"] == "port" and out["cores"] >= 1
