"""Host-side logic on CPU: the reference-interface mirror, the workload
generator, and the multi-process replica path (gloo, world size 2)."""
import os

import numpy as np
import pytest

from aphros_gb300 import linear, workload


def test_registry_mirrors_linsolver_symm():
    for name in ("gpu_cg", "gpu", "gpu_mixed"):
        assert linear.ModuleLinear.GetInstance(name) is not None
    assert linear.ModuleLinear.GetInstance("conjugate") is None
    var = {"linsolver_symm": "gpu_mixed", "hypre_symm_tol": "1e-8",
           "hypre_symm_maxiter": "50", "linsolver_symm_maxnorm": "1",
           "gpu_symm_mg_pre": "3", "gpu_symm_inner_rtol": "1e-3",
           "gpu_symm_cycle": "1", "gpu_symm_sweep_growth": "3"}
    s = linear.MakeLinearSolver(var, "symm", linear.Mesh(16, 1 / 16))
    assert isinstance(s, linear.SolverGpu)
    assert s.kind == "gpu_mixed"
    assert s.GetConf().tol == 1e-8 and s.GetConf().maxiter == 50
    assert s.GetConf().miniter == 0  # ModuleLinear::GetConf default
    assert s.residual_max
    assert s.mg == {"mg_pre": 3, "inner_rtol": 1e-3}
    assert s.options == {"cycle": 1, "sweep_growth": 3}
    with pytest.raises(RuntimeError):
        linear.MakeLinearSolver({"linsolver_symm": "hypre"}, "symm", None)


def test_generator_is_deterministic():
    a = workload.tg_flux(16, seed=1)
    b = workload.tg_flux(16, seed=1)
    c = workload.tg_flux(16, seed=2)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, c)
    # noise has the requested spread: flux/area - TG ~ N(0, 0.01)
    h = 1 / 16
    z = workload.tg_flux(16, noise=0.0, seed=1)
    noise = (a - z) / (h * h)
    assert abs(noise.std() - 0.01) < 0.001


def test_taylor_green_is_discretely_divergence_free():
    n = 16
    f = workload.tg_flux(n, noise=0.0).reshape(3, n, n, n)  # [d, k, j, i]
    div = (np.roll(f[0], -1, axis=2) - f[0] + np.roll(f[1], -1, axis=1) - f[1]
           + np.roll(f[2], -1, axis=0) - f[2])
    assert np.max(np.abs(div)) < 1e-15


def test_sphere_volume_and_periodic_images():
    a = workload.alpha_spheres(32, [[0.5, 0.5, 0.5]], [0.2])
    assert abs(a.sum() / 32 ** 3 - 4 / 3 * np.pi * 0.2 ** 3) < 1e-13
    b = workload.alpha_spheres(32, [[0.01, 0.98, 0.5]], [0.2])
    assert abs(b.sum() - a.sum()) < 1e-10
    assert a.min() >= 0 and a.max() <= 1


def test_sphere_placement_does_not_overlap():
    c, r = workload.place_spheres(2, 16, 0.03, 0.08)
    assert len(r) == 16
    for i in range(16):
        for j in range(i):
            d = np.abs(c[i] - c[j])
            d = np.minimum(d, 1 - d)
            assert np.linalg.norm(d) >= r[i] + r[j]


def test_batch_and_served_shapes():
    cases = workload.batch_cases(64)
    assert {c.n for c in cases} <= {32, 48, 64, 96}
    assert all(10 - 1e-9 <= c.rho1 / c.rho2 <= 1000 + 1e-6 for c in cases)
    served = workload.served_cases(100)
    assert all(32 <= c.n <= 128 and c.n % 16 == 0 for c in served)
    assert len({c.n for c in served}) >= 5


def _replica_worker(rank, world, port, q):
    import time

    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    import oracle
    units, secs = bench.replica_share(rank, world, 10)
    agg = bench.aggregate_over_ranks(units, 1.0 + rank)
    # each rank solves its own share of independent systems (the replicas'
    # work, here by the oracle CG on the host): no data crosses ranks, and
    # the job's value is all ranks' solves over the slowest rank's time
    t0 = time.perf_counter()
    solved = 0
    for u in range(units):
        case = workload.config("c1", n=12)
        e, _, _ = oracle.assemble_projection(12, case.h, case.dt, case.alpha, case.rho1,
                                             case.rho2, case.flux)
        _, info = oracle.cg_solve(12, case.h, e, oracle.rel_tol(e, case.h, 1e-10))
        solved += int(info.residual < oracle.rel_tol(e, case.h, 1e-10))
    work = bench.aggregate_over_ranks(solved, time.perf_counter() - t0)
    q.put((rank, units, agg, work[0]))
    dist.destroy_process_group()


def test_replicas_over_gloo():
    """N>1 runs independent replicas: each rank gets its share of units,
    solves them without exchanging data, and the job value is total units /
    max time over ranks."""
    import multiprocessing as mp
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_replica_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][1] + res[1][1] == 10
    total_units, max_time = res[0][2]
    assert total_units == 10 and max_time == 2.0
    assert res[1][2] == res[0][2]
    # every unit of every rank was solved, and both ranks see the job total
    assert res[0][3] == 10 and res[1][3] == 10


def test_reference_arm_prints_the_contract_line():
    """`bench.py --impl reference` (the oracle's CG on the host cores, no
    GPU) prints one JSON line with the benchmark contract's keys."""
    import json
    import subprocess
    import sys
    from conftest import ROOT
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0", "--cpu-budget", "2"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "impl", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["warmup"] >= 3
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    assert "workload" in line["config"]
    for key in ("value", "unit", "cores", "kind", "sample"):
        assert key in line["cpu_baseline"], key
