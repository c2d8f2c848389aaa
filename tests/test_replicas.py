"""Multi-process (gloo, world size 2, CPU) checks of the replica logic: track
sharding covers every track exactly once with balanced work, the timing
collectives take the max of the per-rank times and the sum of the units, and the
reference arm's non-zero ranks exit without work."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    from mkfbodytracker_pdaf_gb300 import replicas
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        costs = np.random.default_rng(0).integers(100, 10000, 97)
        mine = replicas.shard_by_work(costs, world)[rank]
        units = float(sum(costs[i] for i in mine))
        secs = 1.0 + rank                     # rank 1 is the slow one
        out = {"rank": rank, "mine": mine, "env": replicas.dist_env(),
               "tmax": replicas.max_over_ranks(secs), "usum": replicas.sum_over_ranks(units),
               "rate": replicas.whole_job_rate(units, secs)}
        ids = dist_all_gather(dist, mine, world)
        out["all"] = ids
        q.put(out)
    finally:
        dist.destroy_process_group()


def dist_all_gather(dist, obj, world):
    res = [None] * world
    dist.all_gather_object(res, obj)
    return res


def test_gloo_two_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    outs = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    costs = np.random.default_rng(0).integers(100, 10000, 97)
    total = float(costs.sum())
    for o in outs:
        assert o["env"] == (2, o["rank"], o["rank"])
        assert o["tmax"] == 2.0
        assert o["usum"] == total
        assert abs(o["rate"] - total / 2.0) < 1e-9
        flat = sorted(i for s in o["all"] for i in s)
        assert flat == list(range(97))
        loads = [float(sum(costs[i] for i in s)) for s in o["all"]]
        assert max(loads) - min(loads) <= costs.max()


def test_shard_by_work_single_and_many():
    from mkfbodytracker_pdaf_gb300.replicas import shard_by_work, rank_seed, whole_job_rate
    assert shard_by_work([3, 1, 2], 1) == [[0, 1, 2]]
    s = shard_by_work([5, 5, 5, 5], 4)
    assert sorted(len(x) for x in s) == [1, 1, 1, 1]
    assert shard_by_work([], 3) == [[], [], []]
    with pytest.raises(ValueError):
        shard_by_work([1], 0)
    assert rank_seed(10, 0) == 10 and rank_seed(10, 3) == 3010
    assert whole_job_rate(100.0, 2.0) == 50.0          # no process group: this rank alone


def test_reference_arm_nonzero_rank_exits_without_work(monkeypatch, capsys):
    import importlib.util
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(root, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    sys.modules["bench_mod"] = bench
    spec.loader.exec_module(bench)
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    args = bench.parse_args(["--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3"])
    assert bench.run_reference(args) is None
    assert capsys.readouterr().out == ""


def test_reference_arm_json_line_on_cpu(monkeypatch, capsys):
    """The reference arm (the oracle on the host cores) prints the bench
    contract's line: impl, metric, value, e2e with zero copies, cpu_baseline."""
    import importlib.util
    import json
    import sys
    from mkfbodytracker_pdaf_gb300 import synth
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("bench_ref", os.path.join(root, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    sys.modules["bench_ref"] = bench
    spec.loader.exec_module(bench)
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    small = synth.make_bpf_batch(7, [64, 100, 150], [5, 3, 4], [2.0, 3.0, 1.0], [0.9, 0.8, 0.95])
    monkeypatch.setattr(bench, "workload", lambda rank, n: small)
    args = bench.parse_args(["--impl", "reference", "--steps", "2", "--warmup", "3", "--cpu-sample-tracks", "2"])
    bench.run_reference(args)
    lines = [ln for ln in capsys.readouterr().out.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["value"] > 0 and d["steps"] == 2 and d["warmup"] == 3 and d["higher_is_better"] is True
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"]
    assert d["config"]["tracks_per_step"] == 2


def test_cpu_baseline_record_on_cpu():
    """The cpu_baseline object of the GPU arm's line, from the oracle on a fixed sample."""
    import importlib.util
    import sys
    from mkfbodytracker_pdaf_gb300 import synth
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("bench_cb", os.path.join(root, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    sys.modules["bench_cb"] = bench
    spec.loader.exec_module(bench)
    small = synth.make_bpf_batch(8, [64, 80, 96, 50], [4, 3, 5, 2], [2.0, 3.0, 1.0, 0.5], [0.9, 0.8, 0.95, 0.9])
    cb = bench.cpu_baseline(small, 3, 2)
    assert cb["value"] > 0 and cb["unit"] == bench.UNIT and cb["cores"] == 2 and cb["kind"] == "port"
    assert cb["sample"].startswith("3 fixed tracks")
    # the sample runs longest first (particle-frames), the same one in both arms
    ids = bench.sample_ids(small, 3)
    cost = [small.tracks[b]["n_particles"] * small.tracks[b]["n_frames"] for b in ids]
    assert cost == sorted(cost, reverse=True)
    acc = bench.accuracy_tracks(small, bench.sample_ids(small, 4))
    assert len(acc) == len(set(acc)) and 1 <= len(acc) <= 4
    assert max(small.tracks[b]["n_frames"] for b in acc) == max(t["n_frames"] for t in small.tracks)
