"""Benchmark: track-frame updates/s of the batched bootstrap particle filter on
the batched-uneven-tracks workload (B=8192 tracks, T~U{50..2000},
N log-uniform in [128, 8192], K=15, d=12, clutter lambda~U[0,12],
P_D~U[0.7,1], FP32), synthetic and seeded.

One step = one pass of the hot path over the whole batch (every track, every
frame: propagate, PDA-clutter likelihood, weights/estimate/ESS, exact
systematic resampling).  ``value`` is device-resident throughput (inputs in
HBM before the timed region); ``e2e`` is the same through the host-buffer
C-ABI call (detections copied in, estimates/log-likelihoods/ESS/status copied
out, every step).  ``--impl reference`` times the CPU restatement of the
reference's filter on the host cores.

Launch: python bench.py [--gpus N --steps K --warmup W]; for N > 1 under
torch.distributed.run each rank runs its own batch (weak scaling, no
collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "track-frame updates/s, plain vs batched+adjoint on 1 GB300, at ≤1e-4 rel. error"
UNIT = "track-frames/s"
BYTES_PER_PF = 112          # algorithmic bytes per particle-frame (state in/out 4d+4d, logw 8, anc 8)
# DRAM bytes per particle-frame of bpf_batched_kernel measured by ncu (see
# profiles/bpf_batched_kernel_config2.md); None until a capture exists
TRAFFIC_BYTES_PER_PF = None


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, uuid=None):
        self.proc = None
        self.path = tempfile.mktemp(prefix="mkf_clocks_", suffix=".csv")
        self.uuid = uuid

    def start(self):
        cmd = ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits", "-lms", "200"]
        if self.uuid:
            cmd[1:1] = ["-i", self.uuid]
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(cmd, stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "samples": len(sm),
                "reasons": sorted(reasons)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def workload(rank, n_tracks):
    from mkfbodytracker_pdaf_gb300 import synth
    return synth.config2_batch(n_tracks=n_tracks, seed=synth.MASTER_SEED + 2 + 1000 * rank)


def pf_count(batch, ids=None):
    ids = range(batch.n_tracks) if ids is None else ids
    return int(sum(int(batch.tracks[b]["n_particles"]) * int(batch.tracks[b]["n_frames"]) for b in ids))


def sample_ids(batch, n):
    rng = np.random.default_rng(12345)
    return sorted(rng.choice(batch.n_tracks, size=min(n, batch.n_tracks), replace=False).tolist())


def cpu_run(batch, ids, threads):
    import oracle
    sub = batch.subset(ids)
    t0 = time.perf_counter()
    oracle.bpf_run_tracks(sub, list(range(len(ids))), nthreads=threads)
    dt = time.perf_counter() - t0
    return sub.n_frames_total / dt, dt, sub


def cpu_baseline(batch, n_sample, threads):
    import oracle
    oracle.build()
    ids = sample_ids(batch, n_sample)
    rate, dt, sub = cpu_run(batch, ids, threads)
    return {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d fixed tracks of the batch (%d track-frames, %.3g particle-frames), "
                      "FP64 oracle with Philox draws, OpenMP over tracks, %.1f s"
                      % (len(ids), sub.n_frames_total, pf_count(sub), dt)}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    batch = workload(0, args.tracks)
    import oracle
    oracle.build()
    ids = sample_ids(batch, args.ref_sample_tracks)
    for _ in range(args.warmup):
        cpu_run(batch, ids, threads)
    rates, times = [], []
    for _ in range(args.steps):
        r, dt, sub = cpu_run(batch, ids, threads)
        rates.append(r)
        times.append(dt)
    value = sub.n_frames_total * args.steps / sum(times)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * sum(times) / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)",
            "config": {"workload": "batched uneven tracks: B=%d, T~U{50..2000}, N log-uniform "
                                   "[128,8192], K=15, d=12; CPU sample of %d fixed tracks per step"
                                   % (args.tracks, len(ids)),
                       "tracks_per_step": len(ids), "track_frames_per_step": sub.n_frames_total},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "%d fixed tracks per step (%d track-frames), FP64 restatement of "
                                       "the reference CPU filter, OpenMP over tracks"
                                       % (len(ids), sub.n_frames_total)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def plain_rate(batch, n_tracks, max_frames):
    """The plain per-track GPU path (three launches per frame per track)."""
    import torch
    from mkfbodytracker_pdaf_gb300.filters import BootstrapParticleFilter
    ids = sample_ids(batch, n_tracks)
    J = batch.model["J"]
    tot_frames = 0
    elapsed = 0.0
    for b in ids:
        t = batch.tracks[b]
        T = min(int(t["n_frames"]), max_frames)
        g0 = int(t["frame_base"])
        lo = batch.det_off[g0 * J:(g0 + T) * J + 1].astype(np.int64)
        det = torch.from_numpy(batch.det[lo[0]:lo[-1]].copy()).cuda()
        offs = torch.from_numpy((lo - lo[0]).astype(np.int32)).cuda()
        pf = BootstrapParticleFilter(batch.model, t)
        pf.reset()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for f in range(T):
            pf.update(f, offs[f * J:], det)
        torch.cuda.synchronize()
        elapsed += time.perf_counter() - t0
        tot_frames += T
    return tot_frames / elapsed


def run_gb300(args):
    import torch
    import torch.distributed as dist
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from mkfbodytracker_pdaf_gb300 import build
    build.build()
    from mkfbodytracker_pdaf_gb300.filters import BatchedBootstrapPF

    from mkfbodytracker_pdaf_gb300.autotune import load_tuning
    tb, cps = load_tuning()
    tb = args.block_threads or tb
    cps = cps if args.ctas_per_sm is None else args.ctas_per_sm
    batch = workload(rank, args.tracks)
    runner = BatchedBootstrapPF(batch, block_threads=tb, ctas_per_sm=cps)
    det_off, det = runner.device_inputs()
    outs = runner.alloc_outputs()
    stream = torch.cuda.current_stream()
    G = batch.n_frames_total
    PF = pf_count(batch)

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            dist.barrier()

    # ---- device-resident throughput
    for _ in range(args.warmup):
        runner.run(det_off, det, outs)
    barrier()
    uuid = None
    try:
        uuid = str(torch.cuda.get_device_properties(local).uuid)
        uuid = uuid if uuid.startswith("GPU-") else "GPU-" + uuid
    except Exception:
        uuid = None
    sampler = ClockSampler(uuid)
    sampler.start()
    time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    e0.record(stream)
    for _ in range(args.steps):
        runner.run(det_off, det, outs)
    e1.record(stream)
    barrier()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1) / args.steps
    t_local = ms / 1000.0
    if ws > 1:
        t = torch.tensor([t_local], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_local = float(t.item())
    value = G * ws / t_local
    st = outs[3].cpu().numpy()
    est_ok = bool(torch.isfinite(outs[0]).all().item())

    # ---- end-to-end through the host-buffer C ABI
    h_off = torch.from_numpy(batch.det_off.astype(np.int32)).pin_memory()
    h_det = torch.from_numpy(batch.det.astype(np.float32)).pin_memory()
    h_est = torch.empty((G, batch.model["d"]), dtype=torch.float32).pin_memory()
    h_ll = torch.empty(G, dtype=torch.float32).pin_memory()
    h_ess = torch.empty(G, dtype=torch.float32).pin_memory()
    h_st = torch.empty(batch.n_tracks, dtype=torch.int32).pin_memory()
    hbufs = [x.numpy() for x in (h_off, h_det, h_est, h_ll, h_ess, h_st)]
    for _ in range(args.warmup):
        runner.run_host(hbufs[0], hbufs[1], hbufs[2:])
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        runner.run_host(hbufs[0], hbufs[1], hbufs[2:])
    barrier()
    t_e2e = (time.perf_counter() - t0) / args.steps
    if ws > 1:
        t = torch.tensor([t_e2e], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_e2e = float(t.item())
    h2d = hbufs[0].nbytes + hbufs[1].nbytes
    d2h = sum(h.nbytes for h in hbufs[2:])

    if rank == 0:
        peak, peak_kind = load_peaks()
        achieved = BYTES_PER_PF * PF / t_local / 1e9
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator, no dataset)",
            "config": {"workload": "batched uneven tracks: B=%d, T~U{50..2000}, N log-uniform [128,8192], "
                                   "K=15, d=12, lambda~U[0,12], P_D~U[0.7,1]" % args.tracks,
                       "tracks_per_gpu": batch.n_tracks, "track_frames_per_gpu": G,
                       "particle_frames_per_gpu": PF,
                       "l2": "inputs larger than L2 (%.2f GB of detections per step)" % (h2d / 1e9),
                       "block_threads": runner.block_threads, "ctas_per_sm": runner.ctas_per_sm,
                       "parallelism": "one persistent kernel per GPU; tracks sharded by rank"},
            "e2e": {"value": G * ws / t_e2e, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": args.steps,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind,
                         "traffic": (TRAFFIC_BYTES_PER_PF * PF) if TRAFFIC_BYTES_PER_PF else None,
                         "kernel": "bpf_batched_kernel",
                         "algorithmic_bytes_per_launch": BYTES_PER_PF * PF},
            "clocks": clocks,
            "status_ok": bool(((st & ~8) == 0).all()) and est_ok,
        }
        if not args.no_plain:
            pr = plain_rate(batch, args.plain_tracks, args.plain_frames)
            line["plain_path"] = {"value": pr, "unit": UNIT,
                                  "sample": "%d tracks x <=%d frames through mkf_bpf_update" %
                                            (args.plain_tracks, args.plain_frames),
                                  "batched_over_plain": value / ws / pr}
        if not args.no_cpu:
            line["cpu_baseline"] = cpu_baseline(batch, args.cpu_sample_tracks, os.cpu_count() or 1)
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--tracks", type=int, default=8192)
    ap.add_argument("--block-threads", type=int, default=None, help="default: autotuned choice")
    ap.add_argument("--ctas-per-sm", type=int, default=None)
    ap.add_argument("--cpu-sample-tracks", type=int, default=24)
    ap.add_argument("--ref-sample-tracks", type=int, default=16)
    ap.add_argument("--plain-tracks", type=int, default=8)
    ap.add_argument("--plain-frames", type=int, default=300)
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
