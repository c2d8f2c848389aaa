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
# DRAM bytes per particle-frame of bpf_batched_kernel (autotuned shape: 256
# threads x 3 CTAs/SM, float4 loads + search with ancestors in global memory):
# dram__bytes_read.sum + dram__bytes_write.sum of one ncu capture on 2048
# tracks of the same workload (261.5 GB over 4.148e9 particle-frames), scaled
# to a full launch by particle-frames
TRAFFIC_BYTES_PER_PF = 63.0
# warp instructions issued per particle-frame by the same kernel (smsp__inst_executed.sum
# of the same capture: 1.0040e11 over 4.148e9 particle-frames); with the SM count, the
# four schedulers of an SM and the sampled SM clock it gives the issue roofline, the
# bound this kernel actually meets
WARP_INST_PER_PF = 24.20


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
    from mkfbodytracker_pdaf_gb300.replicas import dist_env as env
    return env()


def workload(rank, n_tracks):
    from mkfbodytracker_pdaf_gb300 import synth
    from mkfbodytracker_pdaf_gb300.replicas import rank_seed
    return synth.uneven_tracks_batch(n_tracks=n_tracks, seed=rank_seed(synth.MASTER_SEED + 2, rank))


def pf_count(batch, ids=None):
    ids = range(batch.n_tracks) if ids is None else ids
    return int(sum(int(batch.tracks[b]["n_particles"]) * int(batch.tracks[b]["n_frames"]) for b in ids))


def sample_ids(batch, n):
    """n fixed tracks of the batch, longest (particle-frames) first: the CPU
    runs them with dynamic scheduling over tracks, so that order keeps every
    host core busy to the end (longest-processing-time-first)."""
    rng = np.random.default_rng(12345)
    ids = rng.choice(batch.n_tracks, size=min(n, batch.n_tracks), replace=False).tolist()
    cost = lambda b: int(batch.tracks[b]["n_particles"]) * int(batch.tracks[b]["n_frames"])
    return sorted(ids, key=lambda b: (-cost(b), b))


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
                      "FP64 oracle with Philox draws, OpenMP over tracks (longest first), %.1f s"
                      % (len(ids), sub.n_frames_total, pf_count(sub), dt)}


def accuracy_tracks(batch, ids, n=4):
    """Tracks of the CPU sample whose full horizon is replayed in FP64: the
    longest, the one with the most particle-frames, the most particles, and
    the fewest particles among the longer half."""
    T = {b: int(batch.tracks[b]["n_frames"]) for b in ids}
    N = {b: int(batch.tracks[b]["n_particles"]) for b in ids}
    picks = [max(ids, key=lambda b: (T[b], N[b])), max(ids, key=lambda b: (N[b] * T[b], b)),
             max(ids, key=lambda b: (N[b], T[b]))]
    long_half = sorted(ids, key=lambda b: -T[b])[:max(1, len(ids) // 2)]
    picks.append(min(long_half, key=lambda b: (N[b], -T[b])))
    out = []
    for b in picks:
        if b not in out:
            out.append(b)
    return out[:n]


def fp64_accuracy(batch, ids, tb, cps, var, full_est=None):
    """Full-horizon FP32-vs-FP64 error of the batched kernel on tracks ids of
    the batch: each track's debug dump (weights, ancestors) and outputs are
    replayed frame by frame in FP64 by the oracle, teacher-forced with the
    device's draws and ancestors.  The tracks run as a sub-batch; tracks are
    independent, so their outputs equal the full run's bit for bit, which is
    checked against full_est (the full run's frame-indexed estimates)."""
    import torch
    import oracle
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from bpf_check import check_track_full
    from mkfbodytracker_pdaf_gb300.filters import BatchedBootstrapPF
    oracle.build()
    sub = batch.subset(ids)
    runner = BatchedBootstrapPF(sub, block_threads=tb, ctas_per_sm=cps, variant=var)
    det_off, det = runner.device_inputs()
    t0 = time.perf_counter()
    rows = []
    for n, b in enumerate(ids):
        t = sub.tracks[n]
        N, T = int(t["n_particles"]), int(t["n_frames"])
        wd = torch.zeros((T, N), dtype=torch.float32, device="cuda")
        ad = torch.zeros((T, N), dtype=torch.int32, device="cuda")
        runner.set_debug(n, wd, ad)
        est, ll, _, _ = runner.run(det_off, det)
        torch.cuda.synchronize()
        est_h = est.cpu().numpy()
        rep = check_track_full(torch, oracle, sub, n, wd, ad, est_h, ll.cpu().numpy())
        s = rep.summary()
        s.update({"track": int(b), "n_particles": N})
        if full_est is not None:
            g0, g1 = int(batch.tracks[b]["frame_base"]), int(t["frame_base"])
            s["same_as_headline_run"] = bool(np.array_equal(full_est[g0:g0 + T], est_h[g1:g1 + T]))
        rows.append(s)
        del wd, ad
    return {"definition": "per frame: posterior mean max_c|est_dev-est_fp64|/max(1,max_c|est_fp64|); "
                          "log-likelihood increment |ll_dev-ll_fp64|/max(1,|ll_fp64|); teacher-forced FP64 "
                          "replay of every frame (device draws and ancestors); ancestors bit-exact",
            "max_rel_err_vs_fp64": max(max(r["max_rel_est"], r["max_rel_loglik"]) for r in rows),
            "tracks": rows, "seconds": time.perf_counter() - t0}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    batch = workload(0, args.tracks)
    import oracle
    oracle.build()
    ids = sample_ids(batch, args.cpu_sample_tracks)
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
                                   "[128,8192], K=15, d=12; CPU sample of %d fixed tracks per step "
                                   "(the GPU line's cpu_baseline sample)" % (args.tracks, len(ids)),
                       "tracks_per_step": len(ids), "track_frames_per_step": sub.n_frames_total},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "%d fixed tracks per step (%d track-frames), FP64 restatement of "
                                       "the reference CPU filter, OpenMP over tracks, longest first"
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
    from mkfbodytracker_pdaf_gb300.replicas import max_over_ranks, sum_over_ranks
    tb, cps, var = load_tuning()
    tb = args.block_threads or tb
    cps = cps if args.ctas_per_sm is None else args.ctas_per_sm
    var = var if args.variant is None else args.variant
    batch = workload(rank, args.tracks)
    runner = BatchedBootstrapPF(batch, block_threads=tb, ctas_per_sm=cps, variant=var)
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
    t_local = max_over_ranks(ms / 1000.0)
    G_all = sum_over_ranks(G)
    value = G_all / t_local
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
    t_e2e = max_over_ranks((time.perf_counter() - t0) / args.steps)
    h2d = hbufs[0].nbytes + hbufs[1].nbytes
    d2h = sum(h.nbytes for h in hbufs[2:])

    if rank == 0:
        peak, peak_kind = load_peaks()
        achieved = BYTES_PER_PF * PF / (ms / 1000.0) / 1e9
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_local * 1000.0, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator, no dataset)",
            "config": {"workload": "batched uneven tracks: B=%d, T~U{50..2000}, N log-uniform [128,8192], "
                                   "K=15, d=12, lambda~U[0,12], P_D~U[0.7,1]" % args.tracks,
                       "tracks_per_gpu": batch.n_tracks, "track_frames_per_gpu": G,
                       "particle_frames_per_gpu": PF,
                       "l2": "inputs larger than L2 (%.2f GB of detections per step)" % (h2d / 1e9),
                       "block_threads": runner.block_threads, "ctas_per_sm": runner.ctas_per_sm,
                       "variant": runner.variant,
                       "parallelism": "one persistent kernel per GPU; tracks sharded by rank"},
            "e2e": {"value": G_all / t_e2e, "unit": UNIT, "h2d_bytes_per_step": h2d,
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
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz")
        if mhz:
            peak_issue = sms * 4 * mhz * 1e6
            ach_issue = WARP_INST_PER_PF * PF / (ms / 1000.0)
            line["roofline"]["issue"] = {
                "bound": "instruction issue (one warp instruction per scheduler per cycle)",
                "warp_inst_per_particle_frame": WARP_INST_PER_PF, "achieved": ach_issue, "peak": peak_issue,
                "unit": "warp-instructions/s", "frac": ach_issue / peak_issue,
                "peak_from": "%d SMs x 4 schedulers x %.0f MHz (median sampled SM clock)" % (sms, mhz)}
        if not args.no_plain:
            pr = plain_rate(batch, args.plain_tracks, args.plain_frames)
            line["plain_path"] = {"value": pr, "unit": UNIT,
                                  "sample": "%d tracks x <=%d frames through mkf_bpf_update" %
                                            (args.plain_tracks, args.plain_frames),
                                  "batched_over_plain": value / ws / pr}
        if not args.no_cpu:
            line["cpu_baseline"] = cpu_baseline(batch, args.cpu_sample_tracks, os.cpu_count() or 1)
            # the metric's error bound, measured on full-length tracks of the same sample
            acc_ids = accuracy_tracks(batch, sample_ids(batch, args.cpu_sample_tracks), args.accuracy_tracks)
            line["accuracy"] = fp64_accuracy(batch, acc_ids, runner.block_threads, runner.ctas_per_sm,
                                             runner.variant, full_est=outs[0].cpu().numpy())
            line["max_rel_err_vs_fp64"] = line["accuracy"]["max_rel_err_vs_fp64"]
        if not args.no_sweep:
            rows = sweep_rows(args.bench_sweep_sizes, args.sweep_frames, 2, 3)
            line["sweep"] = {"workload": "particle-count sweep, one track, T=%d, plain per-track path "
                                         "(C-ABI call per frame, and the frame loop as one CUDA graph)"
                                         % args.sweep_frames,
                             "unit": "particle-frames/s", "rows": rows}
        if not args.no_plain0:
            # the reference's own CPU-runnable case: the two-arm RBPF + PDAF tracker (FP64)
            line["plain0"] = plain0_result(args)
        if not args.no_adjoint:
            # the metric's "+adjoint" half: the mixture-KF gradient (B=1024, T=1000)
            a = adjoint_result(args)
            line["adjoint"] = {k: a[k] for k in ("workload", "forward_ms", "backward_ms", "backward_over_forward",
                                                 "gradient_evals_per_s", "checkpoint_stride", "fd_directions",
                                                 "grad_rel_err_vs_fd", "grad_rel_err_vs_cpu_adjoint",
                                                 "gradient_accuracy")}
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()


# ---------------------------------------------------------------------- extra workloads
def _events(torch):
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def run_sweep(args):
    """Particle-count sweep: one track, T=200, N = 2^12 .. 2^22,
    through the plain per-track C-ABI path (three grid-wide kernels per frame).
    Reports particle-frames/s and the HBM roofline fraction at 112 B per
    particle-frame."""
    from mkfbodytracker_pdaf_gb300 import build
    build.build()
    peak, _ = load_peaks()
    T = args.sweep_frames
    rows = sweep_rows(args.sweep_sizes or list(range(12, 23, 2)), T, args.steps, args.warmup)
    print(json.dumps({"workload": "particle-count sweep, one track, T=%d, plain per-track path: "
                                  "one C-ABI call per frame, and the frame loop captured as one CUDA graph" % T,
                      "unit": "particle-frames/s", "peak_hbm_GBps": peak, "rows": rows}), flush=True)


def sweep_rows(sizes, T, steps, warmup):
    import torch
    from mkfbodytracker_pdaf_gb300 import synth
    from mkfbodytracker_pdaf_gb300.filters import BootstrapParticleFilter
    peak, peak_kind = load_peaks()
    rows = []
    for lg in sizes:
        N = 1 << lg
        batch = synth.sweep_batch(N, n_frames=T)
        t = batch.tracks[0]
        J = batch.model["J"]
        lo = batch.det_off.astype(np.int64)
        det = torch.from_numpy(batch.det.copy()).cuda()
        offs = torch.from_numpy(lo.astype(np.int32)).cuda()
        pf = BootstrapParticleFilter(batch.model, t)
        est = torch.empty((T, batch.model["d"]), dtype=torch.float32, device="cuda")
        ll = torch.empty(T, dtype=torch.float32, device="cuda")
        ess = torch.empty(T, dtype=torch.float32, device="cuda")

        def timed(frames_fn):
            tot = 0.0
            for rep in range(warmup + steps):
                pf.reset()
                e0, e1 = _events(torch)
                e0.record()
                frames_fn()
                e1.record()
                torch.cuda.synchronize()
                if rep >= warmup:
                    tot += e0.elapsed_time(e1) / 1000
            return tot / steps

        def loop():
            for f in range(T):
                pf.update(f, offs[f * J:], det, est=est[f], loglik=ll[f], ess=ess[f])

        sec = timed(loop)
        pf.reset()
        graph = pf.capture(T, offs, det, est, ll, ess)
        sec_g = timed(lambda: graph.launch(0))
        del graph
        pfs = N * T / sec
        ach = BYTES_PER_PF * N * T / sec / 1e9
        ach_g = BYTES_PER_PF * N * T / sec_g / 1e9
        rows.append({"N": N, "T": T, "ms_per_track": sec * 1e3, "particle_frames_per_s": pfs,
                     "track_frames_per_s": T / sec, "achieved_GBps": ach, "frac_of_" + peak_kind + "_hbm": ach / peak,
                     "graph_ms_per_track": sec_g * 1e3, "graph_particle_frames_per_s": N * T / sec_g,
                     "graph_us_per_frame": sec_g / T * 1e6, "graph_frac_of_" + peak_kind + "_hbm": ach_g / peak,
                     "l2_resident": N <= (1 << 18)})
    return rows


def run_plain0(args):
    print(json.dumps(plain0_result(args)), flush=True)


def plain0_result(args):
    """Two-arm pose tracking: two arms, K=15, d=12, N=1000 particles per arm, T=500, FP64
    Rao-Blackwellised filters + PDAF association through PoseTracker, against
    the CPU restatement of the reference frame loop."""
    import torch
    import oracle
    from mkfbodytracker_pdaf_gb300 import build, synth
    from mkfbodytracker_pdaf_gb300.filters import MEAS_PINHOLE, PoseTracker, RaoBlackwellisedPF
    build.build()
    oracle.build()
    T, N, seed = 500, 1000, synth.MASTER_SEED
    sc = synth.make_rbpf_scene(T=T)

    def make():
        arms = []
        for a in range(2):
            arm = sc.arms[a]
            pf = RaoBlackwellisedPF(12, 4, 15, N, meas_mode=MEAS_PINHOLE, seed=seed, track_id=a)
            for k in range(15):
                pf.set_component(k, arm["mu"][k], np.diag(arm["F"][k]), arm["Q"][k], arm["Sigma"][k],
                                 arm["R"][k], arm["weight"][k])
            pf.set_pinhole(arm["Bm"], arm["mm"], synth.CAM)
            pf.set_hand_decode(joint=1)
            pf.resetTracker()
            arms.append(pf)
        return PoseTracker(arms[0], arms[1])

    rois = [None if any(len(h) == 0 for h in fr["heads"]) else np.stack([oracle.scene_roi(fr["heads"][a]) for a in range(2)])
            for fr in sc.frames]
    cands = [torch.from_numpy(fr["hands"]).cuda() if len(fr["hands"]) else None for fr in sc.frames]
    est = np.full((2, T, 12), np.nan)
    times = []
    for rep in range(args.warmup + args.steps):
        trk = make()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for t in range(T):
            e = trk.step(t, rois[t], cands[t])
            if rep == 0 and e is not None:
                for a in range(2):
                    est[a, t] = e[a].cpu().numpy()
        torch.cuda.synchronize()
        if rep >= args.warmup:
            times.append(time.perf_counter() - t0)
    gpu_s = float(np.median(times))
    t0 = time.perf_counter()
    est_c, skipped = oracle.pose_tracker_run(sc, N, seed, T=T)
    cpu_s = time.perf_counter() - t0
    ok = ~skipped
    rel = float(np.abs(est[:, ok] - est_c[:, ok]).max() / np.abs(est_c[:, ok]).max())
    err = float(np.abs(est_c[:, ok] - sc.truth[:, ok]).mean())
    return {"workload": "two-arm pose tracking: 2 arms x T=%d, N=%d, K=15, d=12, FP64 RBPF + PDAF" % (T, N),
            "gpu_track_frames_per_s": 2 * T / gpu_s, "gpu_s": gpu_s,
            "cpu_track_frames_per_s": 2 * T / cpu_s, "cpu_s": cpu_s, "cpu_threads": 1,
            "max_rel_est_err_vs_cpu": rel, "mean_abs_latent_err_vs_truth": err,
            "frames_skipped": int(skipped.sum())}


def run_adjoint(args):
    print(json.dumps(adjoint_result(args)), flush=True)


def adjoint_result(args):
    """Mixture-KF logL over B=1024 x T=1000, K=15, d=12; forward and
    backward times, backward/forward ratio, and gradient accuracy against the
    FP64 CPU adjoint and FP64 central differences on a track subset."""
    import torch
    import oracle
    from mkfbodytracker_pdaf_gb300 import build, mixkf, synth
    build.build()
    oracle.build()
    b = synth.mixkf_batch_k15(n_tracks=args.adj_tracks, T=args.adj_frames)
    tt = b.theta_true()
    om = oracle.MixModel(tt["mu"], tt["a"], tt["Lq"], tt["sigma"], tt["pi"], tt["S0"])
    th = om.theta()
    g = mixkf.MixtureKF(b, tt["pi"], tt["S0"])
    g.set_theta(th)
    for _ in range(args.warmup):
        g.forward()
        g.backward()
    torch.cuda.synchronize()
    fwd, bwd = [], []
    for _ in range(args.steps):
        e0, e1 = _events(torch)
        e2 = torch.cuda.Event(enable_timing=True)
        e0.record()
        g.forward()
        e1.record()
        g.backward()
        e2.record()
        torch.cuda.synchronize()
        fwd.append(e0.elapsed_time(e1))
        bwd.append(e1.elapsed_time(e2))
    L_gpu = g.forward().item()
    grad = g.backward().cpu().numpy()
    # accuracy on a subset (FP64 CPU adjoint and central differences, 64
    # directions), at the generating parameters and at the fitting start point
    # (means + N(0, 0.3), covariances x 1.5)
    sub = list(range(min(args.adj_check_tracks, b.n_tracks)))
    sb = synth.MixBatch(b.gmm, [b.tracks[i] for i in sub], b.Bm, b.mm, b.det_off, b.det, b.truth)
    gs = mixkf.MixtureKF(sb, tt["pi"], tt["S0"])
    K, d = om.K, om.d
    rng0 = np.random.default_rng(4)
    th_start = mixkf.theta_from(tt["mu"] + rng0.normal(0, 0.3, tt["mu"].shape), tt["a"], tt["Lq"] * np.sqrt(1.5),
                                tt["sigma"] * np.sqrt(1.5))
    points = {}
    for name, thp in (("at_generating_params", th), ("at_fit_start", th_start)):
        points[name] = grad_accuracy(oracle, om.with_theta(thp), thp, sb, gs, args.fd_dirs, K, d)
    tf = float(np.median(fwd))
    tb = float(np.median(bwd))
    acc = points["at_generating_params"]
    return {
        "workload": "mixture-KF logL and adjoint, B=%d x T=%d, K=15, d=12, PDAF <=16 candidates, FP32 + FP64 sums"
                    % (b.n_tracks, args.adj_frames),
        "forward_ms": tf, "backward_ms": tb, "backward_over_forward": tb / tf,
        "track_frames_per_s_forward": b.n_frames_total / tf * 1e3,
        "gradient_evals_per_s": 1e3 / (tf + tb), "logL": L_gpu,
        "checkpoint_stride": g.checkpoint_stride,
        "check_subset_tracks": len(sub), "logL_rel_err_subset": acc["logL_rel_err"],
        "fd_directions": args.fd_dirs,
        "grad_rel_err_vs_fd": acc["rel_err_vs_fd"],
        "grad_rel_err_vs_cpu_adjoint": acc["rel_err_vs_cpu_adjoint"],
        "gradient_accuracy": points}


def grad_accuracy(oracle, om, th, sb, gs, ndirs, K, d):
    """GPU gradient on the subset batch sb against the FP64 CPU adjoint and
    FP64 central differences (relative step 1e-6) along ndirs random unit
    directions, plus the normwise error per parameter block."""
    gs.set_theta(th)
    gs.forward()
    grad_s = gs.backward().cpu().numpy()
    L_sub_gpu = float(gs.ll.sum().item())
    t0 = time.perf_counter()
    L_c, _, gref = oracle.mix_batch(om, sb, grad=True)
    cpu_adj_s = time.perf_counter() - t0
    rng = np.random.default_rng(64)
    rel_fd, rel_adj, rel_cpu_fd = [], [], []
    for _ in range(ndirs):
        v = rng.standard_normal(th.size)
        v /= np.linalg.norm(v)
        h = 1e-6 * max(1.0, np.abs(th).max())
        Lp, _ = oracle.mix_batch(om.with_theta(th + h * v), sb)
        Lm, _ = oracle.mix_batch(om.with_theta(th - h * v), sb)
        fd = (Lp - Lm) / (2 * h)
        rel_fd.append(abs(v @ grad_s - fd) / max(abs(fd), 1e-9))
        rel_cpu_fd.append(abs(v @ gref - fd) / max(abs(fd), 1e-9))
        rel_adj.append(abs(v @ grad_s - v @ gref) / max(abs(v @ gref), 1e-9))
    DD = d * (d + 1) // 2
    blocks = {"mu": slice(0, K * d), "a": slice(K * d, 2 * K * d), "Lq": slice(2 * K * d, 2 * K * d + K * DD),
              "sigma": slice(th.size - 1, th.size)}
    normwise = {k: float(np.linalg.norm(grad_s[sl] - gref[sl]) / max(np.linalg.norm(gref[sl]), 1e-300))
                for k, sl in blocks.items()}
    med = lambda x: {"median": float(np.median(x)), "max": float(np.max(x))}
    return {"logL_rel_err": abs(L_sub_gpu - L_c) / abs(L_c), "grad_norm": float(np.linalg.norm(gref)),
            "rel_err_vs_fd": med(rel_fd), "rel_err_vs_cpu_adjoint": med(rel_adj),
            "cpu_adjoint_rel_err_vs_fd": med(rel_cpu_fd),
            "normwise_rel_err_vs_cpu_adjoint": normwise,
            "normwise_rel_err_total": float(np.linalg.norm(grad_s - gref) / np.linalg.norm(gref)),
            "cpu_adjoint_s": cpu_adj_s}


def run_fit(args):
    """Motion-model fit: fit the motion model by gradient on the device from
    data the filter's own generative model produced.  --fit-case config4: K=32,
    d=24 (8 joints x 3D), lambda=5; --fit-case exact: one component (K=1,
    d=12), no clutter, detection probability 0.999, where the filter's
    likelihood is the model's own (an EKF whose linearisation error is small at
    these depths), so that the fit can be judged by parameter recovery."""
    import torch
    from mkfbodytracker_pdaf_gb300 import build, mixkf, synth
    build.build()
    if args.fit_case == "exact":
        K, d = args.fit_components, 12
        b = synth.fit_batch_exact(n_tracks=args.fit_tracks, T=args.fit_frames, K=K)
    else:
        K, d = 32, 24
        b = synth.fit_batch_k32(n_tracks=args.fit_tracks, T=args.fit_frames)
    tt = b.theta_true()
    th_true = mixkf.theta_from(tt["mu"], tt["a"], tt["Lq"], tt["sigma"])
    rng = np.random.default_rng(4)
    mu0 = tt["mu"] + rng.normal(0, 0.3, tt["mu"].shape)
    Lq0 = tt["Lq"] * np.sqrt(1.5)                 # covariances x1.5
    th0 = mixkf.theta_from(mu0, tt["a"], Lq0, tt["sigma"] * np.sqrt(1.5))
    g = mixkf.MixtureKF(b, tt["pi"], tt["S0"])
    g.set_theta(th0)
    L0 = g.forward().item()
    g.set_theta(th_true)
    Ltrue = g.forward().item()
    times = []
    hist = []

    def cb(it, th, tot):
        if it % 10 == 0 or it == 1:
            hist.append((it, float(tot.item())))

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    th, _ = g.fit_adam(th0, args.fit_steps, lr=args.fit_lr, callback=cb)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    thf = th.cpu().numpy()
    g.set_theta(thf)
    Lf = g.forward().item()
    mu_f, a_f, L_f, s_f = mixkf.theta_split(thf, K, d)
    mu_0 = mu0
    err = lambda x, y: float(np.abs(x - y).mean())
    Qt = np.einsum("kij,klj->kil", synth.unpack_lower(tt["Lq"], d), synth.unpack_lower(tt["Lq"], d))
    Qf = np.einsum("kij,klj->kil", synth.unpack_lower(L_f, d), synth.unpack_lower(L_f, d))
    Q0 = np.einsum("kij,klj->kil", synth.unpack_lower(Lq0, d), synth.unpack_lower(Lq0, d))
    # components matched to the truth by their means (Hungarian assignment), then compared
    cost = ((mu_f[:, None, :] - tt["mu"][None, :, :]) ** 2).sum(-1)
    try:
        from scipy.optimize import linear_sum_assignment
        _, perm = linear_sum_assignment(cost)
    except ImportError:
        perm = np.argmin(cost, axis=1)
    matched = {"mu_mae": err(mu_f, tt["mu"][perm]),
               "a_mae": err(a_f, tt["a"][perm]), "Q_mae": err(Qf, Qt[perm]),
               "components_relabelled": int((perm != np.arange(K)).sum())}
    # per parameter block: the fitted parameters with one block put back to the
    # truth; logL(fit) - logL(that) is the block's share of the fit's excess
    DD = d * (d + 1) // 2
    blocks = {"mu": slice(0, K * d), "a": slice(K * d, 2 * K * d), "Lq": slice(2 * K * d, 2 * K * d + K * DD),
              "sigma": slice(th_true.size - 1, th_true.size)}
    per_block = {}
    for name, sl in blocks.items():
        hyb = thf.copy()
        hyb[sl] = th_true[sl]
        g.set_theta(hyb)
        per_block[name] = {"n_params": int(sl.stop - sl.start), "logL_fit_minus_with_true_block": Lf - g.forward().item()}
    print(json.dumps({
        "workload": "motion-model fit (%s): K=%d, d=%d from B=%d x T=%d, %d Adam steps (lr %g) on the device"
                    % (args.fit_case, K, d, b.n_tracks, args.fit_frames, args.fit_steps, args.fit_lr),
        "seconds_total": wall, "seconds_per_gradient_eval": wall / args.fit_steps,
        "logL_init": L0, "logL_final": Lf, "logL_true_params": Ltrue, "logL_history": hist,
        "logL_final_minus_true": Lf - Ltrue, "n_params": int(th_true.size),
        "half_n_params": 0.5 * th_true.size, "per_block": per_block,
        "recovery": {"mu_mae_init": err(mu_0, tt["mu"]), "mu_mae_final": err(mu_f, tt["mu"]),
                     # the drift (1 - a_k) mu_k is what a frame's transition uses
                     "drift_mae_init": err((1 - tt["a"]) * mu_0, (1 - tt["a"]) * tt["mu"]),
                     "drift_mae_final": err((1 - a_f) * mu_f, (1 - tt["a"]) * tt["mu"]),
                     "a_mae_init": 0.0, "a_mae_final": err(a_f, tt["a"]),
                     "Q_mae_init": err(Q0, Qt), "Q_mae_final": err(Qf, Qt),
                     "sigma_init": float(th0[-1]), "sigma_final": s_f, "sigma_true": float(tt["sigma"]),
                     "after_matching_components": matched}}),
          flush=True)


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--tracks", type=int, default=8192)
    ap.add_argument("--block-threads", type=int, default=None, help="default: autotuned choice")
    ap.add_argument("--ctas-per-sm", type=int, default=None)
    ap.add_argument("--variant", type=int, default=None, help="bit 0 float4 loads, bit 1 binary-search resampling")
    ap.add_argument("--cpu-sample-tracks", type=int, default=96)
    ap.add_argument("--accuracy-tracks", type=int, default=4,
                    help="full-length tracks of the CPU sample replayed in FP64 for the error bound")
    ap.add_argument("--plain-tracks", type=int, default=8)
    ap.add_argument("--plain-frames", type=int, default=300)
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the mixture-KF adjoint summary of the default run")
    ap.add_argument("--no-sweep", action="store_true", help="skip the particle-count sweep rows of the default run")
    ap.add_argument("--no-plain0", action="store_true", help="skip the two-arm pose-tracking case of the default run")
    ap.add_argument("--bench-sweep-sizes", type=int, nargs="*", default=[20, 22],
                    help="log2 particle counts of the default run's sweep rows")
    ap.add_argument("--workload", default="batched", choices=["batched", "sweep", "plain0", "adjoint", "fit"])
    ap.add_argument("--sweep-frames", type=int, default=200)
    ap.add_argument("--sweep-sizes", type=int, nargs="*", default=None,
                    help="log2 particle counts of the sweep (default 12 14 ... 22)")
    ap.add_argument("--adj-tracks", type=int, default=1024)
    ap.add_argument("--adj-frames", type=int, default=1000)
    ap.add_argument("--adj-check-tracks", type=int, default=8)
    ap.add_argument("--fd-dirs", type=int, default=64)
    ap.add_argument("--fit-case", default="config4", choices=["config4", "exact"])
    ap.add_argument("--fit-components", type=int, default=1,
                    help="components of the clutter-free control case (1: the filter's likelihood is exact)")
    ap.add_argument("--fit-tracks", type=int, default=None, help="default: 16384 (config4), 128 (exact)")
    ap.add_argument("--fit-frames", type=int, default=None, help="default: 500 (config4), 200 (exact)")
    ap.add_argument("--fit-steps", type=int, default=None, help="default: 200 (config4), 400 (exact)")
    ap.add_argument("--fit-lr", type=float, default=0.02)
    args = ap.parse_args(argv)
    if args.warmup < 3:
        args.warmup = 3
    exact = args.fit_case == "exact"
    args.fit_tracks = args.fit_tracks or (128 if exact else 16384)
    args.fit_frames = args.fit_frames or (200 if exact else 500)
    args.fit_steps = args.fit_steps or (400 if exact else 200)
    return args


def main(argv=None):
    args = parse_args(argv)
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "sweep":
        run_sweep(args)
    elif args.workload == "plain0":
        run_plain0(args)
    elif args.workload == "adjoint":
        run_adjoint(args)
    elif args.workload == "fit":
        run_fit(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
