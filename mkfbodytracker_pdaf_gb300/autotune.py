"""Autotuner for the batched persistent kernel: block size (and so particles
per thread, ceil(N / block)), resident CTAs per SM, and the kernel's code
variants (float4 vs scalar model loads; ancestors by binary search vs the
scatter walk).

Run on the target GPU:
    python -m mkfbodytracker_pdaf_gb300.autotune --tracks 8192 --out tuning.json
It times every candidate on the batched-uneven-tracks workload with CUDA
events and writes the ranking; ``load_tuning()`` returns the stored best
choice (used by the benchmark and the runners when present).  Tune at the
full batch size: with few tracks per CTA the tail of the schedule dominates and
the ranking changes.
"""
from __future__ import annotations

import argparse
import json
import os
import time

HERE = os.path.dirname(os.path.abspath(__file__))
TUNING_FILE = os.path.join(HERE, "tuning_gb300.json")
# variant bits: 1 float4 loads, 2 binary-search resampling, 4 particle pairs,
# 8 the search with 8 bytes/particle of shared memory (ancestors in L2)
# (block_threads, ctas_per_sm): 512x1 and 256x2 compile with a 128-register
# budget; 256x3 and 384x2 (float4 loads + search only) with 80 registers.  At
# 8192 particles the search keeps 12 bytes/particle in shared memory (2 CTAs
# of 102 KB per SM), the LOW layout 8 (3 CTAs of 70 KB).
CANDIDATES = ([(256, 2, v) for v in (0, 1, 2, 3, 7, 11)] + [(512, 1, v) for v in (0, 1, 2, 3, 7, 11)] +
              [(256, 3, 3), (384, 2, 3), (256, 3, 11), (384, 2, 11)])
# the candidates that have ranked at the top, for a short tuning run
QUICK = [(256, 2, 3), (256, 3, 3), (384, 2, 3), (256, 3, 11), (384, 2, 11)]


def load_tuning():
    if os.path.exists(TUNING_FILE):
        with open(TUNING_FILE) as f:
            d = json.load(f)
        b = d["best"]
        return int(b["block_threads"]), int(b["ctas_per_sm"]), int(b.get("variant", 1))
    return 256, 3, 1


def tune(n_tracks=8192, reps=2, seed=None, candidates=CANDIDATES):
    import torch
    from . import build, synth
    from .filters import BatchedBootstrapPF
    build.build()
    kw = {} if seed is None else {"seed": seed}
    batch = synth.uneven_tracks_batch(n_tracks=n_tracks, **kw)
    runner = BatchedBootstrapPF(batch)
    det_off, det = runner.device_inputs()
    outs = runner.alloc_outputs()
    G = batch.n_frames_total
    res = []
    for tb, cps, var in candidates:
        try:
            runner.set_tuning(tb, cps, var)
            runner.run(det_off, det, outs)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                runner.run(det_off, det, outs)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / reps
            res.append({"block_threads": tb, "ctas_per_sm": cps, "variant": var, "ms": ms,
                        "track_frames_per_s": G / ms * 1e3, "grid": runner.last_grid()})
        except Exception as ex:  # a shape that does not fit is reported, not fatal
            res.append({"block_threads": tb, "ctas_per_sm": cps, "variant": var, "error": str(ex)})
    ok = [r for r in res if "ms" in r]
    best = min(ok, key=lambda r: r["ms"])
    return {"workload": "batched uneven tracks subset: %d tracks, %d track-frames" % (n_tracks, G),
            "gpu": torch.cuda.get_device_name(0), "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime()),
            "results": res, "best": best}


def merge_rankings(new, old):
    """A partial (--quick) ranking keeps the previous ranking's full table
    beside it: ``best`` comes from the new run alone (rankings from different
    runs are not compared), the old results move to ``earlier_results``."""
    if not old:
        return new
    out = dict(new)
    out["earlier_results"] = {"when": old.get("when"), "results": old.get("results", [])}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--tracks", type=int, default=8192)
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--out", default=TUNING_FILE)
    ap.add_argument("--quick", action="store_true",
                    help="rank only the usual top candidates, keeping the previous table of --out")
    a = ap.parse_args()
    r = tune(a.tracks, a.reps, candidates=QUICK if a.quick else CANDIDATES)
    if a.quick and os.path.exists(a.out):
        with open(a.out) as f:
            r = merge_rankings(r, json.load(f))
    with open(a.out, "w") as f:
        json.dump(r, f, indent=1)
    print(json.dumps(r))


if __name__ == "__main__":
    main()
