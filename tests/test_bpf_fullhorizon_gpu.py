"""Full-horizon error of the batched FP32 particle filter against FP64.

The headline workload runs tracks of up to 2000 frames with up to 8192
particles in FP32.  This test replays every frame of such tracks in FP64,
teacher-forced (the device's draws and ancestors, the oracle's arithmetic:
pf2D.cpp:148-210's weight / normalise / resample loop with my_gmm.cpp:53-58's
motion), and bounds the device's error over the whole horizon:

* posterior mean: max_c |est_dev - est_64| / max(1, max_c |est_64|) <= 1e-4
  in every frame;
* log-likelihood increment: |ll_dev - ll_64| / max(1, |ll_64|) <= 1e-4;
* weights (normalised to max 1): max_i |w_dev - w_64| <= 1e-4;
* ancestors: bit-exact with the exact resampler applied to the device's
  weights, in every frame.

The shapes are the workload's extremes: T = 2000 with N = 8192 at the highest
clutter rate and lowest detection probability, and at no clutter with
certain detection; N = 128 over 2000 frames; a mid-size track.
"""
import json
import os

import numpy as np
import pytest

from bpf_check import check_track_full

pytestmark = pytest.mark.gpu

TOL = 1e-4


def test_batched_full_horizon_within_1e4_of_fp64(cuda, olib):
    from mkfbodytracker_pdaf_gb300 import synth
    from mkfbodytracker_pdaf_gb300.filters import BatchedBootstrapPF
    torch = cuda
    batch = synth.make_bpf_batch(2024, [8192, 8192, 128, 3000], [2000, 2000, 2000, 1000],
                                 [12.0, 0.0, 6.0, 3.0], [0.7, 1.0, 0.85, 0.9])
    runner = BatchedBootstrapPF(batch)
    det_off, det = runner.device_inputs()
    results = {}
    for b in range(batch.n_tracks):
        N = int(batch.tracks[b]["n_particles"])
        T = int(batch.tracks[b]["n_frames"])
        wd = torch.zeros((T, N), dtype=torch.float32, device="cuda")
        ad = torch.zeros((T, N), dtype=torch.int32, device="cuda")
        runner.set_debug(b, wd, ad)
        est, ll, ess, st = runner.run(det_off, det)
        torch.cuda.synchronize()
        assert (st.cpu().numpy() & ~8 == 0).all()
        rep = check_track_full(torch, olib, batch, b, wd, ad, est.cpu().numpy(), ll.cpu().numpy())
        s = rep.summary()
        results["N%d_T%d_lam%g" % (N, T, batch.tracks[b]["lam"])] = s
        assert s["ancestor_frames_bit_exact"] == T
        assert s["max_rel_est"] <= TOL, s
        assert s["max_rel_loglik"] <= TOL, s
        assert s["max_abs_weight"] <= TOL, s
    out = os.environ.get("MKF_ACCURACY_JSON")
    if out:
        with open(out, "w") as f:
            json.dump(results, f, indent=1)
    print(json.dumps(results))
