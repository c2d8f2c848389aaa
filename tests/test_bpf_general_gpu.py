"""The particle kernels' general paths against the FP64 oracle: a full
(non-diagonal) process-noise factor L_k, and the 24-dimensional state with
three measured joints, through both the per-track streaming kernels and the
batched persistent kernel."""
import numpy as np
import pytest

from bpf_check import check_track
from test_bpf_gpu import _run_stream

pytestmark = pytest.mark.gpu


def _full_noise(batch, seed=4):
    """Replace each component's diagonal L_k by a lower-triangular one."""
    rng = np.random.default_rng(seed)
    Lq = batch.model["Lq"].astype(np.float64)
    d = batch.model["d"]
    for r in range(d):
        for c in range(r):
            Lq[..., r * (r + 1) // 2 + c] = rng.normal(0, 0.03, Lq.shape[:-1])
    batch.model["Lq"] = Lq.astype(np.float32)
    return batch


def _batched_check(torch, olib, batch, tracks):
    from mkfbodytracker_pdaf_gb300.filters import BatchedBootstrapPF
    runner = BatchedBootstrapPF(batch, block_threads=256)
    det_off, det = runner.device_inputs()
    for b in tracks:
        N, T = int(batch.tracks[b]["n_particles"]), int(batch.tracks[b]["n_frames"])
        wd = torch.zeros((T, N), dtype=torch.float32, device="cuda")
        ad = torch.zeros((T, N), dtype=torch.int32, device="cuda")
        runner.set_debug(b, wd, ad)
        est, ll, ess, st = runner.run(det_off, det)
        torch.cuda.synchronize()
        assert (st.cpu().numpy() & ~8 == 0).all()
        g0 = int(batch.tracks[b]["frame_base"])
        frames = [dict(est=est[g0 + f].double().cpu().numpy(), loglik=float(ll[g0 + f].item()),
                       w=wd[f].cpu().numpy(), anc=ad[f].cpu().numpy()) for f in range(T)]
        check_track(torch, olib, batch, b, frames)


def test_full_noise_factor(cuda, olib):
    from mkfbodytracker_pdaf_gb300 import synth
    torch = cuda
    batch = _full_noise(synth.make_bpf_batch(17, [900, 2500], [5, 4], [3.0, 6.0], [0.9, 0.8]))
    frames, pf = _run_stream(torch, batch, 0, 5)
    check_track(torch, olib, batch, 0, frames)
    _batched_check(torch, olib, batch, [0, 1])


def test_state_dimension_24(cuda, olib):
    from mkfbodytracker_pdaf_gb300 import synth
    torch = cuda
    batch = synth.make_bpf_batch(23, [700, 3000], [4, 3], [3.0, 5.0], [0.9, 0.85], d=24, K=8)
    frames, pf = _run_stream(torch, batch, 1, 3)
    check_track(torch, olib, batch, 1, frames)
    _batched_check(torch, olib, batch, [0, 1])
