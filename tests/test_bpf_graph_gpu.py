"""The captured frame loop (CUDA graph of the per-track update) gives bit-for-bit
the results of the same frames run by individual mkf_bpf_update calls, with
chunks staged into the buffers bound at capture, an odd chunk length (the
particle buffers end swapped and are copied back) and a plain update chained
after the graph launches."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_graph_replay_matches_updates(cuda):
    from mkfbodytracker_pdaf_gb300 import synth
    from mkfbodytracker_pdaf_gb300.filters import BootstrapParticleFilter
    torch = cuda
    T, n = 10, 3
    batch = synth.make_bpf_batch(5, [3000], [T], [6.0], [0.85])
    t = batch.tracks[0]
    J, d = batch.model["J"], batch.model["d"]
    offs = batch.det_off[:T * J + 1].astype(np.int64)

    pa = BootstrapParticleFilter(batch.model, t)
    pa.reset()
    det_all = torch.from_numpy(batch.det.copy()).cuda()
    off_all = torch.from_numpy(offs.astype(np.int32)).cuda()
    ref = []
    for f in range(T):
        e = pa.update(f, off_all[f * J:], det_all)
        ref.append((e.cpu().numpy().copy(), float(pa.loglik.item()), float(pa.ess.item())))

    pb = BootstrapParticleFilter(batch.model, t)
    pb.reset()
    off_buf = torch.zeros(n * J + 1, dtype=torch.int32, device="cuda")
    det_buf = torch.zeros((max(1, len(batch.det)), 2), dtype=torch.float32, device="cuda")
    est = torch.zeros((n, d), dtype=torch.float32, device="cuda")
    ll = torch.zeros(n, dtype=torch.float32, device="cuda")
    ess = torch.zeros(n, dtype=torch.float32, device="cuda")
    graph = pb.capture(n, off_buf, det_buf, est, ll, ess)
    got = []
    f0 = 0
    while f0 + n <= T:
        lo = offs[f0 * J:(f0 + n) * J + 1]
        off_buf.copy_(torch.from_numpy((lo - lo[0]).astype(np.int32)))
        if lo[-1] > lo[0]:
            det_buf[:lo[-1] - lo[0]].copy_(torch.from_numpy(batch.det[lo[0]:lo[-1]].copy()))
        graph.launch(f0)
        for k in range(n):
            got.append((est[k].cpu().numpy().copy(), float(ll[k].item()), float(ess[k].item())))
        f0 += n
    for f in range(f0, T):                       # chained plain updates after the launches
        e = pb.update(f, off_all[f * J:], det_all)
        got.append((e.cpu().numpy().copy(), float(pb.loglik.item()), float(pb.ess.item())))
    torch.cuda.synchronize()
    assert len(got) == T
    for f in range(T):
        np.testing.assert_array_equal(got[f][0], ref[f][0])
        assert got[f][1] == ref[f][1] and got[f][2] == ref[f][2]
    assert pb.status() == pa.status()
