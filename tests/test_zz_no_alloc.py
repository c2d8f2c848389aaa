"""The allocation-free resampler entry point (mkf_resample_f32_noalloc), for
callers that must not allocate device memory during their frame loop: its
output must equal mkf_resample_f32's on the same weights and uniform, call
after call, although every call reuses the same fixed scratch array.  This file
sorts last so that a run stopping at the first failure has run everything
else; it also passes alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(torch, fn, w, N, U):
    from mkfbodytracker_pdaf_gb300 import _native as Nn
    dw = torch.from_numpy(w).cuda()
    idx = torch.full((N,), -1, dtype=torch.int32, device="cuda")
    fb = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    st = fn(C.c_void_p(dw.data_ptr()), len(w), N, U, C.c_void_p(idx.data_ptr()), C.c_void_p(fb.data_ptr()),
            C.c_void_p(torch.cuda.current_stream().cuda_stream))
    Nn.check(st, "resample")
    torch.cuda.synchronize()
    return idx.cpu().numpy(), int(fb.item())


def test_noalloc_matches_allocating_resampler_twice(cuda):
    from mkfbodytracker_pdaf_gb300 import _native as Nn
    torch = cuda
    L_ = Nn.lib()
    rng = np.random.default_rng(2026)
    cases = [(700000, 250000), (5000, 8192), (1 << 20, 4096)]   # two calls in a row, then the maximum size
    for L, N in cases:
        w = (rng.random(L) ** 5).astype(np.float32)
        w[rng.random(L) < 0.3] = 0.0
        U = int(rng.integers(0, 2 ** 32))
        ref, fb_ref = _run(torch, L_.mkf_resample_f32, w, N, U)
        got, fb_got = _run(torch, L_.mkf_resample_f32_noalloc, w, N, U)
        assert fb_got == fb_ref == 0
        np.testing.assert_array_equal(got, ref)
    # all-zero weights take the same uniform fallback
    z = np.zeros(1000, np.float32)
    ref, fb_ref = _run(torch, L_.mkf_resample_f32, z, 300, 77)
    got, fb_got = _run(torch, L_.mkf_resample_f32_noalloc, z, 300, 77)
    assert fb_ref == fb_got == 1
    np.testing.assert_array_equal(got, ref)


def test_noalloc_rejects_oversized_input(cuda):
    from mkfbodytracker_pdaf_gb300 import _native as Nn
    torch = cuda
    L_ = Nn.lib()
    w = torch.ones((1 << 20) + 1, dtype=torch.float32, device="cuda")
    idx = torch.empty(16, dtype=torch.int32, device="cuda")
    st = L_.mkf_resample_f32_noalloc(C.c_void_p(w.data_ptr()), w.numel(), 16, 1, C.c_void_p(idx.data_ptr()), None,
                                     C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 1 and b"1048576" in L_.mkf_last_error()
