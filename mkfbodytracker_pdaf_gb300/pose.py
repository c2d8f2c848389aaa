"""Pose decode and 3-D back-projection over the C ABI (the step after the
estimate): e = H_pca^T x + m_pca (pfPose.cpp:347-348), get3Dpose
(pfPose.cpp:93-127) and the publish2Dpos point record (pfPose.cpp:173-208),
batched over estimates on the GPU."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N

# the Kinect intrinsics hard-wired in get3Dpose (pfPose.cpp:101)
KINECT_K = np.array([[525.0, 0.0, 319.5], [0.0, 525.0, 239.5], [0.0, 0.0, 1.0]])
POINT_NAMES = ("hand1", "hand2", "head", "neck", "elbow1", "elbow2", "shoulder1", "shoulder2")


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


class PoseDecoder:
    """Holds H_pca (d x F) and m_pca (F) on the device."""

    def __init__(self, Hpca, mpca, Kc=KINECT_K):
        import torch
        self.torch = torch
        self.H = torch.from_numpy(np.ascontiguousarray(Hpca, np.float64)).cuda()
        self.m = torch.from_numpy(np.ascontiguousarray(mpca, np.float64).ravel()).cuda()
        self.d, self.F = self.H.shape
        self.Kc = np.ascontiguousarray(Kc, np.float64).ravel()
        self.status = torch.zeros(1, dtype=torch.int32, device="cuda")

    def decode(self, x, pose3d=True, stream=None):
        """x: (B, d) float64 CUDA tensor -> (e (B, F), pos3d (B, 3, 5) or None)."""
        t = self.torch
        x = x.reshape(-1, self.d).contiguous()
        B = x.shape[0]
        e = t.empty((B, self.F), dtype=t.float64, device="cuda")
        p3 = t.empty((B, 3, 5), dtype=t.float64, device="cuda") if pose3d else None
        s = stream if stream is not None else t.cuda.current_stream()
        N.check(N.lib().mkf_pose_decode(_ptr(x), B, self.d, self.F, _ptr(self.H), _ptr(self.m),
                                        self.Kc.ctypes.data_as(C.c_void_p), _ptr(e), _ptr(p3),
                                        _ptr(self.status), C.c_void_p(s.cuda_stream)), "mkf_pose_decode")
        return e, p3


def pose2d_record(e1, e2, stream=None):
    """(B, F) decoded vectors of both arms -> (B, 8, 2) points in POINT_NAMES order."""
    import torch
    B, F = e1.shape
    pts = torch.empty((B, 8, 2), dtype=torch.float64, device="cuda")
    s = stream if stream is not None else torch.cuda.current_stream()
    N.check(N.lib().mkf_pose2d_record(_ptr(e1.contiguous()), _ptr(e2.contiguous()), B, F, _ptr(pts),
                                      C.c_void_p(s.cuda_stream)), "mkf_pose2d_record")
    return pts
