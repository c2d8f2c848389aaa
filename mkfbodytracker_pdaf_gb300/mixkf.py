"""Host-side API of the mixture Kalman filter log-likelihood and its adjoint
(forward/backward pair of the C ABI), and the on-device Adam fitting loop of
the motion model.

theta (flat FP64) = [mu (K*d), a (K*d), Lq packed lower (K*d(d+1)/2), sigma].
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .filters import _ptr, _stream


def theta_from(mu, a, Lq_packed, sigma):
    return np.concatenate([np.ravel(mu), np.ravel(a), np.ravel(Lq_packed), [float(sigma)]]).astype(np.float64)


def theta_split(theta, K, d):
    DD = d * (d + 1) // 2
    return (theta[:K * d].reshape(K, d), theta[K * d:2 * K * d].reshape(K, d),
            theta[2 * K * d:2 * K * d + K * DD].reshape(K, DD), float(theta[-1]))


class FitState:
    """Adam fitting state (theta and moments after `step` steps)."""

    def __init__(self, theta, m, v, step, lr, K, d):
        self.theta, self.m, self.v = (np.ascontiguousarray(a, np.float64) for a in (theta, m, v))
        self.step, self.lr, self.K, self.d = int(step), float(lr), int(K), int(d)


_FIT_MAGIC = b"MKFFIT01"


def save_fit_state(path, st):
    """Binary file: magic, uint32 header length, JSON header (sizes, step,
    learning rate, K, d), then theta, m, v as little-endian float64."""
    import json
    import struct
    hdr = json.dumps({"n_theta": int(st.theta.size), "step": st.step, "lr": st.lr, "K": st.K, "d": st.d,
                      "layout": "theta = [mu (K d), a (K d), Lq packed lower (K d(d+1)/2), sigma]"}).encode()
    with open(path, "wb") as f:
        f.write(_FIT_MAGIC)
        f.write(struct.pack("<I", len(hdr)))
        f.write(hdr)
        for a in (st.theta, st.m, st.v):
            f.write(a.astype("<f8").tobytes())


def load_fit_state(path):
    import json
    import struct
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:8] != _FIT_MAGIC:
        raise ValueError("not a fit-state file")
    (n,) = struct.unpack_from("<I", buf, 8)
    hdr = json.loads(buf[12:12 + n].decode())
    k = hdr["n_theta"]
    arr = np.frombuffer(buf, "<f8", 3 * k, 12 + n).reshape(3, k).copy()
    return FitState(arr[0], arr[1], arr[2], hdr["step"], hdr["lr"], hdr["K"], hdr["d"])


class MixtureKF:
    """Batched mixture KF over the tracks of a synth.MixBatch-like object."""

    def __init__(self, batch, pi, S0, cam=(525.0, 525.0, 319.5, 239.5)):
        import torch
        self.torch = torch
        self.batch = batch
        self.K, self.d = np.asarray(S0).shape[0], np.asarray(S0).shape[1]
        self.J = batch.Bm.shape[1]
        self._pi = np.ascontiguousarray(pi, np.float64)
        self._S0 = np.ascontiguousarray(S0, np.float64)
        desc = N.MixModelDesc(self.d, self.K, self.J, self._pi.ctypes.data_as(C.c_void_p),
                              self._S0.ctypes.data_as(C.c_void_p), *cam)
        nt = batch.n_tracks
        nf = np.array([t["n_frames"] for t in batch.tracks], np.int32)
        fb = np.array([t["frame_base"] for t in batch.tracks], np.int64)
        Bm = np.ascontiguousarray(np.stack([batch.Bm[t["body"]] for t in batch.tracks]), np.float64)
        mm = np.ascontiguousarray(np.stack([batch.mm[t["body"]] for t in batch.tracks]), np.float64)
        pd = np.array([t["pd"] for t in batch.tracks], np.float64)
        kp = np.array([t["kappa"] for t in batch.tracks], np.float64)
        pp = lambda a: a.ctypes.data_as(C.c_void_p)
        h = C.c_void_p()
        N.check(N.lib().mkf_mixkf_create(C.byref(desc), nt, pp(nf), pp(fb), pp(Bm), pp(mm), pp(pd), pp(kp),
                                         batch.n_frames_total, C.byref(h)), "mkf_mixkf_create")
        self.h = h
        self.n_theta = N.lib().mkf_mixkf_theta_size(h)
        self.det_off = torch.from_numpy(np.ascontiguousarray(batch.det_off, np.int32)).cuda()
        self.det = torch.from_numpy(np.ascontiguousarray(batch.det, np.float32)).cuda()
        self.ll = torch.zeros(nt, dtype=torch.float64, device="cuda")
        self.total = torch.zeros(1, dtype=torch.float64, device="cuda")
        self.grad = torch.zeros(self.n_theta, dtype=torch.float64, device="cuda")

    def set_theta(self, theta):
        if hasattr(theta, "data_ptr"):
            N.check(N.lib().mkf_mixkf_set_theta_device(self.h, _ptr(theta), _stream(self.torch)),
                    "mkf_mixkf_set_theta_device")
        else:
            th = np.ascontiguousarray(theta, np.float64)
            assert th.size == self.n_theta
            N.check(N.lib().mkf_mixkf_set_theta(self.h, th.ctypes.data_as(C.c_void_p)), "mkf_mixkf_set_theta")

    def forward(self, stream=None):
        N.check(N.lib().mkf_mixkf_forward(self.h, _ptr(self.det_off), _ptr(self.det), _ptr(self.ll),
                                          _ptr(self.total), _stream(self.torch, stream)), "mkf_mixkf_forward")
        return self.total

    def backward(self, stream=None):
        N.check(N.lib().mkf_mixkf_backward(self.h, _ptr(self.det_off), _ptr(self.det), _ptr(self.grad),
                                           _stream(self.torch, stream)), "mkf_mixkf_backward")
        return self.grad

    def set_checkpoint_stride(self, C_=0):
        N.check(N.lib().mkf_mixkf_set_checkpoint_stride(self.h, int(C_)), "mkf_mixkf_set_checkpoint_stride")

    @property
    def checkpoint_stride(self):
        return N.lib().mkf_mixkf_checkpoint_stride(self.h)

    def status(self):
        s = C.c_int()
        N.check(N.lib().mkf_mixkf_status(self.h, C.byref(s)), "mkf_mixkf_status")
        return s.value

    def fit_adam(self, theta0, steps, lr=1e-2, mask=None, callback=None, resume=None):
        """Maximise the total logL with Adam on the device (theta, moments, mask
        and gradient stay in HBM; one forward + backward + update per step).
        resume: a FitState (load_fit_state) to continue from: its theta and
        moments replace theta0, and the step count continues after its step.
        Returns (theta, history); self.fit_state holds the state to save."""
        torch = self.torch
        start = 1
        if resume is not None:
            assert resume.theta.size == self.n_theta
            theta0 = resume.theta
            start = resume.step + 1
        th = torch.from_numpy(np.array(theta0, np.float64, order="C", copy=True)).cuda()
        m = torch.zeros_like(th) if resume is None else torch.from_numpy(resume.m.copy()).cuda()
        v = torch.zeros_like(th) if resume is None else torch.from_numpy(resume.v.copy()).cuda()
        mk = None if mask is None else torch.from_numpy(np.ascontiguousarray(mask, np.uint8)).cuda()
        hist = []
        self._fit_tensors = (th, m, v, start - 1, lr)
        for it in range(start, start + steps):
            self.set_theta(th)
            self.forward()
            self.backward()
            N.check(N.lib().mkf_adam_step(_ptr(th), _ptr(self.grad), _ptr(m), _ptr(v), _ptr(mk), self.n_theta, it,
                                          float(lr), 0.9, 0.999, 1e-8, 1, _stream(torch)), "mkf_adam_step")
            self._fit_tensors = (th, m, v, it, lr)
            if callback is not None:
                callback(it, th, self.total)
            hist.append(self.total)
        return th, hist

    @property
    def fit_state(self):
        th, m, v, step, lr = self._fit_tensors
        return FitState(th.cpu().numpy(), m.cpu().numpy(), v.cpu().numpy(), step, lr, self.K, self.d)

    def __del__(self):
        try:
            if getattr(self, "h", None):
                N.lib().mkf_mixkf_destroy(self.h)
                self.h = None
        except Exception:
            pass
