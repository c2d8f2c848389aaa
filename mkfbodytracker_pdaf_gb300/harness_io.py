"""Frame and output files of the standalone C++ harness (mkf_harness), the
ROS-free stand-in for the reference node's synchronised (image, likelihood,
ROI) input and its HFPose2DArray / TF output (pfPose.cpp:16-21, 173-208).

Frame file: b"MKFFRM01", int32 n, then per frame int32 id, int32 has_roi,
float64 roi[8] (x_offset, y_offset, width, height per arm), int32 M,
float64 cand[2M].  Version b"MKFFRM02" adds int32 W, H after n and a W x H
uint8 likelihood image after each frame's candidates (the image path).
Output file: b"MKFOUT01", int32 n, d, F, then per frame
int32 id, int32 valid, float64 est[2][d], e[2][F], points[8][2] (hand1, hand2,
head, neck, elbow1, elbow2, shoulder1, shoulder2), pos3d[2][3][5]."""
from __future__ import annotations

import os
import struct
import subprocess

import numpy as np

HARNESS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "harness", "mkf_harness")


def write_frames(path, frame_ids, rois, cands, images=None):
    """rois[t]: (2, 4) array or None (no face); cands[t]: (M, 2) array or None;
    images (optional): per-frame (H, W) uint8 likelihood images (version 2)."""
    with open(path, "wb") as f:
        f.write(b"MKFFRM02" if images is not None else b"MKFFRM01")
        f.write(struct.pack("<i", len(frame_ids)))
        if images is not None:
            H, W = np.asarray(images[0]).shape
            f.write(struct.pack("<ii", W, H))
        for t, (fid, roi, c) in enumerate(zip(frame_ids, rois, cands)):
            c = np.zeros((0, 2)) if c is None else np.asarray(c, np.float64).reshape(-1, 2)
            f.write(struct.pack("<ii", int(fid), 0 if roi is None else 1))
            r = np.zeros(8) if roi is None else np.asarray(roi, np.float64).reshape(8)
            f.write(r.astype("<f8").tobytes())
            f.write(struct.pack("<i", c.shape[0]))
            f.write(c.astype("<f8").tobytes())
            if images is not None:
                f.write(np.ascontiguousarray(images[t], np.uint8).tobytes())


def read_output(path):
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:8] != b"MKFOUT01":
        raise ValueError("not a harness output file")
    n, d, F = struct.unpack_from("<iii", buf, 8)
    off = 20
    rec = np.dtype([("id", "<i4"), ("valid", "<i4"), ("est", "<f8", (2, d)), ("e", "<f8", (2, F)),
                    ("points", "<f8", (8, 2)), ("pos3d", "<f8", (2, 3, 5))])
    return np.frombuffer(buf, dtype=rec, count=n, offset=off)


def run_track(arm1_yml, arm2_yml, frames_path, out_path, particles=500, seed=0, pa=0.05, clutter=1e-4,
              own_gamma=False, timeout=600):
    cmd = [HARNESS, "track", "--arm1", arm1_yml, "--arm2", arm2_yml, "--frames", frames_path, "--out", out_path,
           "--particles", str(particles), "--seed", str(seed), "--pa", repr(pa), "--clutter", repr(clutter)]
    if own_gamma:
        cmd.append("--own-gamma")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=timeout)
    if r.returncode:
        raise RuntimeError("mkf_harness failed (%d): %s" % (r.returncode, r.stderr.strip()))
    return r.stdout.strip()
