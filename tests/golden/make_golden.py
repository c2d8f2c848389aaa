"""Regenerate tests/golden/ from the reference checkout (run in the build
container, where the reference is mounted; the test machines never run this).

ref_models.npz: both arms' shipped model parameters (data13D/data23D
_PCA_100000_15_12.yml) as the reference's constructor reads them, including
its quirk of taking gamma for both arms from the right-arm file
(pfPose.cpp:52-53), plus the Kinect K of pfPose.cpp:101 and the cal.yml camera.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from mkfbodytracker_pdaf_gb300 import cvyaml  # noqa: E402

def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <reference checkout>")
    ref = sys.argv[1]
    arms = cvyaml.load_reference_models(os.path.join(ref, "data13D_PCA_100000_15_12.yml"),
                                        os.path.join(ref, "data23D_PCA_100000_15_12.yml"))
    raw_left_gamma = cvyaml.load(os.path.join(ref, "data13D_PCA_100000_15_12.yml"))["gamma"].ravel()
    cal = cvyaml.load(os.path.join(ref, "cal.yml"))
    out = {}
    for a, arm in enumerate(arms):
        for k, v in arm.items():
            out["arm%d_%s" % (a, k)] = v
    out["arm0_gamma_own_file"] = raw_left_gamma
    out["cal_camera_matrix"] = cal["camera_matrix"]
    out["cal_distortion"] = cal["distortion_coefficients"]
    out["kinect_K"] = np.array([[525.0, 0.0, 319.5], [0.0, 525.0, 239.5], [0.0, 0.0, 1.0]])
    np.savez_compressed(os.path.join(HERE, "ref_models.npz"), **out)
    print("wrote", os.path.join(HERE, "ref_models.npz"), sorted(out))


if __name__ == "__main__":
    main()
