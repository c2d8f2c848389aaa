"""CPU checks of the model-file I/O and the harness file formats: the Python
OpenCV-YAML writer and reader round-trip the shipped models exactly, the C++
reader/writer inside the harness agrees with them, and the frame file layout
is what the harness parses."""
import os
import struct

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _arm(z, a):
    return dict(means=z["arm%d_means" % a], covs=z["arm%d_covs" % a], weights=z["arm%d_weights" % a],
                pca_proj=z["arm%d_pca_proj" % a], pca_mean=z["arm%d_pca_mean" % a], gamma=z["arm%d_gamma" % a])


def test_python_yaml_roundtrip(tmp_path):
    from mkfbodytracker_pdaf_gb300 import cvyaml
    z = np.load(os.path.join(HERE, "golden", "ref_models.npz"))
    p = str(tmp_path / "arm0.yml")
    cvyaml.save_arm_model(p, **_arm(z, 0))
    back = cvyaml.load(p)
    np.testing.assert_array_equal(back["means"], z["arm0_means"])
    np.testing.assert_array_equal(back["covs"], z["arm0_covs"])
    np.testing.assert_array_equal(back["weights"].ravel(), z["arm0_weights"])
    assert back["pca_proj"].dtype == np.float32
    np.testing.assert_array_equal(back["pca_proj"].astype(np.float64), z["arm0_pca_proj"])
    np.testing.assert_array_equal(back["gamma"].ravel(), z["arm0_gamma"])
    doc = cvyaml.parse(cvyaml.dump({"image_width": 640, "scale": 0.5, "m": np.arange(6.0).reshape(2, 3)}))
    assert doc["image_width"] == 640 and doc["scale"] == 0.5
    np.testing.assert_array_equal(doc["m"], np.arange(6.0).reshape(2, 3))


def test_cpp_yaml_roundtrip_matches_python(tmp_path):
    from mkfbodytracker_pdaf_gb300 import build, cvyaml
    exe = build.build_harness()
    z = np.load(os.path.join(HERE, "golden", "ref_models.npz"))
    src, dst = str(tmp_path / "in.yml"), str(tmp_path / "out.yml")
    cvyaml.save_arm_model(src, **_arm(z, 1))
    import subprocess
    r = subprocess.run([exe, "yaml-roundtrip", src, dst], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    a, b = cvyaml.load(src), cvyaml.load(dst)
    assert list(a) == list(b)
    for k in a:
        assert a[k].dtype == b[k].dtype, k
        np.testing.assert_array_equal(a[k], b[k])
    # malformed input is reported, not crashed on
    bad = str(tmp_path / "bad.yml")
    open(bad, "w").write("%YAML:1.0\nm: !!opencv-matrix\n   rows: 2\n   cols: 2\n   dt: d\n   data: [ 1, 2, 3 ]\n")
    r = subprocess.run([exe, "yaml-roundtrip", bad, dst], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "3 values for 2x2" in r.stderr


def test_frame_file_layout(tmp_path):
    from mkfbodytracker_pdaf_gb300 import harness_io
    p = str(tmp_path / "f.bin")
    roi = np.arange(8.0).reshape(2, 4)
    harness_io.write_frames(p, [5, 6], [roi, None], [np.array([[1.0, 2.0], [3.0, 4.0]]), None])
    buf = open(p, "rb").read()
    assert buf[:8] == b"MKFFRM01" and struct.unpack_from("<i", buf, 8)[0] == 2
    fid, has = struct.unpack_from("<ii", buf, 12)
    assert (fid, has) == (5, 1)
    np.testing.assert_array_equal(np.frombuffer(buf, "<f8", 8, 20), np.arange(8.0))
    assert struct.unpack_from("<i", buf, 84)[0] == 2
    np.testing.assert_array_equal(np.frombuffer(buf, "<f8", 4, 88), [1, 2, 3, 4])
    fid, has = struct.unpack_from("<ii", buf, 120)
    assert (fid, has) == (6, 0)
    assert len(buf) == 120 + 8 + 64 + 4


def test_fit_state_file_roundtrip(tmp_path):
    from mkfbodytracker_pdaf_gb300 import mixkf
    st = mixkf.FitState(np.linspace(-1, 1, 37), np.full(37, 0.5), np.full(37, 2.0), 12, 0.02, 2, 12)
    p = str(tmp_path / "fit.bin")
    mixkf.save_fit_state(p, st)
    back = mixkf.load_fit_state(p)
    assert (back.step, back.lr, back.K, back.d) == (12, 0.02, 2, 12)
    for a, b in ((back.theta, st.theta), (back.m, st.m), (back.v, st.v)):
        np.testing.assert_array_equal(a, b)
