"""Reader for the OpenCV FileStorage YAML subset used by the tracker's model
and camera files (``!!opencv-matrix`` with rows/cols/dt/data, plain mappings
with rows/cols/data, and scalars).

The reference loads its models with ``cv::FileStorage`` (pfPose.cpp:34-55);
OpenCV is not available here, so this is the in-repo replacement.  Model
semantics follow pfPose.cpp:37-65: per arm ``means`` (K x d), ``covs``
(K*d x d, K stacked d x d blocks), ``weights`` (1 x K), ``pca_proj`` (d x F,
float in the file, converted to double), ``pca_mean`` (1 x F) and ``gamma``
(K x 1).  Note the reference reads ``gamma`` for BOTH arms from the second
(right-arm) file (pfPose.cpp:52-53); ``load_reference_models`` reproduces that
by default.
"""
from __future__ import annotations

import re

import numpy as np

_DT = {"d": np.float64, "f": np.float32, "i": np.int32, "u": np.uint8, "s": np.int16, "w": np.uint16,
       "c": np.int8}


def _scalar(v):
    v = v.strip()
    if v.startswith('"') and v.endswith('"'):
        return v[1:-1]
    try:
        if re.fullmatch(r"[-+]?\d+", v):
            return int(v)
        return float(v)
    except ValueError:
        return v


def parse(text: str) -> dict:
    lines = text.splitlines()
    out = {}
    i = 0
    n = len(lines)
    while i < n:
        line = lines[i]
        if not line.strip() or line.lstrip().startswith("%") or line.lstrip().startswith("#") \
                or line.strip() == "---":
            i += 1
            continue
        if line[0] in " \t":
            raise ValueError("unexpected indentation at line %d" % (i + 1))
        key, _, rest = line.partition(":")
        key = key.strip()
        rest = rest.strip()
        i += 1
        if rest and not rest.startswith("!!"):
            out[key] = _scalar(rest)
            continue
        # mapping (optionally tagged !!opencv-matrix)
        fields = {}
        while i < n and (lines[i].startswith(" ") or lines[i].startswith("\t") or not lines[i].strip()):
            sub = lines[i].strip()
            i += 1
            if not sub:
                continue
            k2, _, v2 = sub.partition(":")
            k2 = k2.strip()
            v2 = v2.strip()
            if k2 == "data":
                buf = v2
                while "]" not in buf and i < n:
                    buf += " " + lines[i].strip()
                    i += 1
                inner = buf[buf.index("[") + 1:buf.rindex("]")]
                fields["data"] = [float(t) for t in inner.replace(",", " ").split()]
            else:
                fields[k2] = _scalar(v2)
        if "rows" in fields and "cols" in fields and "data" in fields:
            dt = _DT.get(str(fields.get("dt", "d")), np.float64)
            arr = np.asarray(fields["data"], dtype=np.float64).astype(dt)
            if arr.size != fields["rows"] * fields["cols"]:
                raise ValueError("matrix %s: %d values for %dx%d" % (key, arr.size, fields["rows"],
                                                                     fields["cols"]))
            out[key] = arr.reshape(fields["rows"], fields["cols"])
        else:
            out[key] = fields
    return out


def load(path: str) -> dict:
    with open(path, "r") as f:
        return parse(f.read())


def load_reference_models(left_path: str, right_path: str, gamma_from_right: bool = True):
    """Both arms' models as the reference's PFTracker constructor reads them."""
    fs1, fs2 = load(left_path), load(right_path)
    arms = []
    for fs in (fs1, fs2):
        arms.append(dict(means=fs["means"].astype(np.float64), covs=fs["covs"].astype(np.float64),
                         weights=fs["weights"].astype(np.float64).ravel(),
                         pca_proj=fs["pca_proj"].astype(np.float64),
                         pca_mean=fs["pca_mean"].astype(np.float64).ravel(),
                         gamma=fs["gamma"].astype(np.float64).ravel()))
    if gamma_from_right:
        arms[0]["gamma"] = arms[1]["gamma"].copy()
    return arms


def dump(doc: dict) -> str:
    """OpenCV FileStorage YAML text for a dict of numpy matrices (written as
    ``!!opencv-matrix``; float32 arrays get dt f, everything else dt d, 1-D
    arrays become 1 x n) and scalars.  ``parse(dump(doc))`` returns the same
    values: 17 significant digits for doubles, 9 for floats."""
    out = ["%YAML:1.0"]
    for key, v in doc.items():
        if isinstance(v, (int, float, str)) and not isinstance(v, bool):
            out.append("%s: %s" % (key, v if not isinstance(v, float) else repr(v)))
            continue
        a = np.asarray(v)
        if a.ndim == 1:
            a = a.reshape(1, -1)
        if a.ndim != 2:
            raise ValueError("%s: only 2-D matrices are written" % key)
        dt = "f" if a.dtype == np.float32 else "d"
        fmt = "%.9g" if dt == "f" else "%.17g"
        vals = [fmt % x for x in a.astype(np.float64).ravel()]
        lines = [", ".join(vals[i:i + 2]) for i in range(0, len(vals), 2)]
        out.append("%s: !!opencv-matrix\n   rows: %d\n   cols: %d\n   dt: %s\n   data: [ %s ]"
                   % (key, a.shape[0], a.shape[1], dt, ",\n       ".join(lines)))
    return "\n".join(out) + "\n"


def save(path: str, doc: dict) -> None:
    with open(path, "w") as f:
        f.write(dump(doc))


def save_arm_model(path: str, means, covs, weights, pca_proj, pca_mean, gamma) -> None:
    """One arm's model file in the layout the tracker reads (pfPose.cpp:37-53):
    means K x d, covs (K*d) x d, weights 1 x K, pca_proj d x F (float, as
    shipped), pca_mean 1 x F, gamma K x 1."""
    means = np.asarray(means, np.float64)
    K, d = means.shape
    save(path, {"means": means,
                "covs": np.asarray(covs, np.float64).reshape(K * d, d),
                "weights": np.asarray(weights, np.float64).reshape(1, K),
                "pca_proj": np.asarray(pca_proj, np.float32),
                "pca_mean": np.asarray(pca_mean, np.float64).reshape(1, -1),
                "gamma": np.asarray(gamma, np.float64).reshape(K, 1)})
