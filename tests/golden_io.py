"""Loading of the golden fixtures (tests/golden/*.npz) and bitwise comparison
helpers shared by the CPU and GPU parity tests."""
from __future__ import annotations

import glob
import os

import numpy as np

from femmd_old_gb300.scene import Scene

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def frame_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "frames", "*.npz")))


def load_frames(name):
    """A writer fixture: the scene, its state dumps, and {file name: bytes}
    of every frame the reference's writers produced."""
    sc, dumps = load(os.path.join("frames", name))
    z = np.load(os.path.join(GOLDEN, "frames", name + ".npz"))
    files = {str(n): z[f"frame{k:03d}"].tobytes() for k, n in enumerate(z["frame_names"])}
    return sc, dumps, files


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    sc = Scene.from_bytes(z["scene"].tobytes())
    dumps = {}
    for key in z.files:
        if key == "scene" or key.startswith("frame"):
            continue
        idx, tag, field = key.split("_", 2)
        k = int(idx[1:])
        dumps.setdefault(k, (tag, {}))[1][field] = z[key]
    return sc, [dumps[k] for k in sorted(dumps)]


def bits(a):
    a = np.asarray(a)
    if a.dtype == np.float32:
        return a.view(np.int32)
    if a.dtype == np.float64:
        return a.view(np.int64)
    return a


def diff_report(ref, got, skip=()):
    """Fields of two dump lists that differ bitwise, as readable strings."""
    out = []
    assert len(ref) == len(got), (len(ref), len(got))
    for k, ((tr, r), (tg, g)) in enumerate(zip(ref, got)):
        assert tr == tg, (k, tr, tg)
        for key, a in r.items():
            if key in skip:
                continue
            b = g[key]
            a = np.asarray(a)
            b = np.asarray(b)
            if a.shape != b.shape:
                out.append(f"dump{k}.{tr}.{key}: shape {a.shape} vs {b.shape}")
            elif not np.array_equal(bits(a), bits(b)):
                d = np.abs(a.astype(np.float64) - b.astype(np.float64))
                i = int(np.argmax(d))
                out.append(f"dump{k}.{tr}.{key}: max|d|={d.max():.3e} at {np.unravel_index(i, a.shape)} "
                           f"ref={a.ravel()[i]!r} got={b.ravel()[i]!r}")
    return out
