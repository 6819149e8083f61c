"""Helpers to read the golden fixtures (tests/golden/rtm_golden.npz)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "rtm_golden.npz")
INT_KEYS = ("nx", "nz", "th_left", "th_right", "th_up", "th_down", "nt", "n_wavelet", "shot_x",
            "shot_z", "rec_first", "rec_spacing", "rec_count", "rec_depth", "time_slices")


def load():
    return np.load(GOLDEN)


def case_params(d, name):
    iv = d[name + "/params"]
    fv = d[name + "/fparams"]
    p = {k: int(v) for k, v in zip(INT_KEYS, iv)}
    p["dx"], p["dt"] = float(fv[0]), float(fv[1])
    return p


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / den) if den > 0 else float(np.linalg.norm(a - b))
