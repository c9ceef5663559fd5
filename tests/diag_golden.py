"""Shared loader and comparison for the reference-generated diagnostics fixtures
(tests/golden/diag_reference.*, written by tests/golden/make_diag_golden.py)."""
import json
import math
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load():
    z = np.load(os.path.join(GOLDEN, "diag_reference.npz"))
    with open(os.path.join(GOLDEN, "diag_reference.json")) as f:
        meta = json.load(f)
    return z, meta


class Field:
    """The to_numpy() surface the reference's diagnostics read."""

    def __init__(self, a):
        self.a = a

    def to_numpy(self):
        return self.a.copy()


class Holder:
    pass


class Pour:
    def __init__(self, rate):
        self.rate = rate

    def get_current_flow_rate(self):
        return self.rate


def compare(ours, ref, path="", rtol=5e-5, atol=1e-6, loose=()):
    """Every key of the reference's report present in ours with the same value: strings and
    integers exactly, floats to the reference's FP32 precision (it reduces float32 arrays with
    numpy).  `loose` lists keys compared to an absolute 1e-2 (sums of ~4,000 float32 values)."""
    if isinstance(ref, dict):
        assert isinstance(ours, dict), path
        assert set(ref) <= set(ours), (path, sorted(set(ref) - set(ours)))
        for k in ref:
            compare(ours[k], ref[k], path + "/" + k, rtol, atol, loose)
    elif isinstance(ref, list):
        assert len(ours) == len(ref), path
        for i, (a, b) in enumerate(zip(ours, ref)):
            compare(a, b, "%s[%d]" % (path, i), rtol, atol, loose)
    elif isinstance(ref, str) or isinstance(ref, bool):
        assert ours == ref, (path, ours, ref)
    elif isinstance(ref, int):
        assert int(ours) == ref, (path, ours, ref)
    else:
        tol = 1e-2 if path.split("/")[-1].split("[")[0] in loose else atol
        assert math.isclose(float(ours), float(ref), rel_tol=rtol, abs_tol=tol), (path, ours, ref)
