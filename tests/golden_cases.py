"""Loading helpers for the golden fixtures written by tests/golden/make_golden.py."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def meta():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        return json.load(f)


def reshape_case(name):
    m = meta()["reshape"][name]
    z = np.load(os.path.join(GOLDEN, "reshape_%s.npz" % name))
    return m, z["src"], z["out"], z["fill"]


def split_case(name):
    m = meta()["split"][name]
    z = np.load(os.path.join(GOLDEN, "split_%s.npz" % name))
    return m, {k: z[k] for k in z.files}


def reshape_names():
    return sorted(meta()["reshape"])


def split_names():
    return sorted(meta()["split"])
