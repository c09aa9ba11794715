"""Shared helpers for the test-suite (fixtures loading, norms)."""
import hashlib
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def topology_json():
    with open(os.path.join(GOLDEN, "topology.json")) as f:
        return json.load(f)


def sha(a):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.int64))
    return hashlib.sha256(a.tobytes() + str(a.shape).encode()).hexdigest()


def rel_norm(a, b):
    """Normwise relative difference ||a-b|| / ||b|| (0 if both are zero)."""
    nb = np.linalg.norm(b)
    d = np.linalg.norm(np.asarray(a) - np.asarray(b))
    return d / nb if nb > 0 else d


def load_test_mesh():
    d = load("test_mesh.npz")
    return d["points"], d["tets"], d["physical"]
