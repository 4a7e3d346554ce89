"""Helpers shared by the GPU parity tests."""
import os

import numpy as np

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel_l2(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def load_golden(name):
    return np.load(os.path.join(GOLD, name))


def ensure_built():
    from split_operator_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from split_operator_gb300 import build
        build.build()
