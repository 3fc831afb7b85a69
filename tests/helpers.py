"""Comparison helpers shared by the parity tests."""

import os

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def ref_tree():
    """The reference source tree, for the tests that build or read it:
    $CGFD_REF_TREE, else the tree the oracle's reference build used
    (oracle/_ref/ref_tree.txt, written by oracle/Makefile); None when
    neither names an existing directory."""
    path = os.environ.get("CGFD_REF_TREE", "")
    if not path:
        rec = os.path.join(REPO, "oracle", "_ref", "ref_tree.txt")
        if os.path.exists(rec):
            with open(rec) as f:
                path = f.read().strip()
    return path if path and os.path.isdir(path) else None

# tolerances of the parity bar: relative L2 and max-abs relative to the peak
REL_L2 = 1e-5
MAX_ABS_OF_PEAK = 1e-4


def rel_l2(got, ref):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    n = np.linalg.norm(ref)
    return float(np.linalg.norm(got - ref) / n) if n > 0 else float(np.linalg.norm(got))


def max_abs_of_peak(got, ref):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    pk = np.abs(ref).max()
    return float(np.abs(got - ref).max() / pk) if pk > 0 else float(np.abs(got).max())


def assert_parity(got, ref, what=""):
    r, m = rel_l2(got, ref), max_abs_of_peak(got, ref)
    assert r <= REL_L2 and m <= MAX_ABS_OF_PEAK, \
        "%s: rel_l2=%.3e max_abs/peak=%.3e" % (what, r, m)
    return r, m
