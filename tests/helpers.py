"""Shared helpers for the test suite."""
from __future__ import annotations

import numpy as np

from parallel_distance_oracle_gb300 import graphs as G
from oracle import orc


def load_golden(path):
    z = np.load(path)
    g = G.CSRGraph(n=int(z["n"]), off=z["off"], adj=z["adj"], w=z["w"] if "w" in z.files else None)
    return z, g


def golden_unw_labels(z) -> orc.UnwLabels:
    return orc.UnwLabels(int(z["n"]), int(z["K"]), z["l_off"], z["l_hub"], z["l_dist"], z["l_bpd"], z["l_bps"])


def golden_w_labels(z) -> orc.WLabels:
    return orc.WLabels(int(z["n"]), z["l_off"], z["l_hub"], z["l_dist"])


def assert_same_unw(a, b, what=""):
    assert a.n == b.n, what
    assert np.array_equal(np.asarray(a.off, np.uint64), np.asarray(b.off, np.uint64)), f"{what}: label counts differ"
    assert np.array_equal(np.asarray(a.hub, np.uint32), np.asarray(b.hub, np.uint32)), f"{what}: hubs differ"
    assert np.array_equal(np.asarray(a.dist, np.uint8), np.asarray(b.dist, np.uint8)), f"{what}: distances differ"
    if a.K:
        assert np.array_equal(np.asarray(a.bpd, np.uint8), np.asarray(b.bpd, np.uint8)), f"{what}: BP dists differ"
        assert np.array_equal(np.asarray(a.bps, np.uint64), np.asarray(b.bps, np.uint64)), f"{what}: BP sets differ"


def assert_same_w(a, b, what=""):
    assert a.n == b.n, what
    assert np.array_equal(np.asarray(a.off, np.uint64), np.asarray(b.off, np.uint64)), f"{what}: label counts differ"
    assert np.array_equal(np.asarray(a.hub, np.uint32), np.asarray(b.hub, np.uint32)), f"{what}: hubs differ"
    assert np.array_equal(np.asarray(a.dist, np.int64), np.asarray(b.dist, np.int64)), f"{what}: distances differ"
