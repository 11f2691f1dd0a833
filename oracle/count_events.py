"""Event counts of the reference algorithm on the bench workloads (TEST
INFRASTRUCTURE ONLY: the oracle is the counter, nothing here is timed).

The labeling loops' algorithmic bytes are a per-event formula over the
reference algorithm's events, counted by the oracle, which keeps the
reference's push order (pado_unw_unv_unp.h:531-775; weighted
pado_weighted_unv_unp.h:409-870):

  unweighted: 4 B per adjacency entry scanned by push, 17*K B per BP test
    (the tail's BP row), 5 B per label entry read by a distance test, 5 B per
    label appended, 4 B per frontier / candidate queue entry written and again
    read (active heads, candidate vertices, candidate roots);
  weighted: 8 B per adjacency entry scanned (id and weight), 8 B per label
    entry read by a check, 8 B per label appended, 8 B per accepted relaxation.

The counts depend only on the graph, the order, K and B, so they are counted
once and kept in profiles/algorithmic_bytes.md, from which bench.py reads the
terms the device does not count itself (the push-order terms; the BP tests
and labels appended it counts in the same run, and tests/test_gpu_events.py
shows the two counts agree).

Usage:  python oracle/count_events.py [rmat14 rmat20 wrmat18 ...]
"""
from __future__ import annotations

import json
import sys
import time
from pathlib import Path

REPO = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(REPO))

from oracle import orc  # noqa: E402
from parallel_distance_oracle_gb300 import graphs as G  # noqa: E402

# the bench workloads' graphs (bench.py WORKLOADS)
CASES = {
    "rmat14": dict(kind="unw", scale=14, ef=8, seed=1, K=50, B=1024),
    "rmat18": dict(kind="unw", scale=18, ef=16, seed=2, K=64, B=1024),
    "rmat20": dict(kind="unw", scale=20, ef=16, seed=2, K=64, B=1024),
    "wrmat16": dict(kind="w", scale=16, ef=8, seed=3, K=0, B=512),
    "wrmat18": dict(kind="w", scale=18, ef=8, seed=3, K=0, B=512),
}


def unw_bytes(st: dict, K: int) -> dict:
    """Terms of the unweighted formula (bytes)."""
    return {"push_edges": 4 * st["edges_scanned"], "bp_tests": 17 * K * st["bp_checks"],
            "distance_entries": 5 * st["dist_entries"], "labels_appended": 5 * st["labels_added"],
            "queues": 8 * (st["head_visits"] + st["cand_vertices"] + st["dist_checks"])}


def w_bytes(st: dict) -> dict:
    return {"edges": 8 * st["edges_scanned"], "check_entries": 8 * st["check_entries"],
            "labels_appended": 8 * st["labels_added"], "relaxations": 8 * st["relax_accepted"]}


def count(name: str) -> dict:
    c = CASES[name]
    g = G.rmat(c["scale"], c["ef"], c["seed"], weights=(1, 100) if c["kind"] == "w" else None)
    rank = G.degree_rank(g)
    t = time.time()
    if c["kind"] == "unw":
        lab = orc.unw_label(g, rank, c["K"], c["B"])
        terms = unw_bytes(lab.stats, c["K"])
    else:
        lab = orc.w_label(g, rank, c["B"])
        terms = w_bytes(lab.stats)
    return {"workload": name, "events": dict(lab.stats), "bytes": terms, "total_bytes": sum(terms.values()),
            "labels": int(len(lab.hub)), "oracle_seconds": round(time.time() - t, 1)}


if __name__ == "__main__":
    for nm in sys.argv[1:] or list(CASES):
        print(json.dumps(count(nm)), flush=True)
