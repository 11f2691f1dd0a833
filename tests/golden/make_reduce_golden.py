"""Generate tests/golden/reduce_ref.npz from the REFERENCE's own graph-conversion tools.

For every case the two tools compiled from the reference tree
(oracle/build_oracle.py: tools/pseudocode-delete_1-degree_vertices.cpp and
distributed_version/tools/graph-convert/remove_equivalent_vertices.cpp) run
on the case's edge list written as "head tail" lines; stored per case: the
input edge arrays, the edge lines the degree-1 tool writes, and the vertex
count and (head, tail) pairs of the binary file the equivalence tool writes.

Inputs on which the reference's degree-1 walk would never end (the oracle
reports them; isolated paths of four or more vertices can do it, so the mixed
cases keep theirs shorter, and a case that still has one is skipped) are not
given to it.  Needs the reference tree and g++.
Usage:  python tests/golden/make_reduce_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from oracle import build_oracle, orc  # noqa: E402
from parallel_distance_oracle_gb300 import graphs as G  # noqa: E402


def cases():
    rng = np.random.Generator(np.random.PCG64(21))
    yield "tiny", np.array([0, 1, 2, 2, 3, 5, 0, 1], np.uint32), np.array([1, 2, 0, 3, 4, 6, 7, 7], np.uint32)
    for i, n in enumerate((120, 400, 1500)):
        yield f"mix{n}", *G.reduction_edges(n, 30 + i, iso_path_max=3)
    n, m = 40, 120
    yield "multi", rng.integers(0, n, m).astype(np.uint32), rng.integers(0, n, m).astype(np.uint32)
    # a random tree (parent of i drawn from [0, i)), edges in random order
    n = 500
    par = np.array([int(rng.integers(0, i)) for i in range(1, n)], np.uint32)
    kid = np.arange(1, n, dtype=np.uint32)
    o = rng.permutation(n - 1)
    yield "tree", par[o], kid[o]
    _, u, v, _ = G.rmat_edges(10, 8, 4)
    yield "rmat10_raw", u.astype(np.uint32), v.astype(np.uint32)


def main():
    build_oracle.build_port()
    if not build_oracle.build_reference_tools():
        sys.exit("reference tree not found")
    out = {}
    for name, u, v in cases():
        _, _, nonterm = orc.reduce_degree1(u, v)
        if nonterm:
            print(f"{name}: skipped (the reference's degree-1 walk would not end)")
            continue
        d1 = orc.ref_delete_degree1(u, v, timeout=120)
        nv, eq = orc.ref_remove_equivalent(u, v, timeout=120)
        out[f"{name}_u"], out[f"{name}_v"] = u, v
        out[f"{name}_d1"] = d1
        out[f"{name}_eq_nv"] = np.uint32(nv)
        out[f"{name}_eq"] = eq
        print(f"{name}: m={len(u)} degree-1 keeps {len(d1)}, equivalence keeps {len(eq)} edges on {nv} vertices")
    np.savez_compressed(HERE / "reduce_ref.npz", **out)


if __name__ == "__main__":
    main()
