"""Generate tests/golden/ingest_ref.npz from the REFERENCE's own graph code.

For every case the reference builds its Graph / WeightedGraph -- from an edge
list (graph.h:125-153, :292-309) or by reading an edge-list text file
(graph.h:95-117, :262-290) -- and relabels it with id_transfer (graph.h:176-206,
:367-400) under the degree order with ascending-id ties.  Stored per case:
the input (edge arrays, or the text), and the expected n, rank, ranked CSR
offsets, adjacency and weights.  The texts are synthetic and well formed
(comments, tabs, CR before LF, '+' signs, extra columns, a last line with or
without its newline): on such input the reference's reader and the device
parser must agree exactly.

Needs the reference tree and g++ (oracle/build_oracle.py compiles the
driver).  Usage:  python tests/golden/make_ingest_golden.py
"""
from __future__ import annotations

import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from oracle import orc  # noqa: E402
from parallel_distance_oracle_gb300 import graphs as G  # noqa: E402


def synthetic_text(rng, m: int, n: int, weighted: bool, trailing_newline: bool) -> bytes:
    u = rng.integers(0, n, m)
    v = rng.integers(0, n, m)
    w = rng.integers(0, 1000, m)  # above 255 on purpose: cast to uint8
    lines = ["# synthetic edge list", "% second comment style"]
    for i in range(m):
        if rng.random() < 0.05:
            lines.append(f"# note {i}")
        sep = [" ", "\t", "  ", " \t "][int(rng.integers(0, 4))]
        lead = ["", " ", "\t", "+"][int(rng.integers(0, 4))] if rng.random() < 0.3 else ""
        s = f"{lead}{u[i]}{sep}{'+' if rng.random() < 0.1 else ''}{v[i]}"
        if weighted:
            s += f"{sep}{w[i]}"
        if rng.random() < 0.1:
            s += " 7 extra"
        if rng.random() < 0.2:
            s += "\r"
        lines.append(s)
    return ("\n".join(lines) + ("\n" if trailing_newline else "")).encode()


def main():
    rng = np.random.Generator(np.random.PCG64(77))
    out = {}

    def put(name, g, rank, **inputs):
        out[f"{name}_n"] = np.uint32(g.n)
        out[f"{name}_rank"] = rank
        out[f"{name}_off"] = g.off
        out[f"{name}_adj"] = g.adj
        if g.w is not None:
            out[f"{name}_wout"] = g.w
        for k, val in inputs.items():
            out[f"{name}_{k}"] = val
        print(f"{name}: n={g.n} entries={len(g.adj)}")

    # edge lists with repeats and self-loops, as Graph keeps them
    u = rng.integers(0, 40, 300).astype(np.uint32)
    v = rng.integers(0, 40, 300).astype(np.uint32)
    u[::23] = v[::23]
    put("dups_unw", *orc.ref_graph_edges(u, v), u=u, v=v)
    u = rng.integers(0, 50, 400).astype(np.uint32)
    v = rng.integers(0, 50, 400).astype(np.uint32)
    w = rng.integers(0, 256, 400).astype(np.uint8)
    u[::17] = v[::17]
    put("dups_w", *orc.ref_graph_edges(u, v, w), u=u, v=v, w=w)
    # raw R-MAT samples (skewed degrees, many ties, self-loops, repeats)
    n, ru, rv, _ = G.rmat_edges(10, 8, 5)
    ru, rv = ru.astype(np.uint32), rv.astype(np.uint32)
    put("rmat10_raw", *orc.ref_graph_edges(ru, rv), u=ru, v=rv)
    # texts read by the reference's file constructors
    for name, weighted, m, nn, nl in [("text_unw", False, 250, 60, True), ("text_w", True, 250, 60, False),
                                       ("text_unw_nolf", False, 120, 30, False)]:
        text = synthetic_text(rng, m, nn, weighted, nl)
        with tempfile.NamedTemporaryFile("wb", suffix=".txt", delete=False) as f:
            f.write(text)
            path = f.name
        try:
            g, rank = orc.ref_graph_file(path, weighted)
        finally:
            Path(path).unlink()
        put(name, g, rank, text=np.frombuffer(text, np.uint8).copy(), weighted=np.uint8(weighted))
    np.savez_compressed(HERE / "ingest_ref.npz", **out)


if __name__ == "__main__":
    main()
