"""End-to-end through the drop-in C++ header on the GPU: a driver written the
way the reference's drivers use the labeler classes labels a graph file,
stores the index in the reference's format, reloads it and answers pairs on
stdin; answers must equal BFS / Dijkstra.  Where unmodified copies of the
reference's own pado.cpp / query_distance.cpp were staged, they are built
against the drop-in header and run the same way."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from dropin.build_dropin import build
from oracle import build_oracle, orc
from parallel_distance_oracle_gb300 import graphs as G

pytestmark = pytest.mark.gpu

STAGED = build_oracle.REF_OUT / "drivers"


def write_edges(path: Path, g, weighted=False):
    src = np.repeat(np.arange(g.n), np.diff(g.off).astype(np.int64))
    keep = src < g.adj
    lines = []
    for u, v, k in zip(src[keep], g.adj[keep], np.nonzero(keep)[0]):
        lines.append(f"{u} {v} {int(g.w[k])}" if weighted else f"{u} {v}")
    path.write_text("\n".join(lines) + "\n")


def run_pairs(exe_args, pairs, cwd):
    inp = "\n".join(f"{a} {b}" for a, b in pairs) + "\n"
    r = subprocess.run(exe_args, input=inp, capture_output=True, text=True, cwd=cwd, timeout=300, check=True)
    return [int(x) for x in r.stdout.split() if x.lstrip("-").isdigit()]


@pytest.mark.parametrize("weighted", [False, True])
def test_dropin_driver_label_store_load_query(cuda_ok, tmp_path, weighted):
    exe = build(tmp_path)
    g = G.rmat(11, 8, 21, weights=(1, 100) if weighted else None)
    # the text loader sets n = max id + 1; keep only the vertices it will see
    edges = tmp_path / "g.txt"
    write_edges(edges, g, weighted)
    idx = tmp_path / "g.idx"
    w = ["-w", "1" if weighted else "0"]
    subprocess.run([str(exe), "label", str(edges), str(idx)] + w, check=True, timeout=300, capture_output=True)
    a, b = G.random_pairs(g.n, 400, 3)
    got = run_pairs([str(exe), "query", str(idx)] + w, list(zip(a, b)), tmp_path)
    assert len(got) == 400
    for i in range(0, 400, 8):
        truth = orc.dijkstra(g, int(a[i]))[b[i]] if weighted else orc.bfs(g, int(a[i]))[b[i]]
        assert got[i] == truth


@pytest.mark.skipif(not (STAGED / "pado.cpp").exists(), reason="reference drivers not staged on this host")
def test_reference_drivers_on_gpu(cuda_ok, tmp_path):
    shim = tmp_path / "shim"
    shim.mkdir()
    for h in ["pado_unw_unv_para.201912311607.parallel_bp_labeling.h", "pado_unw_unv_unp.h", "pado_unw_vec_unp.h",
              "pado_unw_vec_para.h", "pado_weighted_unv_unp.h", "pado_weighted_vec_unp.h", "pado_weighted_unv_para.h",
              "pado_weighted_vec_para.h"]:
        (shim / h).write_text('#include "pado_gpu.hpp"\n')
    inc = [shim, build_oracle.REF_INC]
    pado_exe = build(tmp_path, sources=[STAGED / "pado.cpp"], extra_includes=inc, name="pado")
    q_exe = build(tmp_path, sources=[STAGED / "query_distance.cpp"], extra_includes=inc, name="query_distance")
    for weighted in (False, True):
        g = G.rmat(10, 8, 22, weights=(1, 100) if weighted else None)
        edges = tmp_path / "r.txt"
        write_edges(edges, g, weighted)
        idx = tmp_path / "r.idx"
        w = ["-w", "1" if weighted else "0"]
        subprocess.run([str(pado_exe), str(edges), str(idx)] + w + ["-v", "0", "-p", "0"], check=True, timeout=300,
                       capture_output=True)
        a, b = G.random_pairs(g.n, 200, 4)
        got = run_pairs([str(q_exe), str(idx)] + w, list(zip(a, b)), tmp_path)
        for i in range(0, 200, 5):
            truth = orc.dijkstra(g, int(a[i]))[b[i]] if weighted else orc.bfs(g, int(a[i]))[b[i]]
            assert got[i] == truth
