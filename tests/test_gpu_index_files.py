"""Index-file interchange with the reference, on the GPU library's C ABI
(pado_store / pado_load, which replace store_index_to_file,
pado_unw_unv_unp.h:1120-1180 / pado_weighted_unv_unp.h:1639-1676, and
load_index_from_file, pado_unw_unv_unp.h:1182-1224 /
pado_weighted_unv_unp.h:1678-1711):

* the file pado_store writes for a GPU labeling is byte-identical to the file
  the reference's own writer wrote for the same graph, order, K and B
  (tests/golden/idxfile_*.npz);
* pado_load reads the reference-written file and answers the golden pairs as
  the reference's reloaded index does;
* where the reference's driver is built on this host, the reference's own
  loader reads the GPU-written file and answers the same pairs identically.
The full-size files are covered by test_gpu_full_size.py."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN
from helpers import load_golden
from oracle import orc

pytestmark = pytest.mark.gpu

CASES = sorted(GOLDEN.glob("idxfile_*.npz"))


@pytest.fixture(scope="module")
def pado(cuda_ok):
    from parallel_distance_oracle_gb300 import pado as P
    return P


def _case(path):
    f = np.load(path)
    z, g = load_golden(GOLDEN / f"{str(f['case'])}.npz")
    return f, z, g, int(z["kind"]) == 1


def _gpu_file(pado, g, z, weighted, out):
    if weighted:
        idx = pado.WeightedVertexCentricPLL(g, z["rank"], batch=int(z["B"]))
    else:
        idx = pado.VertexCentricPLL(g, z["rank"], bp_roots=int(z["K"]), batch=int(z["B"]))
    idx.store_index_to_file(str(out))
    return idx


@pytest.mark.parametrize("path", CASES, ids=lambda p: p.stem)
def test_gpu_store_equals_reference_file(pado, path, tmp_path):
    f, z, g, weighted = _case(path)
    out = tmp_path / "gpu.idx"
    idx = _gpu_file(pado, g, z, weighted, out)
    assert out.read_bytes() == f["raw"].tobytes()
    assert np.array_equal(idx.query(f["qa"], f["qb"]), f["qd"])


@pytest.mark.parametrize("path", CASES, ids=lambda p: p.stem)
def test_gpu_loads_reference_file(pado, path, tmp_path):
    f, z, g, weighted = _case(path)
    p = tmp_path / "ref.idx"
    p.write_bytes(f["raw"].tobytes())
    idx = pado.WeightedVertexCentricPLL() if weighted else pado.VertexCentricPLL()
    idx.load_index_from_file(str(p))
    assert idx.num_v == g.n
    assert np.array_equal(idx.query(f["qa"], f["qb"]), f["qd"])
    # and writes it back unchanged
    p2 = tmp_path / "again.idx"
    idx.store_index_to_file(str(p2))
    assert p2.read_bytes() == f["raw"].tobytes()


@pytest.mark.parametrize("path", CASES, ids=lambda p: p.stem)
def test_reference_loads_gpu_file(pado, path, tmp_path):
    f, z, g, weighted = _case(path)
    K = int(z["K"])
    if not orc.ref_available(50 if weighted else K):
        pytest.skip("the reference's driver is not built on this host")
    out = tmp_path / "gpu.idx"
    idx = _gpu_file(pado, g, z, weighted, out)
    ref = orc.ref_load_query(out, f["qa"], f["qb"], weighted=weighted, K=K)
    assert np.array_equal(ref, f["qd"])
    assert np.array_equal(ref, idx.query(f["qa"], f["qb"]))
