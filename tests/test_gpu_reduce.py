"""Graph reductions on the device (pado_reduce_degree1, pado_reduce_equivalent
and their device-pointer forms) against the reference's conversion tools (the
fixtures made by tests/golden/make_reduce_golden.py) and the oracle.  Integer
work: flags, new ids, kept edges and counts must be identical.  At the bench's
full size (16.8M raw R-MAT edges) the results are checked by their defining
properties."""
import ctypes as C

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import orc
from parallel_distance_oracle_gb300 import graphs as G

pytestmark = pytest.mark.gpu

CASES = ["tiny", "mix120", "mix400", "mix1500", "multi", "tree", "rmat10_raw"]


@pytest.fixture(scope="module")
def pado(cuda_ok):
    from parallel_distance_oracle_gb300 import pado as P
    return P


def same_as_oracle(pado, u, v, n=None, what=""):
    d, k = pado.reduce_degree1(u, v, n)
    od, ok, _ = orc.reduce_degree1(u, v, n or 0)
    assert np.array_equal(d, od), f"{what}: deleted"
    assert np.array_equal(k, ok), f"{what}: degree-1 kept edges"
    r, nid, k2, n_out = pado.reduce_equivalent(u, v, n)
    orr, onid, ok2, on_out = orc.reduce_equivalent(u, v, n or 0)
    assert np.array_equal(r, orr), f"{what}: redundant"
    assert np.array_equal(nid, onid), f"{what}: new ids"
    assert np.array_equal(k2, ok2), f"{what}: equivalence kept edges"
    assert n_out == on_out, f"{what}: vertex count"


@pytest.mark.parametrize("name", CASES)
def test_reductions_match_reference_golden(pado, name):
    z = np.load(GOLDEN / "reduce_ref.npz")
    u, v = z[f"{name}_u"], z[f"{name}_v"]
    _, kept = pado.reduce_degree1(u, v)
    assert np.array_equal(np.stack([u[kept], v[kept]], 1).reshape(-1, 2), z[f"{name}_d1"]), name
    _, nid, kept, n_out = pado.reduce_equivalent(u, v)
    assert n_out == int(z[f"{name}_eq_nv"])
    assert np.array_equal(np.stack([nid[u[kept]], nid[v[kept]]], 1).reshape(-1, 2), z[f"{name}_eq"]), name


def test_reductions_on_mixed_graphs_equal_oracle(pado):
    # isolated paths up to 8 vertices: where the reference's walk may not end,
    # the oracle's guarded walk (whole path deleted) is the expectation
    for i, n in enumerate((50, 1000, 20000, 200000)):
        u, v = G.reduction_edges(n, 200 + i, iso_path_max=8)
        same_as_oracle(pado, u, v, what=f"mix n={n}")


def test_reductions_on_random_multigraphs_equal_oracle(pado):
    rng = np.random.Generator(np.random.PCG64(5))
    for t in range(30):
        n = int(rng.integers(1, 3000))
        m = int(rng.integers(0, 3 * n + 1))
        u = rng.integers(0, n, m).astype(np.uint32)
        v = rng.integers(0, n, m).astype(np.uint32)
        same_as_oracle(pado, u, v, n=n, what=f"random {t}")


def test_reductions_on_structured_graphs(pado):
    k = 200  # a clique: every set equal, only vertex 0 stays
    iu, iv = np.triu_indices(k, 1)
    same_as_oracle(pado, iu.astype(np.uint32), iv.astype(np.uint32), what="clique")
    r, nid, kept, n_out = pado.reduce_equivalent(iu, iv)
    assert r.sum() == k - 1 and len(kept) == 0 and n_out == 0
    p = np.arange(50000, dtype=np.uint32)  # a long path: both ends walk it
    same_as_oracle(pado, p[:-1], p[1:], what="path")
    d, kept = pado.reduce_degree1(p[:-1], p[1:])
    assert d.all() and len(kept) == 0
    same_as_oracle(pado, np.zeros(300, np.uint32), np.arange(1, 301, dtype=np.uint32), what="star")
    par = np.array([(i - 1) // 2 for i in range(1, 4096)], np.uint32)  # a complete binary tree
    same_as_oracle(pado, par, np.arange(1, 4096, dtype=np.uint32), what="binary tree")
    loops = np.arange(10, dtype=np.uint32)
    same_as_oracle(pado, loops, loops, what="self-loops only")
    same_as_oracle(pado, np.array([3], np.uint32), np.array([7], np.uint32), what="one edge")
    same_as_oracle(pado, np.array([3, 3], np.uint32), np.array([7, 7], np.uint32), what="one edge twice")


def test_reductions_edge_cases(pado):
    e = np.zeros(0, np.uint32)
    d, kept = pado.reduce_degree1(e, e, 5)
    assert d.tolist() == [0] * 5 and len(kept) == 0
    r, nid, kept, n_out = pado.reduce_equivalent(e, e, 5)
    assert r.tolist() == [0] * 5 and nid.tolist() == [0, 1, 2, 3, 4] and n_out == 0
    # n above max id + 1: trailing isolated vertices stay and are numbered
    same_as_oracle(pado, np.array([0, 1], np.uint32), np.array([1, 2], np.uint32), n=9, what="padded n")
    with pytest.raises(RuntimeError):
        pado.reduce_degree1(np.array([0, 5], np.uint32), np.array([1, 2], np.uint32), 4)
    with pytest.raises(RuntimeError):
        pado.reduce_equivalent(np.array([0, 5], np.uint32), np.array([1, 2], np.uint32), 4)


def test_raw_rmat_equals_oracle(pado):
    for scale in (14, 18):
        _, u, v, _ = G.rmat_edges(scale, 16 if scale == 18 else 8, 3)
        same_as_oracle(pado, u.astype(np.uint32), v.astype(np.uint32), what=f"rmat s{scale} raw")


def test_device_pointer_forms_equal_host_forms(pado):
    import torch
    from parallel_distance_oracle_gb300 import _lib
    lib = _lib.lib
    u, v = G.reduction_edges(5000, 9, iso_path_max=5)
    n, m = int(max(u.max(), v.max())) + 1, len(u)
    du = torch.from_numpy(u.view(np.int32)).cuda()
    dv = torch.from_numpy(v.view(np.int32)).cuda()
    flags = torch.zeros(n, dtype=torch.uint8, device="cuda")
    nid = torch.zeros(n, dtype=torch.int32, device="cuda")
    kept = torch.zeros(m, dtype=torch.int64, device="cuda")
    k, n_out = C.c_uint64(), C.c_uint32()
    s = torch.cuda.current_stream()
    _lib.check(lib.pado_reduce_degree1_device(m, du.data_ptr(), dv.data_ptr(), n, flags.data_ptr(),
                                              kept.data_ptr(), C.byref(k), s.cuda_stream))
    d, hk = pado.reduce_degree1(u, v)
    assert np.array_equal(flags.cpu().numpy(), d) and np.array_equal(kept[:k.value].cpu().numpy(), hk)
    _lib.check(lib.pado_reduce_equivalent_device(m, du.data_ptr(), dv.data_ptr(), n, flags.data_ptr(),
                                                 nid.data_ptr(), kept.data_ptr(), C.byref(k), C.byref(n_out),
                                                 s.cuda_stream))
    r, hn, hk, hout = pado.reduce_equivalent(u, v)
    assert np.array_equal(flags.cpu().numpy(), r)
    assert np.array_equal(nid.cpu().numpy().view(np.uint32), hn)
    assert np.array_equal(kept[:k.value].cpu().numpy(), hk) and n_out.value == hout


def test_full_size_properties(pado):
    """The bench's input, 16.8M raw R-MAT s20 samples: every degree-1 vertex
    is deleted, every deleted vertex has at most two entries, the kept edges
    are exactly those without a dropped end; new ids number the vertices that
    stay; every redundant vertex in a sample has the same set as a smaller id."""
    n, u, v, _ = G.rmat_edges(20, 16, 2)
    u, v = u.astype(np.uint32), v.astype(np.uint32)
    deg = np.bincount(u, minlength=n) + np.bincount(v, minlength=n)
    d, kept = pado.reduce_degree1(u, v, n)
    assert np.all(d[deg == 1] == 1) and np.all(deg[d == 1] <= 2)
    ok = (d[u] == 0) & (d[v] == 0)
    assert np.array_equal(kept, np.flatnonzero(ok).astype(np.uint64))
    r, nid, kept, n_out = pado.reduce_equivalent(u, v, n)
    stay = r == 0
    assert np.array_equal(nid[stay], np.arange(stay.sum(), dtype=np.uint32))
    assert np.all(nid[~stay] == 0xffffffff)
    ok = stay[u] & stay[v]
    assert np.array_equal(kept, np.flatnonzero(ok).astype(np.uint64))
    top = int(max(nid[u[kept]].max(), nid[v[kept]].max())) + 1 if len(kept) else 0
    assert n_out == top
    # sets of a sample of redundant vertices, from a sorted entry list
    src = np.concatenate([u, v]).astype(np.int64)
    dst = np.concatenate([v, u]).astype(np.int64)
    o = np.lexsort((dst, src))
    src, dst = src[o], dst[o]
    off = np.zeros(n + 1, np.int64)
    np.cumsum(np.bincount(src, minlength=n), out=off[1:])

    def cset(x):
        return np.sort(np.append(dst[off[x]:off[x + 1]], x))

    red = np.flatnonzero(~stay)
    assert len(red) > 0
    rng = np.random.Generator(np.random.PCG64(1))
    for x in rng.choice(red, size=min(50, len(red)), replace=False):
        sx = cset(x)
        # its class's smallest id is among its own set (equal sets contain each other's ids)
        assert any(np.array_equal(cset(y), sx) for y in sx if y < x), x
