"""Serving loop (pado_server_*): continuous batching of query requests over
device-resident label sets, with admission and eviction by an HBM budget.

What must hold: every request's results are exactly pado_query's on the same
pairs (integers, tolerance zero) -- submitted alone, replayed in a mix of
hundreds of concurrent requests of different sizes over several indexes
(unweighted and weighted), split across batches, and after its label set was
evicted to host memory and admitted again."""
import numpy as np
import pytest

from parallel_distance_oracle_gb300 import graphs as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pado(cuda_ok):
    from parallel_distance_oracle_gb300 import pado as P
    return P


@pytest.fixture(scope="module")
def indexes(pado):
    out = []
    g = G.rmat(12, 8, 61)
    out.append((g, pado.VertexCentricPLL(g, G.degree_rank(g), bp_roots=32, batch=256)))
    g = G.grid_with_shortcuts(3000, 0.02, 62)
    out.append((g, pado.VertexCentricPLL(g, G.degree_rank(g), bp_roots=16, batch=512)))
    g = G.erdos_renyi(2500, 6, 63)
    out.append((g, pado.VertexCentricPLL(g, G.degree_rank(g), bp_roots=64, batch=128)))
    g = G.rmat(11, 8, 64, weights=(1, 100))
    out.append((g, pado.WeightedVertexCentricPLL(g, G.degree_rank(g), batch=256)))
    return out


def zipf_pairs(g, k, rng):
    """Endpoints Zipf(1.1) over degree rank (rank 0 = highest degree)."""
    order = np.argsort(G.degree_rank(g))  # rank -> vertex
    ra = np.minimum(rng.zipf(1.1, size=k) - 1, g.n - 1)
    rb = np.minimum(rng.zipf(1.1, size=k) - 1, g.n - 1)
    return order[ra].astype(np.uint32), order[rb].astype(np.uint32)


def make_trace(indexes, nreq, rate, seed, kmax=4096):
    rng = np.random.Generator(np.random.PCG64(seed))
    arrival = np.cumsum(rng.exponential(1.0 / rate, size=nreq))
    ids = rng.integers(0, len(indexes), size=nreq).astype(np.uint32)
    ks = np.exp(rng.uniform(0, np.log(kmax), size=nreq)).astype(np.uint64)
    ks[::17] = 0  # empty requests complete immediately
    aa, bb = [], []
    for i, k in zip(ids, ks):
        a, b = zipf_pairs(indexes[i][0], int(k), rng)
        if k > 2:
            a[0] = indexes[i][0].n + 5  # an out-of-range id is answered like pado_query does
        aa.append(a)
        bb.append(b)
    return arrival, ids, ks, aa, bb


def expected(indexes, ids, aa, bb):
    return [indexes[i][1].query(a, b) for i, a, b in zip(ids, aa, bb)]


def split(out8, out16, indexes, ids, ks):
    res, off = [], 0
    for i, k in zip(ids, ks):
        k = int(k)
        src = out8 if indexes[i][1].kind == 0 else out16
        res.append(src[off:off + k].copy())
        off += k
    return res


def test_alone_equals_pado_query(pado, indexes):
    srv = pado.Server(hbm_budget_bytes=8 << 30)
    ids = [srv.add(ix) for _, ix in indexes]
    rng = np.random.Generator(np.random.PCG64(1))
    for i in ids:
        g, ix = indexes[i]
        for k in (1, 37, 5000):
            a, b = zipf_pairs(g, k, rng)
            got = srv.query(i, a, b)
            assert np.array_equal(got, ix.query(a, b))
    srv.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_mix_equals_alone(pado, indexes, mode):
    arrival, ids, ks, aa, bb = make_trace(indexes, 600, 2e5, 7 + mode)
    want = expected(indexes, ids, aa, bb)
    srv = pado.Server(hbm_budget_bytes=8 << 30, max_batch_pairs=1 << 16, slots=4)
    for _, ix in indexes:
        srv.add(ix)
    a = np.concatenate(aa) if aa else np.zeros(0, np.uint32)
    b = np.concatenate(bb) if bb else np.zeros(0, np.uint32)
    out8, out16, lat = srv.replay(arrival, ids, ks, a, b, mode=mode)
    got = split(out8, out16, indexes, ids, ks)
    for r, (x, y) in enumerate(zip(got, want)):
        assert np.array_equal(x, y), f"request {r} (index {ids[r]}, k={ks[r]})"
    assert (lat >= 0).all()
    st = srv.stats()
    if mode == 0:
        # batching happened: fewer launches than non-empty requests
        assert st["batches"] < int((ks > 0).sum())
    srv.close()


def test_requests_split_across_batches(pado, indexes):
    g, ix = indexes[0]
    srv = pado.Server(hbm_budget_bytes=8 << 30, max_batch_pairs=1000, slots=2)
    i = srv.add(ix)
    rng = np.random.Generator(np.random.PCG64(3))
    a, b = zipf_pairs(g, 7777, rng)
    tickets = [srv.submit(i, a, b) for _ in range(3)]
    for t in tickets:
        out, lat = srv.wait(t)
        assert np.array_equal(out, ix.query(a, b))
    assert srv.stats()["batches"] >= 3 * 8
    srv.close()


def test_eviction_and_readmission_keep_results(pado, indexes):
    sizes = [ix.info().device_bytes for _, ix in indexes]
    budget = max(sizes) + min(sizes) // 2  # room for one large set at a time
    srv = pado.Server(hbm_budget_bytes=budget, max_batch_pairs=1 << 14, slots=3)
    for _, ix in indexes:
        srv.add(ix)
    st0 = srv.stats()
    assert st0["resident_bytes"] <= budget
    assert st0["resident_indexes"] < len(indexes)
    # expected results are computed after close: the server borrows the handles
    arrival, ids, ks, aa, bb = make_trace(indexes, 300, 5e4, 11, kmax=2000)
    a = np.concatenate(aa)
    b = np.concatenate(bb)
    out8, out16, lat = srv.replay(arrival, ids, ks, a, b, mode=0)
    st = srv.stats()
    assert st["evictions"] > 0 and st["admissions"] > 0
    assert st["resident_bytes"] <= budget
    srv.close()
    # handles are resident again and answer directly
    want = expected(indexes, ids, aa, bb)
    got = split(out8, out16, indexes, ids, ks)
    for r, (x, y) in enumerate(zip(got, want)):
        assert np.array_equal(x, y), f"request {r}"


def test_offloaded_handle_refuses_direct_queries(pado, indexes):
    from parallel_distance_oracle_gb300 import _lib
    (g0, ix0), (g1, ix1) = indexes[0], indexes[1]
    qa, qb = np.arange(50, dtype=np.uint32), np.arange(50, dtype=np.uint32)[::-1].copy()
    before = ix0.query(qa, qb)
    budget = max(ix0.info().device_bytes, ix1.info().device_bytes) + 1
    srv = pado.Server(hbm_budget_bytes=budget)
    srv.add(ix0)
    srv.add(ix1)  # evicts ix0, the least recently used
    assert srv.stats()["resident_indexes"] == 1
    with pytest.raises(_lib.PadoError, match="offloaded"):
        ix0.query(np.array([0], np.uint32), np.array([1], np.uint32))
    srv.close()
    assert np.array_equal(ix0.query(qa, qb), before)


def test_bad_requests(pado, indexes):
    from parallel_distance_oracle_gb300 import _lib
    g, ix = indexes[0]
    qa, qb = np.arange(50, dtype=np.uint32), np.arange(50, dtype=np.uint32)[::-1].copy()
    before = ix.query(qa, qb)
    srv = pado.Server(hbm_budget_bytes=ix.info().device_bytes - 1)
    i = srv.add(ix)  # larger than the budget: offloaded at once, requests fail
    with pytest.raises(_lib.PadoError):
        srv.query(i, np.array([0], np.uint32), np.array([1], np.uint32))
    with pytest.raises(_lib.PadoError, match="unknown index"):
        srv.submit(99, np.array([0], np.uint32), np.array([1], np.uint32))
    srv.close()
    assert np.array_equal(ix.query(qa, qb), before)
