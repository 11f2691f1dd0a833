"""Index files in the reference's on-disk format, pinned to files the
reference itself wrote (tests/golden/idxfile_*.npz, made by
make_golden.py --index-files with the reference's store_index_to_file,
pado_unw_unv_unp.h:1120-1180 / pado_weighted_unv_unp.h:1639-1676).

CPU checks: the oracle's writer produces the same bytes; a plain parser of the
format recovers exactly the golden canonical labels; and, where the
reference's own driver is built on this host, its load_index_from_file reads an
oracle-written file and answers the golden pairs as the labeler's index does.
The GPU library's writer and loader are checked against the same files in
test_gpu_index_files.py."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN
from helpers import load_golden
from oracle import orc

CASES = sorted(GOLDEN.glob("idxfile_*.npz"))


def parse_index(raw: bytes, weighted: bool):
    """(n, K, off, hub, dist, bpd, bps) of an index file, per original vertex."""
    buf = memoryview(raw)
    pos = 0

    def take(dt, count):
        nonlocal pos
        a = np.frombuffer(buf, dtype=dt, count=count, offset=pos)
        pos += a.nbytes
        return a

    n = int(take("<u4", 1)[0])
    K = 0 if weighted else int(take("<u4", 1)[0])
    bp_row = np.dtype([("d", "u1"), ("s", "<u8", 2)])
    lab = np.dtype([("h", "<u4"), ("d", "<i2" if weighted else "u1")])
    off = np.zeros(n + 1, np.uint64)
    hubs, dists, bpd, bps = [], [], [], []
    for v in range(n):
        if K:
            rows = take(bp_row, K)
            bpd.append(rows["d"])
            bps.append(rows["s"].reshape(-1))
        cnt = int(take("<u4", 1)[0])
        ent = take(lab, cnt)
        hubs.append(ent["h"])
        dists.append(ent["d"])
        off[v + 1] = off[v] + cnt
    assert pos == len(raw), "trailing bytes"
    cat = lambda xs, dt: np.concatenate(xs).astype(dt) if xs else np.zeros(0, dt)  # noqa: E731
    return (n, K, off, cat(hubs, np.uint32), cat(dists, np.int16 if weighted else np.uint8), cat(bpd, np.uint8),
            cat(bps, np.uint64))


def _case(path):
    f = np.load(path)
    z, g = load_golden(GOLDEN / f"{str(f['case'])}.npz")
    return f, z, g, int(z["kind"]) == 1


@pytest.mark.parametrize("path", CASES, ids=lambda p: p.stem)
def test_reference_file_holds_the_golden_labels(path):
    f, z, g, weighted = _case(path)
    n, K, off, hub, dist, bpd, bps = parse_index(f["raw"].tobytes(), weighted)
    assert n == g.n and K == int(z["K"])
    assert np.array_equal(off, z["l_off"].astype(np.uint64))
    assert np.array_equal(hub, z["l_hub"])
    assert np.array_equal(dist.astype(np.int64), z["l_dist"].astype(np.int64))
    if K:
        assert np.array_equal(bpd, z["l_bpd"]) and np.array_equal(bps, z["l_bps"])
    # the reloaded reference index answers as the labeler's own index
    assert np.array_equal(f["qd"], z["qd"])


def _oracle_file(g, z, weighted, out):
    lib = orc.port()
    off, adj, rank = np.ascontiguousarray(g.off, np.uint64), np.ascontiguousarray(g.adj, np.uint32), \
        np.ascontiguousarray(z["rank"], np.uint32)
    if weighted:
        h = lib.orc_w_build(g.n, off, adj, np.ascontiguousarray(g.w, np.uint8), rank, int(z["B"]), 0)
        assert lib.orc_w_store(h, str(out).encode()) == 0
        lib.orc_w_free(h)
    else:
        h = lib.orc_unw_build(g.n, off, adj, rank, int(z["K"]), int(z["B"]))
        assert lib.orc_unw_store(h, str(out).encode()) == 0
        lib.orc_unw_free(h)


@pytest.mark.parametrize("path", CASES, ids=lambda p: p.stem)
def test_oracle_writer_equals_reference_file(path, tmp_path):
    f, z, g, weighted = _case(path)
    out = tmp_path / "orc.idx"
    _oracle_file(g, z, weighted, out)
    assert out.read_bytes() == f["raw"].tobytes()


@pytest.mark.parametrize("path", CASES, ids=lambda p: p.stem)
def test_reference_loader_reads_oracle_file(path, tmp_path):
    f, z, g, weighted = _case(path)
    K = int(z["K"])
    if not weighted and K not in (50, 64):
        pytest.skip("the reference driver is built for 50 and 64 roots")
    if not orc.ref_available(50 if weighted else K):
        pytest.skip("the reference's driver is not built on this host")
    out = tmp_path / "orc.idx"
    _oracle_file(g, z, weighted, out)
    assert np.array_equal(orc.ref_load_query(out, f["qa"], f["qb"], weighted=weighted, K=K), f["qd"])
