"""Full-size parity: the GPU labels of the three headline graphs (R-MAT s14 /
K=50, R-MAT s20 ef16 / K=64 / B=1024, weighted R-MAT s18 / B=512) hash to the
same SHA-256 as the reference's own OpenMP labeler's labels on the same
inputs.  The digests, label counts and the reference's run times were made by
tests/golden/make_golden.py --digests from the compiled reference; the hash
covers the canonical arrays (offsets, hubs, distances and, unweighted, the BP
rows), so equal digests mean bit-identical label sets."""
import json

import numpy as np
import pytest

from conftest import GOLDEN
from parallel_distance_oracle_gb300 import graphs as G

pytestmark = pytest.mark.gpu

CASES = json.loads((GOLDEN / "full_size_digests.json").read_text())


def digest(kind, off, hub, dist, bpd=None, bps=None):
    import hashlib
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(off, np.uint64).tobytes())
    h.update(np.ascontiguousarray(hub, np.uint32).tobytes())
    h.update(np.ascontiguousarray(dist, np.uint8 if kind == "unw" else np.int16).tobytes())
    if bpd is not None and len(bpd):
        h.update(np.ascontiguousarray(bpd, np.uint8).tobytes())
        h.update(np.ascontiguousarray(bps, np.uint64).tobytes())
    return h.hexdigest()


@pytest.mark.parametrize("name", sorted(CASES))
def test_full_size_labels_match_reference_digest(cuda_ok, name):
    from parallel_distance_oracle_gb300 import pado
    c = CASES[name]
    w = (1, 100) if c["kind"] == "w" else None
    g = G.rmat(c["scale"], c["ef"], c["seed"], weights=w)
    rank = G.degree_rank(g)
    if c["kind"] == "unw":
        idx = pado.VertexCentricPLL(g, rank, bp_roots=c["K"], batch=c["B"])
        lab = idx.export()
        got = digest("unw", lab.off, lab.hub, lab.dist, lab.bpd, lab.bps)
    else:
        idx = pado.WeightedVertexCentricPLL(g, rank, batch=c["B"])
        lab = idx.export()
        got = digest("w", lab.off, lab.hub, lab.dist)
    assert int(idx.info().num_labels) == c["labels"]
    assert got == c["sha256"]
