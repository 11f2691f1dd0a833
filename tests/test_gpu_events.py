"""The GPU labeler's event counts equal the CPU restatement's.

The algorithmic bytes of the labeling loop are a per-event formula over the
reference algorithm's events (edges scanned in push, BP tests, label entries
read by distance tests, labels appended, queue entries), counted by the
oracle, which follows the reference's own push order.  Two of those events
are the same in the GPU's pull formulation, so the device counts them too in
profile mode: first offers of a root to a tail within a batch (each is one BP
test, pado_unw_unv_unp.h:580-623) and labels appended (self labels included,
:729-775).  Equal counts tie the device run to the events the formula counts.
"""
import ctypes as C

import pytest

from oracle import orc
from parallel_distance_oracle_gb300 import graphs as G

pytestmark = pytest.mark.gpu


def _profile(lib):
    need = lib.pado_profile_read(None, 0, 0)
    buf = C.create_string_buffer(need + 16)
    lib.pado_profile_read(buf, len(buf), 1)
    out = {}
    for ln in buf.value.decode().splitlines():
        name, launches, ms, count = ln.split()
        out[name] = int(count)
    return out


@pytest.mark.parametrize("scale,ef,seed,K,B", [(14, 8, 1, 50, 1024), (12, 16, 3, 64, 256), (11, 8, 5, 16, 64)])
def test_device_events_equal_oracle_events(cuda_ok, scale, ef, seed, K, B):
    from parallel_distance_oracle_gb300 import _lib, pado
    g = G.rmat(scale, ef, seed)
    rank = G.degree_rank(g)
    ref = orc.unw_label(g, rank, K, B).stats
    _lib.lib.pado_profile_read(None, 0, 1)  # clears what earlier calls left in the table
    _lib.check(_lib.lib.pado_profile(1))
    try:
        idx = pado.VertexCentricPLL(g, rank, bp_roots=K, batch=B)
        got = _profile(_lib.lib)
    finally:
        _lib.check(_lib.lib.pado_profile(0))
    assert got["events.labels_appended"] == ref["labels_added"] == idx.info().num_labels
    assert got["events.first_offers"] == ref["bp_checks"]
