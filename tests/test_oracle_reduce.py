"""The oracle's graph reductions (orc_reduce_degree1, orc_reduce_equivalent)
are pinned to the reference's own conversion tools: the committed fixtures
made by tests/golden/make_reduce_golden.py, and -- where the reference tree is
present and the tools compiled -- the tools run directly on random edge lists.
The C ABI's argument checks need no GPU."""
import ctypes as C

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import orc
from parallel_distance_oracle_gb300 import graphs as G

CASES = ["tiny", "mix120", "mix400", "mix1500", "multi", "tree", "rmat10_raw"]


def golden():
    return np.load(GOLDEN / "reduce_ref.npz")


def degree1_lines(u, v, kept):
    return np.stack([u[kept], v[kept]], 1).astype(np.uint32).reshape(-1, 2)


def equivalent_pairs(u, v, new_id, kept):
    return np.stack([new_id[u[kept]], new_id[v[kept]]], 1).astype(np.uint32).reshape(-1, 2)


@pytest.mark.parametrize("name", CASES)
def test_oracle_reductions_match_reference_golden(name):
    z = golden()
    u, v = z[f"{name}_u"], z[f"{name}_v"]
    _, kept, nonterm = orc.reduce_degree1(u, v)
    assert not nonterm
    assert np.array_equal(degree1_lines(u, v, kept), z[f"{name}_d1"]), name
    _, nid, kept, n_out = orc.reduce_equivalent(u, v)
    assert n_out == int(z[f"{name}_eq_nv"]), name
    assert np.array_equal(equivalent_pairs(u, v, nid, kept), z[f"{name}_eq"]), name


def test_oracle_reports_the_references_endless_walk():
    """The path 0-2-3-1 given as "0 2", "3 1", "2 3": the walk from 1 bounces
    between the deleted 3 and 2 for ever in the reference (not run here); the
    restatement ends it, flags it and has deleted the whole path."""
    deleted, kept, nonterm = orc.reduce_degree1(np.array([0, 3, 2]), np.array([2, 1, 3]))
    assert nonterm and deleted.tolist() == [1, 1, 1, 1] and len(kept) == 0
    # the same path given in path order ends normally
    deleted, kept, nonterm = orc.reduce_degree1(np.array([0, 2, 3]), np.array([2, 3, 1]))
    assert not nonterm and deleted.tolist() == [1, 1, 1, 1]


def test_oracle_degree1_rules():
    # a chain stops before a vertex of degree 3; a repeated edge counts twice
    u = np.array([0, 1, 2, 2, 2, 5, 5, 6], np.uint32)
    v = np.array([1, 2, 3, 4, 9, 6, 6, 7], np.uint32)
    deleted, kept, _ = orc.reduce_degree1(u, v)
    # 0 (degree 1) -> 1 (degree 2) -> 2 (degree 4): 0 and 1 go; 3, 4, 9 are
    # leaves of 2; 7 -> 6 has degree 3 (5 twice): only 7 goes
    assert deleted.tolist() == [1, 1, 0, 1, 1, 0, 0, 1, 0, 1]
    assert kept.tolist() == [5, 6]


def test_oracle_equivalent_rules():
    # the triangle 0-1-2: all three sets equal, 0 stays; the star 3-{4,5}:
    # the leaves' sets differ; the triangle 6-7-8 with a self-loop on 8: 7
    # equals 6, 8's multiset has two more 8s and stays
    u = np.array([0, 1, 2, 3, 3, 6, 7, 8, 8], np.uint32)
    v = np.array([1, 2, 0, 4, 5, 7, 8, 6, 8], np.uint32)
    red, nid, kept, n_out = orc.reduce_equivalent(u, v)
    assert red.tolist() == [0, 1, 1, 0, 0, 0, 0, 1, 0]
    assert nid.tolist() == [0, 0xffffffff, 0xffffffff, 1, 2, 3, 4, 0xffffffff, 5]
    assert kept.tolist() == [3, 4, 7, 8] and n_out == 6


needs_ref = pytest.mark.skipif(not orc.ref_tools_available(), reason="reference tools not built here")


@needs_ref
def test_oracle_reductions_match_reference_tools_on_random_inputs():
    rng = np.random.Generator(np.random.PCG64(77))
    tried = 0
    for t in range(60):
        if t % 3 == 0:
            u, v = G.reduction_edges(int(rng.integers(10, 300)), 100 + t, iso_path_max=3)
        else:
            n = int(rng.integers(2, 80))
            m = int(rng.integers(1, 120))
            u = rng.integers(0, n, m).astype(np.uint32)
            v = rng.integers(0, n, m).astype(np.uint32)
        _, kept, nonterm = orc.reduce_degree1(u, v)
        if nonterm:
            continue
        tried += 1
        assert np.array_equal(degree1_lines(u, v, kept), orc.ref_delete_degree1(u, v, timeout=30)), t
        _, nid, kept, n_out = orc.reduce_equivalent(u, v)
        nv, pairs = orc.ref_remove_equivalent(u, v, timeout=30)
        assert n_out == nv and np.array_equal(equivalent_pairs(u, v, nid, kept), pairs), t
    assert tried >= 40


PADO_E_ARG = 1  # include/pado_gpu.h


def test_capi_reduce_argument_checks():
    from parallel_distance_oracle_gb300 import _lib
    lib = _lib.lib
    k, nout = C.c_uint64(), C.c_uint32()
    assert lib.pado_reduce_degree1(3, None, None, 4, None, None, C.byref(k)) == PADO_E_ARG
    assert lib.pado_reduce_equivalent(0, None, None, 4, None, None, None, C.byref(k), None) == PADO_E_ARG
    assert lib.pado_reduce_degree1_device(2, None, None, 4, None, None, C.byref(k), None) == PADO_E_ARG
    assert lib.pado_reduce_equivalent_device(0, None, None, 3, None, None, None, C.byref(k), C.byref(nout),
                                             None) == PADO_E_ARG


@needs_ref
def test_output_writers_match_reference_tool_files(tmp_path):
    """pado.write_degree1_output / write_equivalent_output (pure host code)
    given the oracle's results write byte-identical files to the tools'."""
    import subprocess
    from oracle import build_oracle
    from parallel_distance_oracle_gb300 import pado
    done = 0
    for seed in range(3, 40):
        if done == 2:
            break
        u, v = G.reduction_edges(700, seed, iso_path_max=3)
        _, kept, nonterm = orc.reduce_degree1(u, v)
        if nonterm:  # a core vertex without core edges can carry a long isolated path
            continue
        done += 1
        fin = tmp_path / f"in{seed}.txt"
        fin.write_text("".join(f"{a} {b}\n" for a, b in zip(u.tolist(), v.tolist())))
        ref_d1, ref_eq, log = tmp_path / f"d1_{seed}.txt", tmp_path / f"eq_{seed}.bin", tmp_path / f"log{seed}"
        log.write_text("")
        subprocess.run([str(build_oracle.ref_tool("delete_1_degree")), str(fin), str(ref_d1)], check=True,
                       timeout=60, stdout=subprocess.DEVNULL)
        subprocess.run([str(build_oracle.ref_tool("remove_equivalent")), str(fin), str(ref_eq), str(log)],
                       check=True, timeout=60, stdout=subprocess.DEVNULL, env={"OMP_NUM_THREADS": "1"})
        ours_d1, ours_eq = tmp_path / f"o_d1_{seed}.txt", tmp_path / f"o_eq_{seed}.bin"
        pado.write_degree1_output(ours_d1, u, v, kept)
        _, nid, kept2, n_out = orc.reduce_equivalent(u, v)
        pado.write_equivalent_output(ours_eq, u, v, nid, kept2, n_out)
        assert ours_d1.read_bytes() == ref_d1.read_bytes()
        assert ours_eq.read_bytes() == ref_eq.read_bytes()
    assert done == 2
