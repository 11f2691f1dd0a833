"""The drop-in header compiles with the drivers: our own driver (always) and,
where the reference tree is available, the reference's unmodified pado.cpp and
query_distance.cpp with their labeler headers mapped to include/pado_gpu.hpp."""

import pytest

from dropin.build_dropin import build

from oracle.build_oracle import _reference_dir

REF = _reference_dir()
LABELER_HEADERS = [
    "pado_unw_unv_para.201912311607.parallel_bp_labeling.h", "pado_unw_unv_unp.h", "pado_unw_vec_unp.h",
    "pado_unw_vec_para.h", "pado_weighted_unv_unp.h", "pado_weighted_vec_unp.h", "pado_weighted_unv_para.h",
    "pado_weighted_vec_para.h",
]


def test_dropin_driver_compiles_and_links(tmp_path):
    exe = build(tmp_path)
    assert exe.exists()


@pytest.mark.skipif(not (REF / "pado.cpp").exists(), reason="reference tree not available on this host")
def test_reference_drivers_compile_unchanged_against_the_gpu_header(tmp_path):
    shim = tmp_path / "shim"
    shim.mkdir()
    # each labeler header the drivers include becomes the drop-in header
    for h in LABELER_HEADERS:
        (shim / h).write_text('#include "pado_gpu.hpp"\n')
    for drv in ("pado.cpp", "query_distance.cpp"):
        exe = build(tmp_path, sources=[REF / drv], extra_includes=[shim, REF / "includes"], name=drv[:-4])
        assert exe.exists()
