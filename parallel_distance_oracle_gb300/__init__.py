"""GB300-native PADO: pruned landmark (2-hop) labeling and exact distance
queries, as hand-written CUDA for sm_103a behind a C ABI (include/pado_gpu.h).

``graphs`` (seeded synthetic inputs) imports without the CUDA library; the
labeler classes live in ``pado`` and load libpado_gpu.so on import.
"""
from . import graphs  # noqa: F401

__all__ = ["graphs"]
