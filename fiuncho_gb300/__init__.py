"""GB300-native (sm_103a) exhaustive k-order epistasis search with Fiuncho's
search API.

The compute path is ``libfiuncho_gpu.so`` (hand-written CUDA, C ABI in
``include/fiuncho_gpu.h``); this package is its Python host side:
``Dataset`` (data model and readers), ``Distribution``, ``Result``,
``GpuSearch`` (the ``Search`` drop-in) and a single- or multi-rank
``MPIEngine``.
"""
from .dataset import Dataset, GenotypeTable, words_for  # noqa: F401
from .search import Context, Distribution, GpuSearch, MPIEngine, Resident, Result, Server  # noqa: F401
from ._lib import FiunchoError  # noqa: F401
