"""GB300-native BatchLayout: force-directed graph layout on one GPU.

Host mirror of the reference's layout engine (class `algorithms`,
sample/algorithms.h:50-85) over the C ABI in include/batchlayout_gb300.h.
"""
from ._lib import Algorithms, BatchedLayout, BatchLayoutError, load, read_matrix_market  # noqa: F401
from .build import build  # noqa: F401
