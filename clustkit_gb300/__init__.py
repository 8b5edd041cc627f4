"""clustkit_gb300 -- GB300 (sm_103a) engine for clustkit's Align phase
(banded Smith-Waterman over candidate pairs) and the MinHash sketching that
feeds its pre-filters.

The compute path is libckgpu.so (CUDA kernels behind the C ABI in
include/clustkit_gb300.h); this package holds the Python host side, which
mirrors clustkit's own entry points so that it can replace them.
"""
from .blosum import BLOSUM62, PROTEIN_ALPHABET  # noqa: F401

__version__ = "0.1.0"


def load():
    """Build (if needed) and load libckgpu.so; returns the ctypes handle."""
    from . import _lib
    return _lib.load()
