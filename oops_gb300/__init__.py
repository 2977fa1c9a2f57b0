"""oops_gb300 -- GB300 (sm_103a) implementation of the nzhao/oops CCE hot path.

All compute runs in the in-tree CUDA library liboops_gb300.so (C-ABI in
include/*.h); this package is its host-side front end.
"""
from ._lib import OopsError, lib  # noqa: F401
from .expv import Hamiltonian, KronTerms, expv_block, main_cache  # noqa: F401

__all__ = ["OopsError", "lib", "Hamiltonian", "KronTerms", "expv_block", "main_cache"]
