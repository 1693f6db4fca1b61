"""minibude_gb300 -- GB300-native (sm_103a) implementation of miniBUDE's energy-evaluation hot path.

The compute lives in libbude_gb300.so (CUDA kernels + the C-ABI of include/minibude_gb300.h).
This package is the Python host side: deck files (`deck`), the reference's validation and
statistics (`validate`), the ctypes binding (`capi`) and the reference-shaped model interface
(`model`).
"""
from .deck import (ATOM_DTYPE, BATCH, FF_DTYPE, LARGE, SMALL, SPECS, BatchDeck, BatchSpec, Deck, DeckSpec,
                   conformation_batch, read_conformations, read_deck, synthetic_batch, synthetic_deck, write_deck)
from .validate import DIFF_TOLERANCE_PCT, evaluate, validate, validate_abs

__all__ = [
    "ATOM_DTYPE", "BATCH", "FF_DTYPE", "LARGE", "SMALL", "SPECS", "BatchDeck", "BatchSpec", "Deck", "DeckSpec",
    "read_deck", "read_conformations", "conformation_batch", "synthetic_batch", "synthetic_deck", "write_deck", "DIFF_TOLERANCE_PCT", "evaluate", "validate", "validate_abs",
]
