"""slothdb_gb300 — a GB300-native GROUP BY execution path for SlothDB.

The product is the CUDA library built from ``csrc/`` (C ABI in
``include/slothdb_gb300.h``); this package holds its build recipe, the
ctypes binding and the host-side helpers (data generators, Parquet writer,
batching and serving layers) that sit above the C ABI.
"""
from .capi import GroupBy, GbError, load  # noqa: F401

__all__ = ["GroupBy", "GbError", "load"]
