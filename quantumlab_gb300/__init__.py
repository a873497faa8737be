"""quantumlab_gb300 -- GB300-native state-vector / density-matrix simulation
below QuantumLab's QuEST C API.

The product is the shared library quantumlab_gb300/_build/libquest_gb300.so
(C ABI: include/QuEST.h, include/quest_gb300.h).  This package only builds it
and binds it through ctypes; there is no Python or CPU fallback: load() raises
if the library has not been built.
"""
from __future__ import annotations

import os

from .quest import QuESTLibrary

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libquest_gb300.so")

_lib = None


def build(verbose: bool = False) -> str:
    from .builder import build as _build
    return _build(verbose=verbose)


def load() -> QuESTLibrary:
    """The GB300 library (built in-tree).  Raises if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with quantumlab_gb300.build() "
                "(the GB300 library has no CPU fallback)")
        _lib = QuESTLibrary(LIB_PATH)
    return _lib


__all__ = ["build", "load", "LIB_PATH", "QuESTLibrary"]
