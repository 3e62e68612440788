"""GB300-native engine for kite's hot path: repeated squaring modulo N = k*2^n - 1 by an FP64
irrational-base discrete weighted transform, behind kite's C API (include/kite.h) as the CUDA
backend.  The product is libkite_gb300.so (csrc/); this package builds it and binds it."""
from .native import load, LIB_PATH  # noqa: F401

__all__ = ["load", "LIB_PATH"]
