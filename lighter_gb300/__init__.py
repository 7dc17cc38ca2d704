"""lighter_gb300 -- GB300-native lightmap baker behind lighter's ltr_* C API.

The product is the shared library ``liblighter_gb300.so`` built from
``lighter_gb300/csrc`` (CUDA kernels for sm_103a plus the C++ host side of the
API). This package only locates, builds and binds it for Python callers; the
bake itself never runs in Python and there is no CPU fallback: if the library
or a CUDA device is missing, the bake fails loudly.
"""
from __future__ import annotations

import ctypes as C
import os

from . import abi

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "liblighter_gb300.so")

_lib = None


def load_library(path: str, with_debug: bool = True, extra: dict | None = None):
    """dlopen an ltr_* library privately (RTLD_LOCAL) and bind its prototypes."""
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} not built (run __graft_entry__.build())")
    lib = C.CDLL(path, mode=os.RTLD_LOCAL | os.RTLD_NOW)
    abi.bind(lib, abi.LTR_API)
    if with_debug:
        abi.bind(lib, abi.LTRDBG_API)
        abi.bind(lib, {k: v for k, v in abi.LTRDBG_OPTIONAL.items() if hasattr(lib, k)})
    if extra:
        abi.bind(lib, extra)
    return lib


def library():
    """The GPU baker (liblighter_gb300.so), bound with every exported entry point."""
    global _lib
    if _lib is None:
        from . import ext
        _lib = load_library(LIB_PATH, True, ext.EXT_API)
    return _lib
