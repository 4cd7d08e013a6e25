"""Loads libcaustic_gb300.so (the CUDA library behind include/caustic.h).

There is no CPU fallback: if the library is missing or fails to load, every
entry point raises NativeLibraryError.
"""
from __future__ import annotations

import ctypes as C
import os
import pathlib
import threading

from . import _abi

PKG_ROOT = pathlib.Path(__file__).resolve().parent.parent
LIB_PATH = PKG_ROOT / "_build" / "libcaustic_gb300.so"

_lock = threading.Lock()
_lib: C.CDLL | None = None


class NativeLibraryError(RuntimeError):
    """The CUDA library is not built or cannot be loaded."""


class CausticError(RuntimeError):
    """A ct_* call returned a non-zero status."""

    def __init__(self, status: int, message: str):
        self.status = status
        self.status_name = _abi.STATUS_NAMES.get(status, str(status))
        super().__init__(f"{self.status_name}: {message}")


def lib() -> C.CDLL:
    """The loaded library, with argument types declared for every entry point."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = pathlib.Path(os.environ.get("CAUSTIC_LIB", LIB_PATH))
        if not path.exists():
            raise NativeLibraryError(
                f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                "or `python caustic-tracer_gb300/csrc/build.py`")
        try:
            handle = C.CDLL(str(path))
        except OSError as exc:
            raise NativeLibraryError(f"cannot load {path}: {exc}") from exc
        for name, (restype, argtypes) in _abi.SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = restype
            fn.argtypes = argtypes
        if handle.ct_abi_version() != 1:
            raise NativeLibraryError(f"{path}: ABI version {handle.ct_abi_version()} != 1")
        _lib = handle
        return handle


def check(status: int) -> None:
    """Raises CausticError for a non-zero ct_status."""
    if status != 0:
        msg = lib().ct_last_error() or b""
        raise CausticError(status, msg.decode(errors="replace"))


def ptr(array) -> C.c_void_p:
    """Address of a numpy array or torch tensor (host or device)."""
    if array is None:
        return C.c_void_p(0)
    if hasattr(array, "data_ptr"):
        return C.c_void_p(array.data_ptr())
    return C.c_void_p(array.ctypes.data)
