"""Loader of the in-tree CUDA library.  There is no CPU fallback: if the library cannot be
loaded, every entry point of this package fails loudly."""
import ctypes as C
import os

from . import abi, build

_lib = None


class NativeUnavailable(RuntimeError):
    pass


def load(rebuild_if_stale=True):
    global _lib
    if _lib is not None:
        return _lib
    path = build.LIB
    if rebuild_if_stale and not build.up_to_date():
        try:
            build.build()
        except Exception as e:          # no nvcc, or a compile error
            if not os.path.exists(path):
                raise NativeUnavailable(f"CUDA library not built and build failed: {e}") from e
    if not os.path.exists(path):
        raise NativeUnavailable(f"CUDA library missing: {path}")
    lib = C.CDLL(path)
    for name in abi.EXPORTED:
        if not hasattr(lib, name):
            raise NativeUnavailable(f"{path} does not export {name}")
    _lib = abi.bind_common(lib)
    return _lib
