"""Pure-Python stand-in for the ``numba`` package.

Fixture tooling only: numba is not installed in the container that generates
the golden vectors, and the reference encoder imports ``numba.njit`` /
``numba.prange``.  ``njit`` returns a wrapper that runs the original Python
body; ``prange`` is ``range``.

numba evaluates int32/uint32/int16 arithmetic in 64-bit registers, while plain
numpy keeps the narrow dtype and can overflow.  To keep the reference's
integer results, the wrapper (1) executes the function with a module object in
place of ``np`` whose narrow integer dtypes name ``int64``, and (2) widens
narrow integer array arguments to int64 for the call, writing the results back
into the caller's arrays afterwards.
"""
import functools
import types

import numpy as _np

_WIDE_NP = types.ModuleType("numpy_wide_ints")
_WIDE_NP.__dict__.update(_np.__dict__)
for _name in ("int16", "int32", "uint16", "uint32"):
    setattr(_WIDE_NP, _name, _np.int64)

_NARROW_TYPES = (_np.int16, _np.int32, _np.uint16, _np.uint32)


def _as_python(fn):
    rebound = {}

    @functools.wraps(fn)
    def call(*args, **kwargs):
        impl = rebound.get("impl")
        if impl is None:
            glb = dict(fn.__globals__)
            if glb.get("np") is _np:
                glb["np"] = _WIDE_NP
            impl = types.FunctionType(fn.__code__, glb, fn.__name__,
                                      fn.__defaults__, fn.__closure__)
            impl.__kwdefaults__ = fn.__kwdefaults__
            rebound["impl"] = impl
        widened = []
        call_args = []
        for a in args:
            if isinstance(a, _np.ndarray) and a.dtype.type in _NARROW_TYPES:
                w = a.astype(_np.int64)
                widened.append((a, w))
                call_args.append(w)
            else:
                call_args.append(a)
        out = impl(*call_args, **kwargs)
        for orig, w in widened:
            orig[...] = w.astype(orig.dtype)
        return out

    return call


def njit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return _as_python(args[0])
    return _as_python


jit = njit
prange = range
