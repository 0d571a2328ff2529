"""Test-only stand-in for numba (absent in this image).

`njit(...)` returns the decorated function unchanged, so the reference's
`@njit(cache=True, fastmath=True)` kernels run as plain Python with IEEE
order (no fastmath reassociation). Used only by tests/golden/make_golden.py
to execute the reference code when generating golden vectors.
"""


def njit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]

    def deco(fn):
        return fn

    return deco


jit = njit
prange = range
