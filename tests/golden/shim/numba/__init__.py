"""Pass-through stand-in for numba, used only by tests/golden/make_golden.py.

numba is not installed here; the reference's RoadRunner modules only use
``njit`` (bare, with keywords, or ``njit(f, **kw)``), ``prange`` and the thread
count helpers, so this stub lets CPython run those modules unmodified.
"""


def njit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]
    if len(args) == 1 and callable(args[0]):
        return args[0]

    def wrap(f):
        return f
    return wrap


jit = njit
prange = range


def get_num_threads():
    return 1


def set_num_threads(n):
    return None
