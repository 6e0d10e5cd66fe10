"""Pass-through stand-in for numba, used only when the fixture script imports
the reference implementation in a container without numba. ``jit``/``njit``
return the undecorated function; type names are inert callables."""


class _Type:
    def __call__(self, *args, **kwargs):
        return self

    def __getitem__(self, item):
        return self


complex64 = complex128 = float32 = float64 = int32 = int64 = boolean = _Type()


class types:  # noqa: N801 - mirrors numba.types
    def __getattr__(self, name):
        return _Type()


types = types()


def _decorator_factory(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs and not isinstance(args[0], _Type):
        return args[0]

    def wrap(fn):
        return fn
    return wrap


jit = njit = vectorize = _decorator_factory
prange = range


class config:  # noqa: N801
    NUMBA_DEFAULT_NUM_THREADS = 1
    NUMBA_NUM_THREADS = 1


def set_num_threads(n):
    return None


def get_num_threads():
    return 1
