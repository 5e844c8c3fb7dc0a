"""Stand-in for numba used only to run the reference when generating golden
vectors: ``njit`` returns the plain Python function."""


def njit(*args, **kwargs):
    if args and callable(args[0]) and not kwargs:
        return args[0]
    return lambda fn: fn
