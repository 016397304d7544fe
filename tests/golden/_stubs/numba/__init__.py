"""Import-time stand-in for numba: the reference's @njit decorators are
commented out and only ``prange`` / ``njit`` names are imported."""
prange = range


def njit(*args, **kwargs):
    if args and callable(args[0]):
        return args[0]
    return lambda fn: fn
