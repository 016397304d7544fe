"""Import-time stand-in for numba.core."""


class types:  # noqa: N801 - mirrors the imported name
    pass
