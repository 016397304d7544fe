"""Import-time stand-in for cirq: cirq is only used by the reference's
statevector cross-checks, which are not on the prime-tableau path."""


class Gate:
    pass


def _unavailable(*args, **kwargs):
    raise RuntimeError("cirq is not available here")


class LineQid:
    __init__ = _unavailable


class Circuit:
    __init__ = _unavailable


class Simulator:
    __init__ = _unavailable


measure = _unavailable
