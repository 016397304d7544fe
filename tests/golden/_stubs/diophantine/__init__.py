"""Import-time stand-in for the PyPI Diophantine package, used only by the
reference's composite-dimension tableau."""


def solve(*args, **kwargs):
    raise RuntimeError("the Diophantine solver is not available here")
