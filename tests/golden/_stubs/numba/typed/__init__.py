"""Import-time stand-in for numba.typed."""
Dict = dict
