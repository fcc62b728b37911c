"""Stand-in for numba used only to import the reference: ``njit`` is a pass-through."""


def njit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]

    def deco(f):
        return f
    return deco


jit = njit
