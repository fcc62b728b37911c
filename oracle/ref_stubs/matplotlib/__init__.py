"""Empty stand-in for matplotlib so the reference's analysis helpers import."""


def use(*a, **k):
    pass
