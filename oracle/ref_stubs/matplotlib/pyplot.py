"""Empty stand-in for matplotlib.pyplot (plotting is not on the MC path)."""


def __getattr__(name):
    def _noop(*a, **k):
        return None
    return _noop
