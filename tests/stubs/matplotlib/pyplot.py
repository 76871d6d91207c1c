"""No-op pyplot: every call returns an object whose methods do nothing."""


class _Nothing:
    def __getattr__(self, name):
        return lambda *a, **k: _Nothing()


def __getattr__(name):
    return lambda *a, **k: _Nothing()
