"""Plotting calls of the reference's analysis scripts, accepted and ignored
(TEST INFRASTRUCTURE ONLY; see the package docstring)."""


class _Ignore:
    """Any attribute, call or item is another _Ignore; iteration yields two."""

    def __getattr__(self, name):
        return _Ignore()

    def __call__(self, *args, **kwargs):
        return _Ignore()

    def __iter__(self):
        return iter((_Ignore(), _Ignore()))

    def __getitem__(self, key):
        return _Ignore()


def subplots(*args, **kwargs):
    return _Ignore(), _Ignore()


def __getattr__(name):
    return _Ignore()
