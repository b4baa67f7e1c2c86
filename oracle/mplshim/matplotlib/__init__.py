"""A do-nothing stand-in for matplotlib (TEST INFRASTRUCTURE ONLY).

matplotlib is not installed here. The reference's analysis script
(jathenax/spectra.py) computes its shell spectra with NumPy, writes them to a
CSV file and only then draws a figure; with this package first on sys.path
the unmodified script runs and writes its CSV, and every plotting call is
accepted and ignored. Used only by tests/golden/make_spectra.py.
"""


def use(backend, *args, **kwargs):
    return None
