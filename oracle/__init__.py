"""CPU oracle for the JathenAX isothermal hydro right-hand side (test infrastructure).

Importable only from ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py``. The shipped ``jathenax_gb300`` package never imports it.
``oracle/jaxshim`` is a NumPy stand-in for jax that lets the unmodified
reference run in a container without jaxlib; it is used only to generate and
check golden fixtures.
"""
