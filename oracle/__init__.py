"""CPU oracle for the statevector gate-application path (test infrastructure only).

Imported only by ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline and reference arm; the product package never imports it.  ``statevec`` is
the numpy restatement of the upstream algorithm; ``upstream`` imports upstream itself
(from the offline install in ``baseline/_ref``) for timing and parity checks.
"""
