"""CPU oracle for the statevector gate-application path (test infrastructure only).

Imported only by ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline; the product package never imports it.
"""
