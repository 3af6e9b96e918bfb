"""Import the upstream torchquantum package from its source tree for fixture generation.

Test infrastructure only: used by ``make_golden.py`` in a container that holds the
reference source tree (``TQ_REFERENCE_ROOT``, default ``/root/reference``).  The stub
finder for upstream's absent optional dependencies and the complex128 switch live in
``oracle/upstream.py``, which the tests and ``bench.py``'s reference arm use to import
the offline install of upstream in ``baseline/_ref``.
"""
from __future__ import annotations

import os
import sys

_REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if _REPO not in sys.path:
    sys.path.insert(0, _REPO)

from oracle import upstream as _upstream  # noqa: E402

REFERENCE_ROOT = os.environ.get("TQ_REFERENCE_ROOT", "/root/reference")


def import_reference():
    """Return the upstream ``torchquantum`` package imported from its source tree."""
    return _upstream.import_upstream(REFERENCE_ROOT)


def set_reference_precision(double: bool) -> None:
    """Switch the upstream package's module-level dtypes (complex128 oracle mode)."""
    _upstream.set_precision(double)
