"""Upstream torchquantum, imported as-is for timing and parity checks (test infrastructure).

Used only by the tests, ``bench.py``'s reference arm and fixture generation -- never by
the package.  Upstream is pure Python over torch; it is found, in order, in

* ``$TQ_REFERENCE_ROOT`` (a source tree or an install directory), then
* ``baseline/_ref`` under the repository root: the offline ``pip install --no-deps
  --target baseline/_ref`` of the reference (git-ignored, travels with the repository
  copy, so the GPU machine can import it too).

Upstream imports several optional dependencies at module import time (qiskit,
torchpack, matplotlib, pathos, dill, torchdiffeq, tensorflow, pyscf, torchvision,
tqdm, ...).  None of them is on the statevector path, so a ``sys.meta_path`` finder
serves an empty stand-in module for each missing root; ``torchpack.utils.logging.logger``
is mapped to a stdlib logger because the gate wrapper imports it by name
(``torchquantum/functional/gate_wrapper.py:8``).  torch itself is imported before the
finder is installed, so none of torch's own optional imports is stubbed.
"""
from __future__ import annotations

import importlib.abc
import importlib.machinery
import logging
import os
import sys
import types
from typing import Optional

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INSTALL_DIR = os.path.join(ROOT, "baseline", "_ref")

_STUB_ROOTS = (
    "qiskit", "qiskit_nature", "qiskit_ibm_runtime", "qiskit_aer", "torchpack",
    "matplotlib", "pathos", "dill", "torchdiffeq", "tensorflow",
    "tensorflow_model_optimization", "pyscf", "torchvision", "tqdm", "opt_einsum",
    "pylatexenc", "imp",
)


class _StubModule(types.ModuleType):
    """Module whose every missing attribute is another stub (classes, functions)."""

    def __getattr__(self, item):
        if item.startswith("__") and item.endswith("__"):
            raise AttributeError(item)
        full = f"{self.__name__}.{item}"
        if full in sys.modules:
            return sys.modules[full]
        stub = _make_stub(full)
        sys.modules[full] = stub
        setattr(self, item, stub)
        return stub

    def __call__(self, *args, **kwargs):
        return _make_stub(self.__name__ + "()")

    def __iter__(self):
        return iter(())

    def __mro_entries__(self, bases):
        return (object,)


def _make_stub(name: str) -> _StubModule:
    mod = _StubModule(name)
    mod.__file__ = os.path.join("/nonexistent", *name.split(".")) + ".py"
    mod.__path__ = []  # behave as a package so submodule imports resolve
    if name == "torchpack.utils.logging":
        mod.logger = logging.getLogger("torchquantum-reference")
    return mod


class _StubLoader(importlib.abc.Loader):
    def create_module(self, spec):
        return _make_stub(spec.name)

    def exec_module(self, module):
        return None


class StubFinder(importlib.abc.MetaPathFinder):
    """Serves stand-ins for upstream's optional dependencies that are not installed."""

    def find_spec(self, fullname, path, target=None):
        root = fullname.split(".")[0]
        if root not in _STUB_ROOTS:
            return None
        if importlib.machinery.PathFinder.find_spec(root) is not None and root == fullname:
            return None  # really installed: use it
        return importlib.machinery.ModuleSpec(fullname, _StubLoader(), is_package=True)


def locate(root: Optional[str] = None) -> Optional[str]:
    """Directory holding upstream's ``torchquantum`` package, or None."""
    for cand in (root, os.environ.get("TQ_REFERENCE_ROOT"), INSTALL_DIR):
        if cand and os.path.isfile(os.path.join(cand, "torchquantum", "__init__.py")):
            return cand
    return None


def available(root: Optional[str] = None) -> bool:
    return locate(root) is not None


def import_upstream(root: Optional[str] = None):
    """Return upstream's ``torchquantum`` package (raises ImportError when absent)."""
    mod = sys.modules.get("torchquantum")
    if mod is not None:
        return mod
    where = locate(root)
    if where is None:
        raise ImportError("upstream torchquantum not found: set TQ_REFERENCE_ROOT or install the reference into "
                          "baseline/_ref (pip install --no-deps --target baseline/_ref <reference>)")
    import torch  # noqa: F401  (before the stub finder: torch's own optional imports stay real)

    if not any(isinstance(f, StubFinder) for f in sys.meta_path):
        sys.meta_path.insert(0, StubFinder())
    if where not in sys.path:
        sys.path.insert(0, where)
    import torchquantum  # noqa: E402

    return torchquantum


def set_precision(double: bool) -> None:
    """Switch upstream's module-level dtypes (complex128 oracle mode).

    The matrix builders and ``apply_unitary_bmm`` read ``C_DTYPE``/``F_DTYPE`` from
    their module globals at call time (``torchquantum/macro.py:27-28``), so rebinding
    them in every loaded module switches the whole statevector path.
    """
    import torch

    c, f = (torch.complex128, torch.float64) if double else (torch.complex64, torch.float32)
    for name, mod in list(sys.modules.items()):
        if not name.startswith("torchquantum") or name.startswith("torchquantum_gb300") or mod is None:
            continue
        if hasattr(mod, "C_DTYPE"):
            mod.C_DTYPE = c
        if hasattr(mod, "F_DTYPE"):
            mod.F_DTYPE = f
    fn = sys.modules.get("torchquantum.functional")
    if fn is not None:
        for key, val in list(fn.mat_dict.items()):
            if isinstance(val, torch.Tensor):
                fn.mat_dict[key] = val.to(c)
