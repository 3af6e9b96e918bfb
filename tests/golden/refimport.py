"""Import the upstream torchquantum package from its source tree for fixture generation.

Test infrastructure only: used by ``make_golden.py`` in a container that holds the
reference source tree.  Nothing in the product, the GPU tests, ``smoke()`` or
``bench.py`` imports this module.

The upstream package imports several optional dependencies at module import time
(qiskit, torchpack, matplotlib, pathos, dill, torchdiffeq, tensorflow, pyscf,
torchvision, tqdm, ...).  None of them is needed for the statevector path, so a
``sys.meta_path`` finder serves an empty stand-in module for each missing root.
``torchpack.utils.logging.logger`` is mapped to a stdlib logger because the gate
wrapper imports it by name.
"""
from __future__ import annotations

import importlib.abc
import importlib.machinery
import importlib.util
import logging
import os
import sys
import types

REFERENCE_ROOT = os.environ.get("TQ_REFERENCE_ROOT", "/root/reference")

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


class _StubFinder(importlib.abc.MetaPathFinder):
    def find_spec(self, fullname, path, target=None):
        root = fullname.split(".")[0]
        if root not in _STUB_ROOTS:
            return None
        if importlib.machinery.PathFinder.find_spec(root) is not None and root == fullname:
            return None  # really installed: use it
        return importlib.machinery.ModuleSpec(fullname, _StubLoader(), is_package=True)


def import_reference():
    """Return the upstream ``torchquantum`` package imported from its source tree."""
    if "torchquantum" in sys.modules:
        return sys.modules["torchquantum"]
    if not any(isinstance(f, _StubFinder) for f in sys.meta_path):
        sys.meta_path.insert(0, _StubFinder())
    if REFERENCE_ROOT not in sys.path:
        sys.path.insert(0, REFERENCE_ROOT)
    import torchquantum  # noqa: E402

    return torchquantum


def set_reference_precision(double: bool) -> None:
    """Switch the upstream package's module-level dtypes (complex128 oracle mode).

    The matrix builders and ``apply_unitary_bmm`` read ``C_DTYPE``/``F_DTYPE`` from
    their module globals at call time, so rebinding them in every loaded module
    switches the whole statevector path.
    """
    import torch

    c, f = (torch.complex128, torch.float64) if double else (torch.complex64, torch.float32)
    for name, mod in list(sys.modules.items()):
        if not name.startswith("torchquantum") or mod is None:
            continue
        if hasattr(mod, "C_DTYPE"):
            mod.C_DTYPE = c
        if hasattr(mod, "F_DTYPE"):
            mod.F_DTYPE = f
    # constant gate matrices (Pauli matrices used by expval_joint_analytical's kron)
    fn = sys.modules.get("torchquantum.functional")
    if fn is not None:
        for key, val in list(fn.mat_dict.items()):
            if isinstance(val, torch.Tensor):
                fn.mat_dict[key] = val.to(c)
