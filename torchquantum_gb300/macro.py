"""Package-wide constants under upstream's names (``torchquantum/macro.py:41-50``).

The engine stores states in complex64 and gate parameters in float32, as upstream does;
``ABC`` / ``ABC_ARRAY`` are upstream's einsum alphabet, kept for user code that builds
einsum strings.
"""
import math
from string import ascii_lowercase

import numpy as np
import torch

__all__ = ["C_DTYPE", "F_DTYPE", "ABC", "ABC_ARRAY", "INV_SQRT2", "C_DTYPE_NUMPY", "F_DTYPE_NUMPY"]

C_DTYPE = torch.complex64
F_DTYPE = torch.float32
ABC = ascii_lowercase
ABC_ARRAY = np.array(list(ABC))
INV_SQRT2 = 1 / math.sqrt(2)
C_DTYPE_NUMPY = np.complex64
F_DTYPE_NUMPY = np.float32
