"""The no-allocation Pauli expval entry point (tqk_pauli_expval_noalloc), called through
the C ABI, against the scratch-taking entry point (tqk_pauli_expval).

It exists for callers that cannot allocate device memory: a host program binding the
C ABI over FFI with only raw pointers and no device allocator of its own, or a service
held to a fixed device-memory budget.  Its partials live in one array inside the
library that every call shares, so two calls in a row must each give the full,
correct result (nothing left over from the previous call may leak into the next).
This file is collected last so a stop-at-first-failure run has run everything else.
"""
import ctypes

import numpy as np
import pytest
import torch

from torchquantum_gb300 import _lib
from torchquantum_gb300.measurement import pauli_masks

pytestmark = pytest.mark.gpu


def _state(rng, bsz, n):
    s = rng.normal(size=(bsz, 1 << n)) + 1j * rng.normal(size=(bsz, 1 << n))
    s /= np.linalg.norm(s, axis=1, keepdims=True)
    return torch.tensor(s, dtype=torch.complex64, device="cuda")


def _noalloc(lib, st, n, xs, zs):
    out = torch.full((st.shape[0], len(xs)), float("nan"), dtype=torch.float64, device="cuda")
    rc = lib.tqk_pauli_expval_noalloc(st.data_ptr(), st.shape[0], n, _lib._u64(xs), _lib._u64(zs), len(xs),
                                      out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == 0, lib.tqk_last_error().decode()
    return out


@pytest.mark.parametrize("n,bsz,m", [(12, 3, 20), (20, 16, 9), (20, 32, 9), (20, 128, 5)])
def test_noalloc_matches_scratch_entry_point_twice(n, bsz, m):
    lib = _lib.load()
    rng = np.random.default_rng(n + bsz)
    strings = ["".join(rng.choice(list("IXYZ"), size=n)) for _ in range(m - 1)] + ["Z" * n]
    xs, zs = zip(*[pauli_masks(p, n) for p in strings])
    for call in range(2):  # two calls in a row share the static array
        st = _state(rng, bsz, n)
        ref = _lib.pauli_expval(st, n, list(xs), list(zs))
        got = _noalloc(lib, st, n, list(xs), list(zs))
        torch.cuda.synchronize()
        assert not torch.isnan(got).any()
        # the scratch entry point sweeps whole rows for several X-masks (n <= 24), this
        # one makes a pass per X-mask: the same sums in a different float32 order
        assert (got - ref).abs().max().item() < 2e-6, call


def test_noalloc_rejects_oversized_calls():
    lib = _lib.load()
    cap = lib.tqk_pauli_expval_noalloc_capacity()
    assert cap == 1 << 20
    st = torch.zeros(8, 16, dtype=torch.complex64, device="cuda")
    xs = [0] * 5000
    out = torch.zeros(8, 5000, dtype=torch.float64, device="cuda")
    rc = lib.tqk_pauli_expval_noalloc(st.data_ptr(), 8, 4, _lib._u64(xs), _lib._u64(xs), 5000, out.data_ptr(),
                                      torch.cuda.current_stream().cuda_stream)
    assert rc == 2 and b"exceed the limit" in lib.tqk_last_error()
    big = torch.zeros(20000, 1 << 10, dtype=torch.complex64, device="cuda")  # 20000 rows of partials > 1 MiB
    rc = lib.tqk_pauli_expval_noalloc(big.data_ptr(), 20000, 10, _lib._u64([0]), _lib._u64([1]), 1,
                                      out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == 7 and b"static array holds" in lib.tqk_last_error()


def test_noalloc_capacity_boundary():
    """The largest call whose partials fill the 1 MiB array exactly is accepted and
    matches the scratch entry point; one more row is rejected before any launch.
    At n = 10 each row has one block of partials (8 doubles = 64 B), so 16384 rows fill
    1 MiB."""
    lib = _lib.load()
    rng = np.random.default_rng(3)
    n = 10
    strings = ["".join(rng.choice(list("IXYZ"), size=n)) for _ in range(3)] + ["Z" * n]
    xs, zs = zip(*[pauli_masks(p, n) for p in strings])
    st = _state(rng, 16384, n)
    ref = _lib.pauli_expval(st, n, list(xs), list(zs))
    got = _noalloc(lib, st, n, list(xs), list(zs))
    torch.cuda.synchronize()
    assert not torch.isnan(got).any()
    assert (got - ref).abs().max().item() < 2e-6
    del st
    big = torch.zeros(16385, 1 << n, dtype=torch.complex64, device="cuda")
    out = torch.zeros(16385, 1, dtype=torch.float64, device="cuda")
    rc = lib.tqk_pauli_expval_noalloc(big.data_ptr(), 16385, n, _lib._u64([0]), _lib._u64([1]), 1,
                                      out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == 7 and b"static array holds" in lib.tqk_last_error()
