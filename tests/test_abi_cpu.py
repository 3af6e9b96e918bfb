"""CPU checks of the C ABI: the library loads, exports every symbol declared in
include/tqk.h, and its host-side validation rejects bad arguments before any CUDA
call (no GPU compute happens here)."""
import ctypes
import os

import pytest

from torchquantum_gb300 import _lib

LIB = _lib.LIB_PATH


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB):
        from torchquantum_gb300 import build

        build.build()
    return _lib.load()


def test_exports_every_header_symbol(lib):
    names = _lib.header_symbols()
    assert len(names) >= 15
    raw = ctypes.CDLL(LIB)
    for name in names:
        assert hasattr(raw, name), f"libtqk.so does not export {name}"
    assert set(_lib._SIGS) <= set(names), "ctypes signature for a symbol the header does not declare"


def _call(fn, *args):
    return fn(*args)


def test_null_state_rejected(lib):
    w = _lib._i32([0])
    rc = lib.tqk_apply_matrix(None, 1, 3, w, 1, 16, 1, None)
    assert rc == 3 and b"null state" in lib.tqk_last_error()


def test_misaligned_state_rejected(lib):
    w = _lib._i32([0])
    rc = lib.tqk_apply_matrix(8, 1, 3, w, 1, 16, 1, None)
    assert rc == 3 and b"16-byte aligned" in lib.tqk_last_error()


def test_wire_out_of_range_rejected(lib):
    w = _lib._i32([3])
    rc = lib.tqk_apply_matrix(16, 1, 3, w, 1, 16, 1, None)
    assert rc == 1 and b"out of range" in lib.tqk_last_error()


def test_duplicate_wires_rejected(lib):
    w = _lib._i32([1, 1])
    rc = lib.tqk_apply_matrix(16, 1, 3, w, 2, 16, 1, None)
    assert rc == 1 and b"used twice" in lib.tqk_last_error()


def test_control_overlapping_target_rejected(lib):
    c = _lib._i32([2])
    t = _lib._i32([2])
    rc = lib.tqk_apply_controlled(16, 1, 3, c, 1, t, 1, 16, 1, None)
    assert rc == 1


def test_bad_operand_batch_rejected(lib):
    w = _lib._i32([0])
    rc = lib.tqk_apply_matrix(16, 4, 3, w, 1, 16, 3, None)
    assert rc == 2 and b"must be 1 or bsz" in lib.tqk_last_error()


def test_too_many_qubits_rejected(lib):
    w = _lib._i32([0])
    rc = lib.tqk_apply_matrix(16, 1, 40, w, 1, 16, 1, None)
    assert rc == 4


def test_scratch_too_small_rejected(lib):
    rc = lib.tqk_pauli_expval(16, 2, 10, _lib._u64([1]), _lib._u64([0]), 1, 16, 16, 8, 16, None)
    assert rc == 7
    assert lib.tqk_pauli_expval_scratch_bytes(2, 10, 1) > 8


def test_pauli_mask_beyond_n_rejected(lib):
    need = lib.tqk_pauli_expval_scratch_bytes(1, 3, 1)
    rc = lib.tqk_pauli_expval(16, 1, 3, _lib._u64([8]), _lib._u64([0]), 1, 16, 16, need, 16, None)
    assert rc == 1


def test_product_refuses_cpu_device():
    import torchquantum_gb300 as tq

    with pytest.raises(RuntimeError, match="CUDA devices only"):
        tq.QuantumDevice(n_wires=2, device="cpu")


def test_segment_entry_points_marshal_without_launching(lib):
    """The tape-level entry points through ctypes with an empty table: arguments marshal
    (NULL hook included) and nothing is launched; a bad table is rejected on the host."""
    import ctypes

    final = ctypes.c_void_p()
    count = ctypes.c_int64(-1)
    rc = lib.tqk_segment_forward(16, 1, 4, None, 0, 16, ctypes.byref(final), ctypes.byref(count), _lib.EXEC_HOOK(),
                                 None, None)
    assert rc == 0 and final.value == 16 and count.value == 0
    start = ctypes.c_void_p()
    rc = lib.tqk_segment_backward(16, 32, None, 1, 4, None, 0, 16, ctypes.byref(start), ctypes.byref(count),
                                  _lib.EXEC_HOOK(), None, None)
    assert rc == 0 and start.value == 16
    bad = (_lib.ExecOp * 1)()
    bad[0].kind = 99
    rc = lib.tqk_segment_forward(16, 1, 4, bad, 1, 16, ctypes.byref(final), None, _lib.EXEC_HOOK(), None, None)
    assert rc == 2 and b"unknown kind" in lib.tqk_last_error()
    called = []
    hook = _lib.EXEC_HOOK(lambda i, kind, after, user: called.append((i, kind, after)))
    two = (_lib.ExecOp * 2)()
    two[1].skip_reverse = 1
    rc = lib.tqk_segment_backward(16, 32, None, 1, 4, two, 2, 16, None, None, hook, None, None)
    assert rc == 2 and b"only op 0" in lib.tqk_last_error() and called == []


def test_zero_input_block_op_is_checked_on_the_host(lib):
    """A TQK_X_BLOCK_ZERO op needs 6 wires and its U, and in a reverse table it must carry
    skip_reverse (it has no reverse step); tqk_fused_zero_input rejects bad wires and
    batches before any launch."""
    import ctypes

    ops = (_lib.ExecOp * 1)()
    ops[0].kind, ops[0].nw = _lib.X_BLOCK_ZERO, 6
    for j in range(6):
        ops[0].wires[j] = j
    final = ctypes.c_void_p()
    rc = lib.tqk_segment_forward(16, 1, 8, ops, 1, 16, ctypes.byref(final), None, _lib.EXEC_HOOK(), None, None)
    assert rc == 2 and b"zero-input block" in lib.tqk_last_error()  # no U
    ops[0].u = 64
    rc = lib.tqk_segment_backward(16, 32, None, 1, 8, ops, 1, 16, None, None, _lib.EXEC_HOOK(), None, None)
    assert rc == 2 and b"skip_reverse" in lib.tqk_last_error()
    w = (ctypes.c_int32 * 6)(0, 1, 2, 3, 4, 4)
    rc = lib.tqk_fused_zero_input(16, 1, 8, w, 64, 1, None)
    assert rc != 0 and b"used twice" in lib.tqk_last_error()
    w = (ctypes.c_int32 * 6)(0, 1, 2, 3, 4, 5)
    rc = lib.tqk_fused_zero_input(16, 4, 8, w, 64, 3, None)
    assert rc != 0
