"""The tape-level C ABI (tqk_segment_forward / tqk_segment_backward), driven the way an
FFI host drives it: a C2-shaped circuit (depth-400 random circuit at n = 16) is compiled
through the public API, then its segment is replayed through the two entry points with
exec tables and buffers owned by the test.

* Forward: the replay's final state equals the public API's bit for bit (fused method
  with stored block inputs, and the plain method with staged low-qubit runs).
* Reverse: one call of tqk_segment_backward gives, bit for bit, the cotangent at the
  segment's start, every block cross term and every operand cotangent (those of staged
  runs to 1e-12 relative: their per-CTA float64 partials meet in atomics whose order
  varies) that the same reverse steps give when issued one per-op entry point at a time
  (tqk_fused_adjoint_stored, tqk_adjoint_matrix, tqk_staged_adjoint, ...) -- the sequence
  upstream's autograd graph of apply_unitary_bmm (functional/gate_wrapper.py:96-140) stands
  for.
"""
import ctypes

import pytest
import torch

from torchquantum_gb300 import _lib, engine, program

pytestmark = pytest.mark.gpu


def _compile(method, n=16, bsz=2):
    import torchquantum_gb300 as tq
    from torchquantum_gb300 import workloads as W

    gates, ncols = W.random_circuit(n, 400, seed=0)
    th = torch.tensor(W.random_params(bsz, ncols, seed=1), device="cuda", requires_grad=True)
    q = tq.QuantumDevice(n_wires=n, bsz=bsz, device="cuda")
    q.method = method
    if method == "fused":
        q.fuse_wires = 6
        q.fused_backend = "tc"
        q.checkpoint = True
    W.apply_circuit(q, gates, th)
    ev = tq.expval_joint_analytical_batch(q, W.random_paulis(n, 8, seed=2))
    final = q.get_states_1d().detach().clone()
    ev.sum().backward()  # also builds the reverse-sweep images of the blocks
    assert len(q._tape) == 1
    return q, q._tape[0], final


def _replay(sg, n, bsz):
    """Forward through tqk_segment_forward from |0...0> with the test's own block output
    buffers; returns (final state, [(op, stored input)])."""
    lib = _lib.load()
    state = torch.zeros(bsz, 1 << n, dtype=torch.complex64, device="cuda")
    state[:, 0] = 1
    recs, keep, stored, cur = [], [], [], state
    for i, op in enumerate(sg.exec_ops):
        if isinstance(op, program.StagedRun):
            recs.append(program._staged_record(op, op.descs(), keep))
        elif getattr(op, "members", None) is not None and op.tc:
            if i == 0:  # the first block acts on |0...0>: U[:, 0] written in place, nothing kept
                recs.append(program._exec(_lib.X_BLOCK_ZERO, op.wires, batch=op.block_batch, u=op.u128))
                continue
            r = program._exec(_lib.X_BLOCK_TC, op.wires, batch=op.block_batch, image=op.image)
            out = torch.empty_like(state)
            r.out = out.data_ptr()
            stored.append((op, cur))
            cur = out
            recs.append(r)
        elif getattr(op, "members", None) is not None:
            recs.append(program._exec(_lib.X_BLOCK_DENSE, op.wires, batch=op.block_batch, operand=op.operand))
        else:
            recs.append(program._plain_record(op))
    table = (_lib.ExecOp * len(recs))(*recs)
    final = ctypes.c_void_p()
    rc = lib.tqk_segment_forward(state.data_ptr(), bsz, n, table, len(recs), _lib.status_word("cuda").data_ptr(),
                                 ctypes.byref(final), None, _lib.EXEC_HOOK(), None,
                                 torch.cuda.current_stream().cuda_stream)
    assert rc == 0, lib.tqk_last_error().decode()
    assert final.value == cur.data_ptr()
    return cur, dict((id(op), t) for op, t in stored)


def _grad_buffers(sg):
    """Zeroed float64 cotangent slots for every op (and staged member), cross-term
    buffers for the tensor-core blocks."""
    g, mr = {}, {}
    for op in sg.exec_ops:
        if isinstance(op, program.StagedRun):
            for m in op.ops:
                if m.operand is not None:
                    g[id(m)] = torch.zeros(2 * m.operand.numel(), dtype=torch.float64, device="cuda")
        elif getattr(op, "members", None) is not None:
            g[id(op)] = torch.zeros(2 * op.u128.numel(), dtype=torch.float64, device="cuda")
            if op.tc:
                mr[id(op)] = torch.zeros(op.block_batch, 128, 128, dtype=torch.float64, device="cuda")
        elif op.operand is not None:
            g[id(op)] = torch.zeros(2 * op.operand.numel(), dtype=torch.float64, device="cuda")
    return g, mr


def _backward_tape_level(sg, final, lam, stored, n):
    g, mr = _grad_buffers(sg)
    recs, keep = [], []
    for i, op in enumerate(sg.exec_ops):
        if isinstance(op, program.StagedRun):
            recs.append(program._staged_record(op, op.descs([g.get(id(m)) for m in op.ops]), keep))
        elif getattr(op, "members", None) is not None and op.tc:
            r = program._exec(_lib.X_BLOCK_TC, op.wires, batch=op.block_batch, image_h=op.image_h, u=op.u128,
                              grad=g[id(op)], mr=mr[id(op)])
            if i == 0 and id(op) not in stored:
                r.skip_reverse = 1
            elif id(op) in stored:
                r.stored = stored[id(op)].data_ptr()
            recs.append(r)
        elif getattr(op, "members", None) is not None:
            recs.append(program._exec(_lib.X_BLOCK_DENSE, op.wires, batch=op.block_batch, operand=op.operand,
                                      grad=g[id(op)]))
        else:
            recs.append(program._plain_record(op, g.get(id(op))))
    table = (_lib.ExecOp * len(recs))(*recs)
    work = torch.empty_like(final)
    start = ctypes.c_void_p()
    lib = _lib.load()
    rc = lib.tqk_segment_backward(final.data_ptr(), lam.data_ptr(), work.data_ptr(), lam.shape[0], n, table,
                                  len(recs), _lib.status_word("cuda").data_ptr(), ctypes.byref(start), None,
                                  _lib.EXEC_HOOK(), None, torch.cuda.current_stream().cuda_stream)
    assert rc == 0, lib.tqk_last_error().decode()
    return g, mr


def _backward_per_op(sg, final, lam, stored, n):
    """The same reverse steps, one per-op entry point at a time."""
    g, mr = _grad_buffers(sg)
    psi, owned, work = final, False, torch.empty_like(final)

    def writable():
        nonlocal psi, owned
        if not owned:
            work.copy_(psi)
            psi, owned = work, True
        return psi

    for i in range(len(sg.exec_ops) - 1, -1, -1):
        op = sg.exec_ops[i]
        if isinstance(op, program.StagedRun):
            _lib.staged_adjoint(writable(), lam, n, op.descs([g.get(id(m)) for m in op.ops]), op.tile_bits)
        elif getattr(op, "members", None) is not None and op.tc:
            if i == 0 and id(op) not in stored:
                break
            if id(op) in stored:
                _lib.fused_adjoint_stored(stored[id(op)], lam, n, op.wires, op.image_h, op.block_batch, mr[id(op)])
                psi, owned = stored[id(op)], False
            else:
                _lib.fused_adjoint(writable(), lam, n, op.wires, op.image_h, op.block_batch, mr[id(op)])
                _lib.fused_cross_grad(mr[id(op)], op.u128, g[id(op)])
        elif getattr(op, "members", None) is not None:
            _lib.adjoint_matrix(writable(), lam, n, op.wires, op.operand, op.block_batch, g[id(op)])
        else:
            k, slot, p = op.kind, g.get(id(op)), writable()
            if k == engine.KIND_DENSE:
                _lib.adjoint_matrix(p, lam, n, op.wires, op.operand, op.batch, slot, op.uncompute)
            elif k == engine.KIND_CTRL:
                _lib.adjoint_controlled(p, lam, n, op.controls, op.targets, op.operand, op.batch, slot, op.uncompute)
            elif k == engine.KIND_X:
                _lib.apply_mcx(p, n, op.controls, op.ctrl_val, op.targets[0])
                _lib.apply_mcx(lam, n, op.controls, op.ctrl_val, op.targets[0])
            elif k == engine.KIND_PHASE:
                _lib.adjoint_phase(p, lam, n, op.wires, op.operand, op.batch, slot)
            elif k == engine.KIND_DIAG:
                _lib.adjoint_diagonal(p, lam, n, op.wires, op.operand, op.batch, slot)
            else:
                _lib.apply_swap(p, n, op.controls, op.targets[0], op.targets[1])
                _lib.apply_swap(lam, n, op.controls, op.targets[0], op.targets[1])
    return g, mr


@pytest.mark.parametrize("method", ["fused", "plain"])
def test_segment_entry_points_bit_for_bit(method):
    n, bsz = 16, 2
    q, sg, api_final = _compile(method, n, bsz)
    kinds = {type(op).__name__ if not hasattr(op, "members") else ("tc" if op.tc else "block") for op in sg.exec_ops}
    assert ("tc" in kinds) if method == "fused" else ("StagedRun" in kinds)
    final, stored = _replay(sg, n, bsz)
    torch.cuda.synchronize()
    assert torch.equal(final, api_final)
    if method == "fused":
        assert len(stored) > 0
    gen = torch.Generator(device="cuda").manual_seed(3)
    lam0 = torch.randn(bsz, 1 << n, dtype=torch.complex64, device="cuda", generator=gen)
    lam_a, lam_b = lam0.clone(), lam0.clone()
    ga, mra = _backward_per_op(sg, final, lam_a, stored, n)
    gb, mrb = _backward_tape_level(sg, final, lam_b, stored, n)
    torch.cuda.synchronize()
    _lib.check_status(final.device)
    assert torch.equal(lam_a, lam_b)
    # cotangents: a staged run's per-CTA float64 partials meet in float64 atomics (their
    # order varies from launch to launch), every other cotangent and cross term is exact
    assert ga.keys() == gb.keys()
    for k in ga:
        tol = 1e-12 * max(1.0, float(ga[k].abs().max()))
        assert float((ga[k] - gb[k]).abs().max()) <= tol, k
    assert all(torch.equal(mra[k], mrb[k]) for k in mra)
    assert any(float(v.abs().max()) > 0 for v in list(gb.values()) + list(mrb.values()))
    del q
