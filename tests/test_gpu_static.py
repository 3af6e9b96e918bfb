"""Static mode and op-history replay, the self-consistency checks of upstream's
test/static_mode_test.py (dynamic vs static states :320, gradients :258, get_unitary
:362): a module's ``static_on(wires_per_block=k)`` runs the fused method and gives the
dynamic (plain) states and gradients; ``get_unitary`` is the circuit's unitary; a device's
``op_history`` replayed through ``QuantumModule.from_op_history`` gives the same state."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _model(n, n_ops, seed):
    import torchquantum_gb300 as tq

    class M(tq.QuantumModule):
        def __init__(self):
            super().__init__()
            self.n_wires = n
            self.layer = tq.RandomLayer(n_ops=n_ops, wires=list(range(n)), seed=seed,
                                        op_types=(tq.RX, tq.RY, tq.RZ, tq.U3, tq.CNOT, tq.CZ, tq.CRX, tq.RZZ))

        @tq.static_support
        def forward(self, q_device):
            self.layer(q_device)

    torch.manual_seed(seed)
    return M().to("cuda")


@pytest.mark.parametrize("k", [2, 3, 4, 6])
def test_static_matches_dynamic(k):
    import torchquantum_gb300 as tq

    n, bsz = 7, 3
    m = _model(n, 120, seed=k)
    obs = ["ZIXIYZI", "IIIIIIZ"]
    res = {}
    for static in (False, True):
        if static:
            m.static_on(wires_per_block=k)
        else:
            m.static_off()
        m.zero_grad()
        q = tq.QuantumDevice(n_wires=n, bsz=bsz, device="cuda")
        m(q)
        ev = tq.expval_joint_analytical_batch(q, obs)
        ev.sum().backward()
        grads = torch.cat([p.grad.reshape(-1) for p in m.parameters()])
        res[static] = (q.get_states_1d().detach().cpu().numpy(), grads.cpu().numpy())
        if static:
            assert any(getattr(op, "members", None) for sg in q._tape for op in sg.exec_ops)
    m.static_off()
    assert np.abs(res[True][0] - res[False][0]).max() < 1e-5
    assert np.abs(res[True][1] - res[False][1]).max() < 1e-5


def test_get_unitary_and_op_history_replay():
    import torchquantum_gb300 as tq

    n = 5
    m = _model(n, 60, seed=9)
    u = m.get_unitary().detach()
    ud = u.to(torch.complex128).cpu().numpy()
    assert np.abs(ud @ ud.conj().T - np.eye(1 << n)).max() < 1e-5
    q = tq.QuantumDevice(n_wires=n, bsz=1, device="cuda", record_op=True)
    m(q)
    psi = q.get_states_1d().detach().cpu().numpy()[0]
    assert np.abs(ud[:, 0] - psi).max() < 1e-5
    replay = tq.QuantumModule.from_op_history(q.op_history).to("cuda")
    q2 = tq.QuantumDevice(n_wires=n, bsz=1, device="cuda")
    replay(q2)
    assert np.abs(q2.get_states_1d().detach().cpu().numpy()[0] - psi).max() < 1e-5
