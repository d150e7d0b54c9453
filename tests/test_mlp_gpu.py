"""Hand-written closure training kernels against the float64 oracle MLP."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _net_and_data(n, seed=0):
    import torch
    from fluidsim_gb300.closure import ClosureMLP
    net = ClosureMLP(seed=seed)
    rng = np.random.default_rng(seed)
    G = torch.from_numpy(rng.standard_normal((9, n)).astype(np.float32)).cuda()
    Tau = torch.from_numpy(rng.standard_normal((6, n)).astype(np.float32)).cuda()
    net.in_scale.copy_(torch.linspace(0.5, 1.5, 9))
    net.out_scale.copy_(torch.linspace(0.8, 1.3, 6))
    return net, G, Tau


def _oracle(net):
    from oracle.turb import MLPClosure
    w = net.numpy_params()
    return MLPClosure(w["W1"], w["b1"], w["W2"], w["b2"], w["W3"], w["b3"],
                      w["in_scale"], w["out_scale"])


def test_forward_matches_oracle(cuda):
    from fluidsim_gb300.closure import predict
    net, G, _ = _net_and_data(7000)
    tau = predict(net, G).cpu().numpy()
    ref = _oracle(net).forward(G.cpu().numpy().astype(np.float64).T).T
    assert np.abs(tau - ref).max() / np.abs(ref).max() < 1e-5


def test_forward_bf16_close_to_oracle(cuda):
    """The BF16 form (activations rounded to BF16, hardware tanh): relative
    error of the order of the BF16 rounding (2^-9), not of FP32."""
    from fluidsim_gb300.closure import predict
    net, G, _ = _net_and_data(7000)
    tau = predict(net, G, precision="bf16").cpu().numpy()
    ref = _oracle(net).forward(G.cpu().numpy().astype(np.float64).T).T
    err_max = np.abs(tau - ref).max() / np.abs(ref).max()
    err_l2 = np.linalg.norm(tau - ref) / np.linalg.norm(ref)
    assert err_max < 3e-2 and err_l2 < 1e-2, (err_max, err_l2)
    assert err_l2 > 1e-5  # a different evaluation from the FP32 form
    with pytest.raises(ValueError):
        predict(net, G, precision="fp16")


@pytest.mark.parametrize("pi_weight", [0.0, 0.05])
def test_gradient_matches_oracle(cuda, pi_weight):
    import torch
    from fluidsim_gb300.closure import ClosureTrainer
    net, G, Tau = _net_and_data(5000, seed=1)
    tr = ClosureTrainer(net, batch=5000)
    tr.pi_weight = pi_weight
    idx = torch.arange(5000, device="cuda", dtype=torch.int64)
    grad, loss = tr.gradient(G, Tau, idx)
    g64 = G.cpu().numpy().astype(np.float64).T
    t64 = Tau.cpu().numpy().astype(np.float64).T
    ref_loss, ref = _oracle(net).loss_and_grads(g64, t64, pi_weight=pi_weight)
    flat = np.concatenate([ref[k].ravel() for k in ("W1", "b1", "W2", "b2", "W3", "b3")])
    got = grad.cpu().numpy().astype(np.float64)
    assert abs(loss.item() - ref_loss) < 1e-5 * ref_loss
    assert np.linalg.norm(got - flat) / np.linalg.norm(flat) < 1e-4
    # deterministic
    grad2, _ = tr.gradient(G, Tau, idx)
    assert np.array_equal(grad2.cpu().numpy(), got.astype(np.float32))


def test_training_reduces_loss_on_teacher_data(cuda):
    import torch
    from fluidsim_gb300.closure import ClosureMLP, ClosureTrainer, predict
    teacher = ClosureMLP(seed=11)
    rng = np.random.default_rng(3)
    G = torch.from_numpy(rng.standard_normal((9, 200000)).astype(np.float32)).cuda()
    Tau = predict(teacher, G)
    student = ClosureMLP(seed=12)
    tr = ClosureTrainer(student, batch=16384, lr=3e-3)
    tr.set_scales(G, Tau)
    hist = tr.train(G, Tau, 400, log_every=100)
    assert hist[-1][1] < 0.1 * hist[0][1], hist
