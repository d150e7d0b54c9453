"""Learned subgrid-stress closure for coarse-grid LES (device weights).

The network maps the resolved velocity-gradient tensor ``g[3*i + j] =
d_j u_i`` at a grid point to the symmetric subgrid stress
``tau = (xx, yy, zz, xy, xz, yz)``: 9 -> 64 -> 64 -> 6 with tanh, weights
stored in BF16, arithmetic in FP32.  Inputs are multiplied by ``in_scale``
and outputs by ``out_scale`` (set from the training data).  The ns3d solver
uses it through ``SimulNS3D.set_closure`` as the turbulence model of
``fluidsim/base/turb_model`` (forcing ``-d_j tau_ij``).

Master weights are FP32 (flat buffer, layout W1, b1, W2, b2, W3, b3); the
BF16 copies used by the kernels are refreshed after every update.
"""

import ctypes

import numpy as np
import torch

from . import _lib
from .fft import current_stream_handle

N_IN, N_H, N_OUT = 9, 64, 6
SIZES = (("W1", (N_H, N_IN)), ("b1", (N_H,)), ("W2", (N_H, N_H)), ("b2", (N_H,)),
         ("W3", (N_OUT, N_H)), ("b3", (N_OUT,)))
N_PARAMS = sum(int(np.prod(s)) for _, s in SIZES)


class ClosureMLP:
    def __init__(self, seed=0, device=None):
        self.device = torch.device(device) if device is not None else torch.device(
            "cuda", torch.cuda.current_device())
        rng = np.random.default_rng(seed)
        flat = np.zeros(N_PARAMS, np.float32)
        off = 0
        for name, shape in SIZES:
            n = int(np.prod(shape))
            if name.startswith("W"):
                fan_in = shape[1]
                flat[off:off + n] = rng.uniform(-1, 1, n) * np.sqrt(3.0 / fan_in)
            off += n
        self.master = torch.from_numpy(flat).to(self.device)
        self.in_scale = torch.ones(N_IN, dtype=torch.float32, device=self.device)
        self.out_scale = torch.ones(N_OUT, dtype=torch.float32, device=self.device)
        self.bf16 = {}
        self.refresh_bf16()

    def views(self, t=None):
        t = self.master if t is None else t
        out, off = {}, 0
        for name, shape in SIZES:
            n = int(np.prod(shape))
            out[name] = t[off:off + n].view(shape)
            off += n
        return out

    def refresh_bf16(self):
        v = self.views()
        for name in ("W1", "W2", "W3"):
            self.bf16[name] = v[name].to(torch.bfloat16).contiguous()

    def c_weights(self):
        v = self.views()
        w = _lib.MLPWeights()
        for name in ("W1", "W2", "W3"):
            setattr(w, name, self.bf16[name].data_ptr())
        for name in ("b1", "b2", "b3"):
            setattr(w, name, v[name].data_ptr())
        w.in_scale = self.in_scale.data_ptr()
        w.out_scale = self.out_scale.data_ptr()
        self._keep = w
        return w

    def numpy_params(self):
        """float64 copies with the BF16 rounding the kernels see."""
        v = self.views()
        out = {k: v[k].detach().cpu().numpy().astype(np.float64) for k in ("b1", "b2", "b3")}
        for k in ("W1", "W2", "W3"):
            out[k] = self.bf16[k].float().cpu().numpy().astype(np.float64)
        out["in_scale"] = self.in_scale.cpu().numpy().astype(np.float64)
        out["out_scale"] = self.out_scale.cpu().numpy().astype(np.float64)
        return out

    def state_dict(self):
        return {"master": self.master.cpu(), "in_scale": self.in_scale.cpu(),
                "out_scale": self.out_scale.cpu()}

    def load_state_dict(self, d):
        self.master.copy_(d["master"])
        self.in_scale.copy_(d["in_scale"])
        self.out_scale.copy_(d["out_scale"])
        self.refresh_bf16()


class ClosureTrainer:
    """Adam on the closure with the hand-written gradient kernels.

    ``G`` (9, ld) and ``Tau`` (6, ld) are float32 CUDA tensors of velocity
    gradients and target subgrid stresses (structure of arrays); every step
    draws ``batch`` random points.
    """

    def __init__(self, net: ClosureMLP, batch=65536, lr=2e-3, betas=(0.9, 0.999),
                 eps=1e-8, seed=0, lambda_pi=0.0):
        self.net = net
        self.lambda_pi = float(lambda_pi)
        self.pi_weight = 0.0
        self.lib = _lib.load()
        self.batch = int(batch)
        self.lr, self.betas, self.eps = lr, betas, eps
        dev = net.device
        nbytes = self.lib.gbs_mlp_grad_workspace(self.batch)
        self.ws = torch.empty(nbytes // 4 + 1, dtype=torch.float32, device=dev)
        self.m = torch.zeros(N_PARAMS, dtype=torch.float32, device=dev)
        self.v = torch.zeros(N_PARAMS, dtype=torch.float32, device=dev)
        self.grad = torch.zeros(N_PARAMS, dtype=torch.float32, device=dev)
        self.loss = torch.zeros(1, dtype=torch.float32, device=dev)
        self.step_count = 0
        self.gen = torch.Generator(device=dev)
        self.gen.manual_seed(seed)

    def set_scales(self, G, Tau):
        """Unit-variance inputs and outputs (per component); the weight of
        the dissipation term is lambda_pi / var(tau_ij S_ij)."""
        self.net.in_scale.copy_(1.0 / G.float().std(dim=1).clamp_min(1e-30))
        self.net.out_scale.copy_(Tau.float().std(dim=1).clamp_min(1e-30))
        if self.lambda_pi > 0:
            pi = subgrid_dissipation(G, Tau)
            self.pi_weight = self.lambda_pi / max(float(pi.double().var()), 1e-300)

    def gradient(self, G, Tau, idx):
        w = self.net.c_weights()
        _lib.check(self.lib.gbs_mlp_grad(
            ctypes.byref(w), ctypes.c_void_p(G.data_ptr()), ctypes.c_void_p(Tau.data_ptr()),
            G.shape[1], ctypes.c_void_p(idx.data_ptr()), idx.numel(), self.pi_weight,
            ctypes.c_void_p(self.ws.data_ptr()), ctypes.c_void_p(self.grad.data_ptr()),
            ctypes.c_void_p(self.loss.data_ptr()), current_stream_handle()), "gbs_mlp_grad")
        return self.grad, self.loss

    def step(self, G, Tau):
        idx = torch.randint(0, G.shape[1], (self.batch,), generator=self.gen,
                            device=G.device, dtype=torch.int64)
        self.gradient(G, Tau, idx)
        self.step_count += 1
        w = self.net.c_weights()
        _lib.check(self.lib.gbs_mlp_adam(
            ctypes.c_void_p(self.net.master.data_ptr()), ctypes.c_void_p(self.m.data_ptr()),
            ctypes.c_void_p(self.v.data_ptr()), ctypes.c_void_p(self.grad.data_ptr()),
            self.step_count, self.lr, self.betas[0], self.betas[1], self.eps,
            ctypes.byref(w), current_stream_handle()), "gbs_mlp_adam")
        return self.loss

    def train(self, G, Tau, steps, log_every=0, lr_final=None):
        """``steps`` Adam steps; with ``lr_final`` the learning rate decays
        from ``lr`` to ``lr_final`` on a cosine."""
        from math import cos, pi
        history = []
        lr0 = self.lr
        for it in range(steps):
            if lr_final is not None:
                self.lr = lr_final + 0.5 * (lr0 - lr_final) * (1 + cos(pi * it / max(steps, 1)))
            loss = self.step(G, Tau)
            if log_every and (it % log_every == 0 or it == steps - 1):
                history.append((it, float(loss.item())))
        self.lr = lr0
        return history


def subgrid_dissipation(G, Tau):
    """tau_ij S_ij per point for (9, n) gradients and (6, n) stresses."""
    return (G[0] * Tau[0] + G[4] * Tau[1] + G[8] * Tau[2] + (G[1] + G[3]) * Tau[3]
            + (G[2] + G[6]) * Tau[4] + (G[5] + G[7]) * Tau[5])


PRECISIONS = ("fp32", "bf16")


def predict(net: ClosureMLP, G, precision="fp32"):
    """tau = MLP(G) for a (9, n) float32 CUDA tensor (inference kernel).

    precision "fp32": FP32 activations (three BF16 terms per tensor-core
    operand); "bf16": activations rounded to BF16 and the hardware tanh
    (relative error ~3e-3, a third of the tensor-core work)."""
    if precision not in PRECISIONS:
        raise ValueError(f"precision {precision!r} not in {PRECISIONS}")
    lib = _lib.load()
    n = G.shape[1]
    tau = torch.empty((N_OUT, n), dtype=torch.float32, device=G.device)
    w = net.c_weights()
    fn = lib.gbs_mlp_forward if precision == "fp32" else lib.gbs_mlp_forward_bf16
    _lib.check(fn(ctypes.byref(w), ctypes.c_void_p(G.data_ptr()), n,
                  ctypes.c_void_p(tau.data_ptr()), n, current_stream_handle()),
               "gbs_mlp_forward")
    return tau
