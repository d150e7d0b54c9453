"""Turbulence-model hook on the GPU: learned closure forcing vs the oracle."""
from math import pi

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape,precision,tol", [((32, 32, 32), "fp32", 2e-5),
                                                 ((16, 24, 20), "fp32", 2e-5),
                                                 ((32, 32, 32), "bf16", 1e-2)])
def test_mlp_closure_tendency_matches_oracle(cuda, shape, precision, tol):
    import torch
    from fluidsim_gb300.closure import ClosureMLP
    from fluidsim_gb300.init_fields import isotropic_3d
    from fluidsim_gb300.solvers import SimulNS3D
    from oracle.solvers import NS3DOracle
    from oracle.spectral import OperNumpy3D
    from oracle.turb import MLPClosure, closure_forcing
    nz, ny, nx = shape
    p = SimulNS3D.create_default_params()
    p.precision = "float32"
    p.oper.nx, p.oper.ny, p.oper.nz = nx, ny, nz
    p.turb_model.enable, p.turb_model.type = True, "mlp_closure"
    sim = SimulNS3D(p)
    net = ClosureMLP(seed=3)
    net.in_scale.fill_(0.2)
    net.out_scale.fill_(0.05)
    sim.set_closure(net, precision=precision)
    v0 = isotropic_3d(nx, ny, nz, seed=2)
    tend = sim.tendencies_nonlin(torch.from_numpy(v0).cuda().to(torch.complex64)).cpu().numpy()
    w = net.numpy_params()
    mlp = MLPClosure(w["W1"], w["b1"], w["W2"], w["b2"], w["W3"], w["b3"],
                     w["in_scale"], w["out_scale"])
    oper = OperNumpy3D(nx, ny, nz)
    orc = NS3DOracle(oper, turb_model=lambda o, a, b, c: closure_forcing(o, (a, b, c), mlp))
    ref = orc.tendencies_nonlin(v0.astype(np.complex128))
    # the closure alone must matter: compare against the tendency without it
    orc0 = NS3DOracle(oper)
    ref0 = orc0.tendencies_nonlin(v0.astype(np.complex128))
    assert np.linalg.norm(ref - ref0) > 1e-3 * np.linalg.norm(ref)
    err = np.linalg.norm(tend - ref) / np.linalg.norm(ref)
    assert err < tol, err
