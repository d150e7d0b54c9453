"""Forcing and the learned-closure pipeline on a small grid (GPU)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_forcing_injects_the_requested_power(cuda):
    from fluidsim_gb300.les import make_sim
    from fluidsim_gb300.init_fields import isotropic_3d
    sim = make_sim(32, 1e-2, seed=3)
    v0 = isotropic_3d(32, 32, 32, seed=1)
    sim.state.init_statespect_from(vx_fft=v0[0], vy_fft=v0[1], vz_fft=v0[2])
    ts = sim.time_stepping
    for _ in range(3):
        ts.one_time_step()
    sim.forcing.compute()
    assert abs(sim.forcing.injection_rate() - 1.0) < 1e-4
    # the forced modes are the only ones the forcing touches, and it is solenoidal
    f = sim.forcing.dense.cpu().numpy()
    assert np.count_nonzero(np.abs(f).sum(0)) == len(sim.forcing.flat)


def test_pipeline_small_grid(cuda):
    from fluidsim_gb300 import les
    out = les.pipeline(n_dns=64, n_les=32, nu=5e-3, t_coarse=0.3, t_fine=0.1, n_snap=2,
                       t_between=0.05, train_steps=200, les_steps=100)
    assert out["train"]["rel_mse"] < 1.0
    for name in ("none", "smagorinsky", "learned"):
        assert np.isfinite(out["les"][name]["spectral_error"])
