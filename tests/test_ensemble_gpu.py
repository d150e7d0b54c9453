"""Batched ns2d ensembles against individually solved runs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_ensemble_matches_individual_runs(cuda):
    from fluidsim_gb300.ensemble import EnsembleNS2D, make_group, reference_run
    groups = [make_group(128, 3, seed=1), make_group(256, 2, seed=2)]
    ens = EnsembleNS2D(groups)
    ens.autotune(steps=1, candidates=[(8, 2, 8), (16, 4, 4)])
    ens.run(20)
    assert not ens.nan_flag()
    for gi, g in enumerate(groups):
        got = ens.groups[gi]["S"].cpu().numpy()
        for i in range(len(g["nu2"])):
            ref = reference_run(g, i, 20)
            assert np.linalg.norm(got[i] - ref) / np.linalg.norm(ref) < 2e-5
            ref32 = reference_run(g, i, 20, precision="float32")
            # same kernels, same order of operations as a single float32 run
            assert np.linalg.norm(got[i] - ref32) / np.linalg.norm(ref32) < 1e-6


def test_graph_replay_equals_direct_launch(cuda):
    from fluidsim_gb300.ensemble import EnsembleNS2D, make_group
    groups = [make_group(128, 2, seed=5), make_group(256, 2, seed=6)]
    ens = EnsembleNS2D(groups)
    ens.run(6)
    direct = [g["S"].clone() for g in ens.groups]
    ens.reset()
    ens.capture(3)
    ens.reset()
    ens.run(6)
    for g, d in zip(ens.groups, direct):
        assert np.array_equal(g["S"].cpu().numpy(), d.cpu().numpy())
