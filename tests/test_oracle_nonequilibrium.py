"""The oracle's restatement of the regularised restart's first-order
non-equilibrium part carries no density, psi or momentum, and vanishes for a
uniform flow."""
import numpy as np

from oracle.lbm_oracle import EX, EY, OracleParams, nonequilibrium


def _params(H, W, variant):
    return OracleParams(H=H, W=W, variant=variant, tau=0.8, eta_n=0.1, M=3.0, a=-0.05, kappa=0.1, gamma=1.0,
                        psi_wall=-0.5, inlet_ux=np.zeros(H), outlet_coef=1.5)


def test_moments_vanish():
    H, W = 16, 24
    rng = np.random.default_rng(0)
    solid = rng.random((H, W)) < 0.2
    for variant in ("walls", "periodic", "periodic_xy"):
        df, dg = nonequilibrium(1 + 0.01 * rng.random((H, W)), rng.uniform(-1, 1, (H, W)),
                                0.01 * rng.random((H, W)), 0.01 * rng.random((H, W)), 0.8 + 0.1 * rng.random((H, W)),
                                solid, _params(H, W, variant))
        assert np.abs(df).max() > 1e-4
        for d in (df, dg):
            assert np.abs(d.sum(axis=0)).max() < 1e-16
            assert np.abs((d * EX[:, None, None]).sum(axis=0)).max() < 1e-16
            assert np.abs((d * EY[:, None, None]).sum(axis=0)).max() < 1e-16
            assert not d[:, solid].any()


def test_uniform_flow_has_none():
    H, W = 8, 12
    one = np.ones((H, W))
    df, dg = nonequilibrium(one, 0.3 * one, 0.01 * one, -0.02 * one, 0.9 * one, np.zeros((H, W), bool),
                            _params(H, W, "periodic_xy"))
    assert np.abs(df).max() < 1e-18 and np.abs(dg).max() < 1e-18
