"""CUDA path against the reference's outputs (golden fixtures) and the oracle.

FP64: the reference-order kernels and the fused kernel are compared with the
reference's own outputs bit for bit (the kernels keep the reference's
operand order and are built without FMA contraction).
FP32: fields after 500 steps agree with the FP64 oracle to 1e-5 relative
(normwise: max |a - b| <= 1e-5 * max |b| per field).
"""
import numpy as np
import pytest

from fixtures import FIELDS, fixture_geometry, lbm_params, load, oracle_fields, oracle_from_fixture

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

SMALL = ["periodic_circles_24x48", "walls_rects_24x48"]
LONG = ["periodic_circles_64x128_500", "walls_rects_64x128_500"]
FP32_REL = 1e-5


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fingering_dynamics_gb300 import build
    build.build()


def make_lattice(fx, dtype):
    from fingering_dynamics_gb300 import geometry as geo
    from fingering_dynamics_gb300.lattice import Lattice
    prm = lbm_params(fx)
    H, W = prm.H, prm.W
    rects = [((int(r[0]), int(r[1])), (int(r[2]), int(r[3]))) for r in fx["rects"]]
    circles = [((int(c[0]), int(c[1])), int(c[2])) for c in fx["circles"]]
    g = geo.build_geometry(H, W, rects=rects, circles=circles, walls=prm.variant == "walls")
    _, rho0, _, _ = fixture_geometry(fx)
    return Lattice(prm, g, dtype=dtype, device="cuda", rho0=rho0)


def _eq(a, b):
    return np.array_equal(a, b, equal_nan=True)


def _first_diff(a, b):
    d = np.abs(np.nan_to_num(a) - np.nan_to_num(b))
    return float(d.max()), np.unravel_index(int(d.argmax()), d.shape)


@pytest.mark.parametrize("name", SMALL)
def test_init_bitwise(name):
    fx = load(name)
    lat = make_lattice(fx, "f64")
    st = lat.state()
    for k in ("f", "g") + FIELDS:
        assert _eq(st[k], fx[f"s0_{k}"]), (k, _first_diff(st[k], fx[f"s0_{k}"]))


@pytest.mark.parametrize("name", SMALL)
def test_reference_order_steps_bitwise(name):
    fx = load(name)
    lat = make_lattice(fx, "f64")
    snaps = sorted(int(s) for s in fx["snap_steps"])
    done = 0
    for s in snaps:
        lat.step_reference(s - done)
        done = s
        st = lat.state()
        for k in ("f", "g") + FIELDS:
            assert _eq(st[k], fx[f"s{s}_{k}"]), (s, k, _first_diff(st[k], fx[f"s{s}_{k}"]))


@pytest.mark.parametrize("name", SMALL)
def test_fused_steps_bitwise(name):
    fx = load(name)
    lat = make_lattice(fx, "f64")
    snaps = sorted(int(s) for s in fx["snap_steps"])
    done = 0
    for s in snaps:
        lat.step(s - done)
        done = s
        st = lat.state()
        for k in ("f", "g") + FIELDS:
            assert _eq(st[k], fx[f"s{s}_{k}"]), (s, k, _first_diff(st[k], fx[f"s{s}_{k}"]))


@pytest.mark.parametrize("rows", [1, 3, 7, 64])
def test_fused_strip_heights_agree(rows):
    """The result must not depend on how many rows a warp marches."""
    fx = load("walls_rects_24x48")
    ref = make_lattice(fx, "f64")
    ref.step_reference(12)
    lat = make_lattice(fx, "f64")
    lat.enter_fused()
    lat.advance(11, rows_per_warp=rows)
    lat.exit_fused()
    a, b = lat.state(), ref.state()
    for k in ("f", "g") + FIELDS:
        assert _eq(a[k], b[k]), (rows, k)


@pytest.mark.parametrize("name", LONG)
def test_fused_500_steps_fp64_bitwise(name):
    fx = load(name)
    lat = make_lattice(fx, "f64")
    lat.step(500)
    st = lat.state()
    for k in FIELDS:
        assert _eq(st[k], fx[f"s500_{k}"]), (k, _first_diff(st[k], fx[f"s500_{k}"]))


def _colour_fields(st):
    rho, psi = st["rho"], st["psi"]
    return {"rho_r": rho * (1 + psi) / 2, "rho_b": rho * (1 - psi) / 2, "ux": st["ux"], "uy": st["uy"]}


@pytest.mark.parametrize("name", LONG)
def test_fused_500_steps_fp32_vs_oracle(name):
    fx = load(name)
    lat = make_lattice(fx, "f32")
    lat.step(500)
    got = _colour_fields(lat.state())
    ref = _colour_fields({k: fx[f"s500_{k}"] for k in ("rho", "psi", "ux", "uy")})
    for k in got:
        a, b = got[k], ref[k]
        m = np.isfinite(b)
        err = np.abs(a[m] - b[m]).max()
        scale = np.abs(b[m]).max()
        assert err <= FP32_REL * scale, (k, err, scale)


def test_fused_matches_oracle_on_random_blocks():
    """A geometry not in the fixtures: seeded circles and squares, walls."""
    from fingering_dynamics_gb300 import geometry as geo
    from fingering_dynamics_gb300.lattice import Lattice
    from fingering_dynamics_gb300.params import walls_reference_params
    from oracle.lbm_oracle import OracleParams, OracleState
    H, W = 48, 96
    prm = walls_reference_params().with_size(H, W)
    rects, circles = geo.random_blocks(H, W, 0.8, 3, 6, seed=11, x_margin=8)
    g = geo.build_geometry(H, W, rects=rects, circles=circles, walls=True)
    rng = np.random.default_rng(2)
    rho0 = 1.0 - 0.001 * rng.random((H, W))
    lat = Lattice(prm, g, dtype="f64", rho0=rho0)
    lat.step(60)
    op = OracleParams(H=H, W=W, variant="walls", tau=prm.tau, eta_n=prm.eta_n, M=prm.M, a=prm.a, kappa=prm.kappa,
                      gamma=prm.gamma, psi_wall=prm.psi_wall, inlet_ux=prm.inlet_ux, outlet_coef=prm.outlet_coef)
    st = OracleState(op, g.solid, prm.initial_psi(g.solid), rho0=rho0, init_mu=True, init_uy=True)
    for _ in range(60):
        st.step(g.corner_list, g.circle_masks)
    ref = oracle_fields(st)
    got = lat.state()
    for k in ("f", "g") + FIELDS:
        assert _eq(got[k], ref[k]), (k, _first_diff(got[k], ref[k]))
