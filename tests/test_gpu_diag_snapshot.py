"""Diagnostics against the oracle, and bitwise checkpoint / resume."""
import numpy as np
import pytest

from fixtures import load, oracle_from_fixture, packed_planes

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fingering_dynamics_gb300 import build
    build.build()


def _lattice(name, dtype):
    from test_gpu_parity import make_lattice
    return make_lattice(load(name), dtype)


@pytest.mark.parametrize("name", ["periodic_circles_24x48", "walls_rects_24x48"])
def test_diagnostics_fp64_match_oracle(name):
    from oracle.lbm_oracle import diagnostics
    fx = load(name)
    lat = _lattice(name, "f64")
    lat.step(40)
    got = lat.diagnostics()
    st, corners, circ = oracle_from_fixture(fx)
    for _ in range(40):
        st.step(corners, circ)
    ref = diagnostics(st)
    for k in ("invaded", "fluid", "tip_x", "breakthrough"):
        assert got[k] == ref[k], k
    for k in ("mass_r", "mass_b", "saturation"):
        assert abs(got[k] - ref[k]) <= 1e-12 * max(1.0, abs(ref[k])), (k, got[k], ref[k])


@pytest.mark.parametrize("dtype", ["f32", "f16"])
def test_diagnostics_packed_state(dtype):
    """Diagnostics read from the packed fused state agree with those of the
    reference-mode state after the same number of iterations."""
    name = "walls_rects_64x128_500"
    lat = _lattice(name, dtype)
    lat.enter_fused()
    lat.advance(99)
    packed = lat.diagnostics()           # post-collision state of iteration 99
    lat.exit_fused()                     # reference mode at iteration 100
    ref = _lattice(name, dtype)
    ref.step(99)                         # reference mode at iteration 99
    plain = ref.diagnostics()
    assert packed["fluid"] == plain["fluid"]
    assert abs(packed["invaded"] - plain["invaded"]) <= 2
    assert abs(packed["mass_r"] - plain["mass_r"]) <= 1e-4 * plain["mass_r"]


@pytest.mark.parametrize("dtype", ["f64", "f32", "f16"])
def test_snapshot_resume_bitwise(dtype, tmp_path):
    name = "walls_rects_24x48"
    straight = _lattice(name, dtype)
    straight.enter_fused()
    straight.advance(9)
    a = _lattice(name, dtype)
    a.enter_fused()
    a.advance(4)
    a.save_snapshot(str(tmp_path / "s.npz"))
    b = _lattice(name, dtype)
    b.load_snapshot(str(tmp_path / "s.npz"))
    b.advance(5)
    assert b.iteration == straight.iteration
    if dtype == "f64":
        assert torch.equal(b.current_buffer(), straight.current_buffer())
    else:  # packed: compare the planes, not the padding between them
        assert torch.equal(packed_planes(b.current_buffer(), b.H, b.W, dtype),
                           packed_planes(straight.current_buffer(), b.H, b.W, dtype))
    # reference-mode snapshot
    straight.exit_fused()
    c = _lattice(name, dtype)
    c.step(4)
    c.save_snapshot(str(tmp_path / "r.npz"))
    d = _lattice(name, dtype)
    d.load_snapshot(str(tmp_path / "r.npz"))
    d.step(6)
    e = _lattice(name, dtype)   # the same kernel sequence without the snapshot
    e.step(4)
    e.step(6)
    for k, v in e.state().items():
        assert np.array_equal(v, d.state()[k], equal_nan=True), k
