"""Parity at the full workload size through a size-independent property: the
FP64 fused kernel equals the oracle bit for bit (test_gpu_parity.py), so at
4096 x 2048 it is the reference for the packed kernels over a short run.
Also the edge cases of the step API: zero steps, the smallest lattices."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fingering_dynamics_gb300 import build
    build.build()


def test_full_size_packed_kernels_follow_fp64():
    from bench import workload
    from fingering_dynamics_gb300.lattice import Lattice
    prm, g = workload(2048, 4096)
    fluid = torch.from_numpy(~g.solid).cuda()
    ref = Lattice(prm, g, dtype="f64")
    ref.step(40)
    psi64 = ref.psi.clone()
    rho64 = ref.rho.clone()
    del ref
    torch.cuda.empty_cache()
    for dtype, tol in (("f32", 1e-5), ("f16", 1e-3)):
        lat = Lattice(prm, g, dtype=dtype)
        lat.step(40)
        dpsi = (lat.psi.double() - psi64).abs()[fluid].max().item()
        drho = (lat.rho.double() - rho64).abs()[fluid].max().item()
        assert dpsi <= tol and drho <= tol, (dtype, dpsi, drho)
        del lat
        torch.cuda.empty_cache()


def test_zero_steps_is_a_no_op():
    from bench import workload
    from fingering_dynamics_gb300.lattice import Lattice
    prm, g = workload(32, 64)
    for dtype in ("f64", "f32", "f16"):
        lat = Lattice(prm, g, dtype=dtype)
        before = lat.current_buffer().clone()
        lat.step(0)
        lat.enter_fused()
        fused = lat.current_buffer().clone()
        lat.advance(0)
        assert torch.equal(lat.current_buffer(), fused) and lat.iteration == 0
        assert before.shape[0] == 18


@pytest.mark.parametrize("dtype", ["f64", "f32", "f16"])
def test_smallest_walled_lattice(dtype):
    """H = 3 (one fluid row between the wall rows) and the narrowest widths
    the fused kernels take run and stay finite."""
    from fingering_dynamics_gb300 import geometry as geo
    from fingering_dynamics_gb300.lattice import Lattice
    from fingering_dynamics_gb300.params import walls_reference_params
    W = 16 if dtype != "f64" else 8
    prm = walls_reference_params().with_size(3, W)
    g = geo.build_geometry(3, W, walls=True)
    lat = Lattice(prm, g, dtype=dtype)
    lat.step(20)
    assert bool(torch.isfinite(lat.psi).all())
