"""Batched ensembles: every member advanced by the persistent batched launch
(with and without the CUDA graph, for every tile shape) equals the same member
advanced alone, bit for bit."""
import pytest

from fixtures import packed_planes

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _members():
    from fingering_dynamics_gb300.ensemble import ensemble_specs
    specs = ensemble_specs(5, seed=3, sizes_w=(64, 128, 256), sizes_h=(48, 64, 96), ratio=(2.0, 5.0))
    return [s.build() for s in specs]


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fingering_dynamics_gb300 import build
    build.build()


@pytest.mark.parametrize("dtype", ["f32", "f16"])
def test_batch_equals_single_lattices(dtype):
    from fingering_dynamics_gb300.ensemble import Ensemble
    from fingering_dynamics_gb300.lattice import Lattice
    members = _members()
    ens = Ensemble(members, dtype=dtype, rows_per_strip=16, band_width=64)
    singles = [Lattice(p, g, dtype=dtype, seed=k) for k, (p, g) in enumerate(members)]
    for s in singles:
        s.enter_fused()
    ens.step(3, use_graph=False)
    ens.step(6, use_graph=True)
    ens.configure(256, 7)
    ens.step(5, use_graph=True)
    for s in singles:
        s.advance(14)
    torch.cuda.synchronize()
    for a, b in zip(ens.lattices, singles):
        assert a.iteration == b.iteration
        assert torch.equal(packed_planes(a.current_buffer(), a.H, a.W, dtype),
                           packed_planes(b.current_buffer(), b.H, b.W, dtype))
        assert torch.equal(a.side[a.scur], b.side[b.scur])
    ens.close()


def test_autotune_and_diagnostics():
    from fingering_dynamics_gb300.ensemble import Ensemble
    ens = Ensemble(_members(), dtype="f32")
    res = ens.autotune(steps=4)
    assert len(res) >= 3 and all(v > 0 for v in res.values())
    assert ens.config == max(res, key=res.get)
    ens.step(4)
    d = ens.diagnostics()
    assert len(d) == 5 and all(x["fluid"] > 0 and 0.0 <= x["saturation"] <= 1.0 for x in d)
    ens.close()
