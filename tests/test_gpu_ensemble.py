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


def _inject_nan(lat):
    """Host-side fault injection: NaN into the f_0 plane of one fluid cell of
    the lattice's current packed state (FP32 storage)."""
    import numpy as np
    solid = lat.geometry.solid
    ys, xs = np.nonzero(~solid[:, lat.W // 4:3 * lat.W // 4])
    y, x = int(ys[len(ys) // 2]), int(xs[len(xs) // 2]) + lat.W // 4
    buf = lat.ppop[lat.pcur]
    buf[4 * (y * lat.W + x):4 * (y * lat.W + x) + 4].view(torch.float32).fill_(float("nan"))


def test_quarantine_of_a_non_finite_member():
    """One member of a batch made non-finite on the host: the batch flags that
    member only (fd_batch_member_status), skips it from then on (its buffers
    no longer change), and every other member stays bit-identical to the same
    lattice stepped alone, also after a new tile table has left the flagged
    member out; clearing the flag and configuring again takes it back."""
    from fingering_dynamics_gb300.ensemble import Ensemble
    from fingering_dynamics_gb300.lattice import Lattice
    members = _members()[:4]
    ens = Ensemble(members, dtype="f32", rows_per_strip=16)
    solo = [Lattice(m[0], m[1], dtype="f32") for m in members]
    for lat in solo:
        lat.enter_fused()
    ens.step(4)
    assert ens.member_status() == [False] * 4
    _inject_nan(ens.lattices[2])
    ens.step(3)
    assert ens.member_status() == [False, False, True, False]
    bad = ens.lattices[2]
    frozen = [b.clone() for b in bad.ppop]
    ens.step(6)
    torch.cuda.synchronize()
    assert all(torch.equal(a, b) for a, b in zip(frozen, bad.ppop)), "a quarantined member was stepped"
    for k in (0, 1, 3):
        solo[k].advance(13)
        torch.cuda.synchronize()
        got, ref = ens.lattices[k], solo[k]
        assert torch.equal(packed_planes(got.ppop[got.pcur], got.H, got.W, "f32"),
                           packed_planes(ref.ppop[ref.pcur], ref.H, ref.W, "f32")), k
    # a new tile table leaves the quarantined member out; the others go on as before
    full = ens.tiles
    ens.configure(*ens.config)
    assert ens.tiles == full - _member_tiles(bad, ens.config)
    assert ens.tiles == ens.tiles_for(*ens.config)
    ens.step(5)
    torch.cuda.synchronize()
    assert all(torch.equal(a, b) for a, b in zip(frozen, bad.ppop)), "a quarantined member was stepped"
    for k in (0, 1, 3):
        solo[k].advance(5)
        torch.cuda.synchronize()
        got, ref = ens.lattices[k], solo[k]
        assert torch.equal(packed_planes(got.ppop[got.pcur], got.H, got.W, "f32"),
                           packed_planes(ref.ppop[ref.pcur], ref.H, ref.W, "f32")), k
    # clearing the flag and configuring again takes the member back
    assert ens.member_status(clear=True)[2]
    assert ens.member_status() == [False] * 4
    ens.configure(*ens.config)
    assert ens.tiles == full
    ens.close()


def _member_tiles(lat, config):
    from fingering_dynamics_gb300.ensemble import tile_count
    return tile_count([(lat.H, lat.W)], *config)


@pytest.mark.parametrize("W", [128, 92], ids=["staged_kernel", "register_kernel"])
def test_single_lattice_reports_non_finite(W):
    """A single lattice made non-finite on the host: the next packed step
    latches FD_STATUS_NONFINITE, which Lattice.check_finite turns into
    FloatingPointError (the reference's np.seterr(all='raise')); a finite
    lattice leaves the bit clear."""
    from fingering_dynamics_gb300 import geometry as geo
    from fingering_dynamics_gb300.lattice import Lattice
    from fingering_dynamics_gb300.params import walls_reference_params
    prm = walls_reference_params().with_size(48, W)
    g = geo.build_geometry(48, W, rects=[((40, 12), (46, 20))], walls=True)
    ok = Lattice(prm, g, dtype="f32")
    ok.check_finite()  # clear
    ok.step(4)
    ok.check_finite()
    lat = Lattice(prm, g, dtype="f32")
    lat.enter_fused()
    _inject_nan(lat)
    lat.advance(2)
    with pytest.raises(FloatingPointError):
        lat.check_finite()
    ok.check_finite()  # cleared by the raising call
