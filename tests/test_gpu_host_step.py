"""The host-resident step (fd_fused_step_packed_host through
Lattice.advance_host) against the resident step: the state uploaded from host
memory, advanced over pipelined row chunks and downloaded must equal, byte for
byte, the same iterations of fd_fused_step_packed on the device, for every
storage type, both variants, heights that are not a multiple of the chunk, and
several chunk sizes, in place and into a separate buffer, over repeated calls.
"""
import pytest

from fixtures import packed_planes as planes

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fingering_dynamics_gb300 import build
    build.build()


def pair(variant, H, W, dtype, rounding="stochastic"):
    from fingering_dynamics_gb300 import geometry as geo
    from fingering_dynamics_gb300.lattice import Lattice
    from fingering_dynamics_gb300.params import from_relaxation_times
    prm = from_relaxation_times(H, W, 0.6, 1.0, 5e-4, 120.0, 0.01, variant=variant)
    rects, circles = geo.random_blocks(H, W, 0.8, 3, 6, seed=7, x_margin=8)
    g = geo.build_geometry(H, W, rects=rects, circles=circles, walls=variant == "walls")
    kw = {} if dtype == "f32" else {"rounding": rounding}
    out = []
    for _ in range(2):
        lat = Lattice(prm, g, dtype=dtype, device="cuda", seed=11, **kw)
        lat.step(3)
        lat.enter_fused()
        out.append(lat)
    return out


def pinned_copy(t):
    h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
    h.copy_(t)
    return h


CASES = [("walls", 75, 96, "f32"), ("periodic", 130, 256, "f32"), ("walls", 130, 256, "f16"),
         ("periodic", 74, 96, "bf16"), ("walls", 75, 96, "bf16"), ("walls", 1000, 64, "f32")]


@pytest.mark.parametrize("variant,H,W,dtype", CASES, ids=[f"{c[0]}_{c[1]}x{c[2]}_{c[3]}" for c in CASES])
@pytest.mark.parametrize("chunk_rows", [0, 16, 7, 48, 10000])
def test_host_step_equals_resident_step(variant, H, W, dtype, chunk_rows):
    ref, lat = pair(variant, H, W, dtype)
    host = pinned_copy(lat.current_buffer())
    out = torch.empty_like(host).pin_memory()
    # calls of 1, 2 and 3 iterations: in place, then into a separate buffer
    for n, dst in ((1, None), (2, out), (3, None)):
        ref.advance(n)
        lat.advance_host(host, dst, n=n, chunk_rows=chunk_rows)
        torch.cuda.synchronize()
        got = out if dst is not None else host
        want = ref.current_buffer()
        assert torch.equal(planes(got, H, W, dtype), planes(want, H, W, dtype)), \
            f"{n} iterations differ from the resident step"
        assert torch.equal(planes(lat.current_buffer(), H, W, dtype), planes(want, H, W, dtype))
        assert torch.equal(lat.side[lat.scur], ref.side[ref.scur])
        assert lat.iteration == ref.iteration
        if dst is not None:
            host.copy_(out)


def test_host_step_rejects_bad_buffers():
    from fingering_dynamics_gb300 import _lib as L
    _, lat = pair("walls", 75, 96, "f32")
    host = pinned_copy(lat.current_buffer())
    with pytest.raises(ValueError):
        lat.advance_host(host[:-1])
    with pytest.raises(ValueError):
        lat.advance_host(host.cuda())
    with pytest.raises(L.FDError):
        a, b = lat.ppop[lat.pcur], lat.ppop[1 - lat.pcur]
        import ctypes as C
        L.call("fd_fused_step_packed_host", C.byref(lat.prm), C.byref(lat.storage), C.c_void_p(lat.mask.data_ptr()),
               C.c_void_p(lat.inlet_ux.data_ptr()), C.c_void_p(host.data_ptr()), C.c_void_p(host.data_ptr()),
               C.c_void_p(a.data_ptr()), C.c_void_p(a.data_ptr()), C.c_void_p(lat.side[0].data_ptr()),
               C.c_void_p(lat.side[1].data_ptr()), 1, 0, None)
