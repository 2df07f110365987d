"""The fused step entry point that allocates nothing
(fd_fused_step_packed_noalloc) against the regular one.

It exists for callers that cannot allocate device memory themselves: a host
whose memory manager owns all of device memory and does not let a library
call cudaMalloc.  Such a caller passes one boundary buffer instead of two; the
library keeps the second in a fixed device array.  Two calls in a row must give
exactly what fd_fused_step_packed gives with two caller buffers, on both
kernels the packed step uses (the staged kernel for widths that are a
multiple of 8, the register kernel otherwise) and for FP32 and FP16 storage.
"""
import ctypes as C

import pytest

from fixtures import packed_planes

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _lattice(dtype, W):
    from fingering_dynamics_gb300 import build
    from fingering_dynamics_gb300 import geometry as geo
    from fingering_dynamics_gb300.lattice import Lattice
    from fingering_dynamics_gb300.params import walls_reference_params
    build.build()
    H = 48
    prm = walls_reference_params().with_size(H, W)
    g = geo.build_geometry(H, W, rects=[((30, 12), (38, 20))], circles=[((64, 30), 6)], walls=True)
    lat = Lattice(prm, g, dtype=dtype)
    lat.enter_fused()
    return lat


def _p(t):
    return C.c_void_p(t.data_ptr())


@pytest.mark.parametrize("W", [96, 92], ids=["staged_kernel", "register_kernel"])
@pytest.mark.parametrize("dtype", ["f32", "f16"])
@pytest.mark.parametrize("nsteps", [3, 4])
def test_noalloc_matches_regular_entry_point(nsteps, dtype, W):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fingering_dynamics_gb300 import _lib as L
    ref = _lattice(dtype, W)
    lat = _lattice(dtype, W)
    a = [ref.ppop[ref.pcur].clone(), ref.ppop[1 - ref.pcur].clone()]
    b = [lat.ppop[lat.pcur].clone(), lat.ppop[1 - lat.pcur].clone()]
    sides = [ref.side[ref.scur].clone(), torch.zeros_like(ref.side[0])]
    side = lat.side[lat.scur].clone()
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        L.call("fd_fused_step_packed", C.byref(ref.prm), C.byref(ref.storage), _p(ref.mask), _p(ref.inlet_ux),
               _p(a[0]), _p(a[1]), _p(sides[0]), _p(sides[1]), nsteps, 0, s)
        L.call("fd_fused_step_packed_noalloc", C.byref(lat.prm), C.byref(lat.storage), _p(lat.mask),
               _p(lat.inlet_ux), _p(b[0]), _p(b[1]), _p(side), nsteps, 0, s)
        if nsteps % 2:
            a.reverse()
            b.reverse()
            sides.reverse()
        torch.cuda.synchronize()
        # the planes only: the padding that rounds each plane up to 256 bytes is never written
        assert torch.equal(packed_planes(a[0], ref.H, ref.W, dtype), packed_planes(b[0], lat.H, lat.W, dtype)), \
            f"populations differ after call {call + 1}"
        assert torch.equal(sides[0], side), f"boundary values differ after call {call + 1}"


def test_noalloc_rejects_tall_lattice():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fingering_dynamics_gb300 import _lib as L
    lat = _lattice("f32", 96)
    prm = L.fd_params.from_buffer_copy(lat.prm)
    prm.H = 16385
    with pytest.raises(L.FDError) as e:
        L.call("fd_fused_step_packed_noalloc", C.byref(prm), C.byref(lat.storage), _p(lat.mask), _p(lat.inlet_ux),
               _p(lat.ppop[0]), _p(lat.ppop[1]), _p(lat.side[0]), 1, 0, None)
    assert e.value.code == -5 and "16384" in str(e.value)
