"""The C-ABI library builds, loads and exports every symbol include/*.h
declares, and the ctypes table binds exactly those (no GPU needed: nothing is
launched)."""
import ctypes
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for fn in sorted(os.listdir(os.path.join(REPO, "include"))):
        if fn.endswith(".h"):
            src = open(os.path.join(REPO, "include", fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names += re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*((?:fd|sg)_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from fingering_dynamics_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "fd_fused_step" in names and "fd_compute_init" in names
    assert len(names) >= 15


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_table_matches_headers():
    from fingering_dynamics_gb300 import _lib as L
    assert sorted(L.SIGNATURES) == declared_functions()
    assert any(n.startswith("sg_") for n in L.SIGNATURES)


def test_abi_version_and_error_path(lib):
    from fingering_dynamics_gb300 import _lib as L
    assert L.lib().fd_abi_version() == 5
    # host-side argument checks run without a GPU and report through fd_last_error
    with pytest.raises(L.FDError) as e:
        L.call("fd_fused_step", None, 1, None, None, None, None, None, None, 1, 0, None)
    assert e.value.code == -1 and "NULL" in str(e.value)
    prm = L.fd_params(10, 10, 7, 0, 0.8, 0.1, 2.0, -0.01, 0.01, 1.0, 0.0, 1.5)
    with pytest.raises(L.FDError) as e:
        L.call("fd_collide", ctypes.byref(prm), 1, None, None, None)
    assert e.value.code == -1
    prm.variant = 0
    with pytest.raises(L.FDError) as e:
        L.call("fd_collide", ctypes.byref(prm), 2, None, None, None)
    assert e.value.code == -4


def test_package_fails_loudly_without_library(monkeypatch):
    from fingering_dynamics_gb300 import _lib as L
    monkeypatch.setattr(L, "_handle", None)
    monkeypatch.setattr(L, "LIB_PATH", "/nonexistent/libfdlbm.so")
    with pytest.raises(RuntimeError, match="not built"):
        L.lib()


def test_new_entry_points_check_their_arguments_on_the_host(lib):
    """The host-resident step, the batch grid query and the wait self-test
    reject bad arguments before touching the device."""
    from fingering_dynamics_gb300 import _lib as L
    prm = L.fd_params(64, 64, 1, 0, 0.8, 0.1, 2.0, -0.01, 0.01, 1.0, 0.0, 1.5)
    st = L.fd_storage(L.FD_F32, 0, 0, 0, 0)
    with pytest.raises(L.FDError) as e:  # NULL buffers
        L.call("fd_fused_step_packed_host", ctypes.byref(prm), ctypes.byref(st), None, None, None, None, None, None,
               None, None, 1, 0, None)
    assert e.value.code == -1 and "NULL" in str(e.value)
    dummy = ctypes.c_void_p(256)
    with pytest.raises(L.FDError) as e:  # no iteration to run
        L.call("fd_fused_step_packed_host", ctypes.byref(prm), ctypes.byref(st), dummy, dummy, dummy, dummy,
               ctypes.c_void_p(512), ctypes.c_void_p(768), ctypes.c_void_p(1024), ctypes.c_void_p(1280), 0, 0, None)
    assert e.value.code == -1
    prm.W = 60  # not a multiple of 8
    with pytest.raises(L.FDError) as e:
        L.call("fd_fused_step_packed_host", ctypes.byref(prm), ctypes.byref(st), dummy, dummy, dummy, dummy,
               ctypes.c_void_p(512), ctypes.c_void_p(768), ctypes.c_void_p(1024), ctypes.c_void_p(1280), 1, 0, None)
    assert e.value.code == -2
    st.rounding = 7  # unknown rounding
    prm.W = 64
    with pytest.raises(L.FDError):
        L.call("fd_fused_step_packed_host", ctypes.byref(prm), ctypes.byref(st), dummy, dummy, dummy, dummy,
               ctypes.c_void_p(512), ctypes.c_void_p(768), ctypes.c_void_p(1024), ctypes.c_void_p(1280), 1, 0, None)
    assert L.lib().fd_batch_grid(None) == -1 and L.lib().fd_batch_tiles(None) == -1
    with pytest.raises(L.FDError) as e:  # no batch
        L.call("fd_batch_member_status", None, (ctypes.c_uint32 * 1)(), 0)
    assert e.value.code == -1
    for polls, unit in ((0, 0), (1 << 21, 0), (100, 2)):
        with pytest.raises(L.FDError) as e:
            L.call("fd_selftest_wait_timeout", polls, unit, None)
        assert e.value.code == -1
    # the TMA-fed convolution takes widths that are multiples of 128 and channel counts that are multiples of 16
    vp = ctypes.c_void_p
    for w, cin, cout, code in ((64, 16, 16, -2), (128, 24, 16, -2), (128, 16, 40, -2), (128, 16, 16, -1)):
        act = 5 if code == -1 else 1  # unknown activation
        for fn in ("sg_conv3x3_tma", "sg_conv3x3_tma_ws"):
            with pytest.raises(L.FDError) as e:
                L.call(fn, vp(256), 1, 4, w, cin, vp(512), None, cout, act, None, vp(768), None)
            assert e.value.code == code
        if code == -2:
            with pytest.raises(L.FDError) as e:
                L.call("sg_conv3x3_wgrad_tc", vp(256), vp(512), 1, 4, w, cin, cout, vp(768), vp(1024), 1 << 20, 0,
                       None)
            assert e.value.code == code


def test_integration_stub_struct_matches_the_binding():
    """The ctypes binding offered to the reference's maintainers
    (fingering_dynamics_gb300/binding/reference_gb300.py, quoted in the
    integration notes) declares fd_params and fd_storage with the same fields,
    types and sizes as the package binding."""
    from fingering_dynamics_gb300 import _lib as L
    from fingering_dynamics_gb300.binding import reference_gb300 as rb
    for stub, ours in ((rb.fd_params, L.fd_params), (rb.fd_storage, L.fd_storage)):
        assert [n for n, _ in stub._fields_] == [n for n, _ in ours._fields_]
        assert ctypes.sizeof(stub) == ctypes.sizeof(ours)
        for (n, t), (_, u) in zip(stub._fields_, ours._fields_):
            assert ctypes.sizeof(t) == ctypes.sizeof(u), n


def test_wgrad_partial_buffer_covers_both_kernels():
    """sg_wgrad_partial_floats (a host function) sizes the FP32 partial buffer
    for the warp-level weight gradient's splits and, at widths that are
    multiples of 128, for the tcgen05 one's: the most CTAs that fill two waves
    of one CTA per SM (152 SMs), three taps per CTA, the larger channel count
    on 128 rows, no more splits than 128-pixel chunks."""
    from fingering_dynamics_gb300 import _lib as L
    lib = L.lib()
    for n, h, w, cin, cout in [(32, 256, 512, 96, 32), (32, 64, 128, 384, 128), (32, 128, 256, 64, 192),
                               (32, 64, 128, 128, 128), (1, 2, 128, 16, 16), (2, 8, 40, 32, 32)]:
        got = int(lib.sg_wgrad_partial_floats(n, h, w, cin, cout))
        per_split = cout * 9 * cin
        assert got % per_split == 0 and got >= per_split
        if w % 128 == 0:
            mrows, nch = max(cin, cout), min(cin, cout)
            bn = next(b for b in (128, 64, 32, 16) if nch % b == 0)
            per = -(-mrows // 128) * (nch // bn) * 3
            want = max(1, min(n * h * (w // 128), (2 * 152) // per))
            assert got >= want * per_split, (n, h, w, cin, cout, got // per_split, want)
    assert lib.sg_wgrad_partial_floats(0, 1, 128, 16, 16) == 0
