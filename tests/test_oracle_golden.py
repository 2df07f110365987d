"""The oracle against the reference's own outputs (golden fixtures made by
tests/golden/make_golden.py).  The oracle keeps the reference's operand
order, so the comparison is bit-for-bit."""
import hashlib

import numpy as np
import pytest

from fixtures import FIELDS, load, oracle_fields, oracle_from_fixture

SMALL = ["periodic_circles_24x48", "walls_rects_24x48"]
LONG = ["periodic_circles_64x128_500", "walls_rects_64x128_500"]


def _eq(a, b):
    return np.array_equal(a, b, equal_nan=True)


@pytest.mark.parametrize("name", SMALL)
def test_oracle_init_bitwise(name):
    fx = load(name)
    st, _, _ = oracle_from_fixture(fx)
    got = oracle_fields(st)
    for k in ("f", "g") + FIELDS:
        assert _eq(got[k], fx[f"s0_{k}"]), k


@pytest.mark.parametrize("name", SMALL)
def test_oracle_phases_and_steps_bitwise(name):
    fx = load(name)
    st, corners, circ = oracle_from_fixture(fx)
    from oracle import lbm_oracle as O
    phases = set(int(p) for p in fx["phases_at"])
    snaps = set(int(s) for s in fx["snap_steps"])
    for i in range(int(fx["steps"])):
        if i in phases:
            # replay the step phase by phase and compare each intermediate
            st.collide()
            assert _eq(st.f, fx[f"p{i}_collided_f"]) and _eq(st.g, fx[f"p{i}_collided_g"])
            fb, gb = st.f.copy(), st.g.copy()
            st.f, st.g = O.stream(st.f), O.stream(st.g)
            assert _eq(st.f, fx[f"p{i}_streamed_f"]) and _eq(st.g, fx[f"p{i}_streamed_g"])
            if corners:
                O.halfway_bounceback_rec(corners, fb, gb, st.f, st.g)
            if circ is not None:
                O.halfway_bounceback_circle(*circ, fb, gb, st.f, st.g)
            if st.prm.variant == "walls":
                O.bottom_top_wall(fb[:, 1:-1], gb[:, 1:-1], st.f[:, 1:-1], st.g[:, 1:-1])
            assert _eq(st.f, fx[f"p{i}_bounced_f"]) and _eq(st.g, fx[f"p{i}_bounced_g"])
            st.zou_he()
            assert _eq(st.f, fx[f"p{i}_zouhe_f"]) and _eq(st.g, fx[f"p{i}_zouhe_g"])
            st.macros()
            st.steps += 1
        else:
            st.step(corners, circ)
        if i + 1 in snaps:
            got = oracle_fields(st)
            for k in ("f", "g") + FIELDS:
                assert _eq(got[k], fx[f"s{i + 1}_{k}"]), (i + 1, k)


@pytest.mark.parametrize("name", LONG)
def test_oracle_500_steps_bitwise(name):
    fx = load(name)
    st, corners, circ = oracle_from_fixture(fx)
    n = int(fx["steps"])
    for _ in range(n):
        st.step(corners, circ)
    got = oracle_fields(st)
    for k in FIELDS:
        assert _eq(got[k], fx[f"s{n}_{k}"]), k
    assert hashlib.sha256(st.f.tobytes()).hexdigest() == str(fx[f"s{n}_f_sha256"])
    assert hashlib.sha256(st.g.tobytes()).hexdigest() == str(fx[f"s{n}_g_sha256"])
