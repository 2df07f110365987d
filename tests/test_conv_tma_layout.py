"""Host model of the TMA-fed tcgen05 convolution (k_conv3x3_tma in
fingering_dynamics_gb300/csrc/sg_tcgen05.cu), no GPU.

The model rebuilds one stage of the kernel's shared memory the way its
tensor-map boxes fill it (unwritten bytes are NaN), reads every MMA operand
through the kernel's matrix-descriptor addressing (canonical K-major layout
without swizzle: element (row, k) at start + (row // 8) * SBO + (row % 8) * 16
+ (k // 8) * LBO + (k % 8) * 2 bytes), accumulates the tiles chunk by chunk
and tap by tap as the kernel issues the MMAs, and compares the result with a
direct 3x3 convolution with zero padding.  It also checks that every box
lands on a 128-byte boundary inside its stage, that every box starts on a
16-byte multiple of its innermost coordinate, and that the accumulators fit
the TMEM columns the kernel allocates.
"""
import numpy as np
import pytest

# the kernel's constants (kTcBM, kHaloPx) and TmaConvCfg<BN, R, S>
BM, PX = 128, 130


def cfg(BN, R):
    a_box = (R + 2) * PX * 16
    c = {"A_BOX": a_box, "SLICE": (a_box + 127) // 128 * 128, "ROWB": PX * 16, "BSL": BN * 16}
    c["A_BYTES"] = 2 * c["SLICE"]
    c["TB"] = 2 * c["BSL"]
    c["STAGE"] = c["A_BYTES"] + 9 * c["TB"]
    c["TX"] = 2 * a_box + 18 * c["BSL"]
    ncol = R * BN
    c["COLS"] = next(v for v in (32, 64, 128, 256, 512) if ncol <= v)
    return c


def smem_bytes(BN, R, S):
    c = cfg(BN, R)
    return S * c["STAGE"] + 2 * S * 8 + 16 + 128


def fill_stage(x, w, n, yy, x0, co0, kc, BN, R):
    """One stage as the boxes of chunk kc write it: float64 per bf16 element
    (index = byte offset // 2), NaN where no box writes."""
    c = cfg(BN, R)
    N, H, W, Cin = x.shape
    st = np.full(c["STAGE"] // 2, np.nan)
    written = 0
    for s in range(2):  # A: 4-D box (8 channels, 130 pixels, R+2 rows, 1 image) at (kc*16+8s, x0-1, yy-1, n)
        ch0 = kc * 16 + 8 * s
        assert (ch0 * 2) % 16 == 0
        dst = s * c["SLICE"]
        assert dst % 128 == 0
        for q in range(R + 2):
            for p in range(PX):
                yi, xi = yy - 1 + q, x0 - 1 + p
                vals = x[n, yi, xi, ch0:ch0 + 8] if (0 <= yi < H and 0 <= xi < W) else np.zeros(8)
                o = (dst + (q * PX + p) * 16) // 2
                st[o:o + 8] = vals
        written += c["A_BOX"]
    for tap in range(9):  # B: 3-D box (8 channels, 1 tap, BN output channels) at (kc*16+8s, tap, co0)
        for s in range(2):
            ch0 = kc * 16 + 8 * s
            dst = c["A_BYTES"] + tap * c["TB"] + s * c["BSL"]
            assert dst % 128 == 0
            for r in range(BN):
                o = (dst + r * 16) // 2
                st[o:o + 8] = w[co0 + r, tap, ch0:ch0 + 8]
            written += c["BSL"]
    assert written == c["TX"]  # the stage's expect_tx byte count
    return st


def operand(st, start, lbo, sbo, rows):
    r = np.arange(rows)[:, None]
    k = np.arange(16)[None, :]
    addr = start + (r // 8) * sbo + (r % 8) * 16 + (k // 8) * lbo + (k % 8) * 2
    assert addr.min() >= 0 and addr.max() + 2 <= 2 * st.size
    return st[addr // 2]


def model_tile(x, w, n, yy, x0, co0, BN, R):
    c = cfg(BN, R)
    Cin = x.shape[3]
    acc = np.zeros((R, BM, BN))
    for kc in range(Cin // 16):
        st = fill_stage(x, w, n, yy, x0, co0, kc, BN, R)
        for tap in range(9):
            ky, kx = tap // 3, tap % 3
            b = operand(st, c["A_BYTES"] + tap * c["TB"], c["BSL"], 128, BN)
            for r in range(R):
                a = operand(st, (r + ky) * c["ROWB"] + kx * 16, c["SLICE"], 128, BM)
                acc[r] += a @ b.T
    return acc


def direct_conv(x, w):
    N, H, W, Cin = x.shape
    Cout = w.shape[0]
    xp = np.zeros((N, H + 2, W + 2, Cin))
    xp[:, 1:-1, 1:-1] = x
    out = np.zeros((N, H, W, Cout))
    for tap in range(9):
        ky, kx = tap // 3, tap % 3
        out += np.einsum("nhwc,oc->nhwo", xp[:, ky:ky + H, kx:kx + W], w[:, tap, :])
    return out


@pytest.mark.parametrize("BN,R,H,W,Cin,Cout", [(64, 4, 8, 256, 32, 128), (32, 2, 6, 128, 16, 32),
                                               (16, 1, 3, 128, 48, 16)])
def test_tma_conv_tiles_match_direct_convolution(BN, R, H, W, Cin, Cout):
    rng = np.random.default_rng(7)
    N = 2
    x = rng.integers(-3, 4, size=(N, H, W, Cin)).astype(np.float64)
    w = rng.integers(-2, 3, size=(Cout, 9, Cin)).astype(np.float64)
    ref = direct_conv(x, w)
    c = cfg(BN, R)
    assert R * BN <= c["COLS"] <= 512
    for rblk in range(N * H // R):  # every tile of the grid
        row = rblk * R
        n, yy = row // H, row % H
        for tx in range(W // BM):
            x0 = tx * BM
            for co0 in range(0, Cout, BN):
                acc = model_tile(x, w, n, yy, x0, co0, BN, R)
                assert np.isfinite(acc).all()  # no operand read an unwritten byte
                for r in range(R):
                    np.testing.assert_array_equal(acc[r], ref[n, yy + r, x0:x0 + BM, co0:co0 + BN])


SM_BYTES = 233472  # shared memory of an SM; 1 KB of it reserved per CTA


def launch_choice(BN, H, Cin, pair=True):
    """The launcher's choice (launch_tma, launch_tma_s, launch_tma_r): rows per
    CTA, stages, the shared memory requested and the CTAs that fit an SM."""
    R = 4 if H % 4 == 0 else (2 if H % 2 == 0 else 1)
    nk = Cin // 16
    half = SM_BYTES // 2 - 1024
    if nk == 1:
        S = 1
    elif pair and BN <= 64 and smem_bytes(BN, R, 2) <= half:
        S = 3 if (nk >= 3 and smem_bytes(BN, R, 3) <= half) else 2
    else:
        S = next(S for S in (4, 3, 2) if (nk >= S or S == 2) and smem_bytes(BN, R, S) <= 227 * 1024)
    smem = smem_bytes(BN, R, S)
    fit = 512 // cfg(BN, R)["COLS"]
    if SM_BYTES // (smem + 1024) > fit:
        smem = SM_BYTES // (fit + 1) - 1024 + 1
    smem = min(smem, 227 * 1024)
    return R, S, smem, SM_BYTES // (smem + 1024)


@pytest.mark.parametrize("pair", [True, False])
def test_launch_choice_fits_shared_and_tensor_memory(pair):
    """For every output tile width, height parity and chunk count: the chosen
    stages fit the shared memory requested, the request fits a CTA, the CTAs
    that fit an SM fit its 512 tensor-memory columns, and a chunk count of
    one takes one stage (a ring of one stage holds only one chunk)."""
    for BN in (16, 32, 64, 128):
        for H in (2, 3, 4, 8):
            for Cin in (16, 32, 48, 64, 96, 384):
                R, S, smem, ctas = launch_choice(BN, H, Cin, pair)
                assert smem_bytes(BN, R, S) <= smem <= 227 * 1024
                assert ctas >= 1 and ctas * cfg(BN, R)["COLS"] <= 512
                assert S == 1 or Cin // 16 >= 2
                assert H % R == 0
    assert smem_bytes(128, 4, 4) > 227 * 1024 and smem_bytes(128, 4, 3) <= 227 * 1024
    # 64-channel tiles are paired (two CTAs an SM); 128-channel tiles keep one CTA of four rows
    assert launch_choice(64, 8, 384)[:2] == (4, 2) and launch_choice(64, 8, 384)[3] == 2
    assert launch_choice(128, 8, 384)[:2] == (4, 3) and launch_choice(128, 8, 384)[3] == 1


# ---------------------------------------------------------------------------
# The tcgen05 weight gradient (k_wgrad_tc): both operands MN-major.
# ---------------------------------------------------------------------------
WG_BGRP = 2176  # bytes between the 8-channel groups of the x halo (130 pixels x 16 B, padded to 128 B)


def operand_mn(st, start, lbo, sbo, rows):
    """MN-major canonical layout without swizzle: element (mn, k) at start +
    (mn // 8) * SBO + (mn % 8) * 2 + (k // 8) * LBO + (k % 8) * 16 bytes (the
    16-byte rows of a core matrix run along MN, its eight rows along K; as for
    K-major operands, LBO strides along K and SBO along MN, the reading the GPU
    tests of the kernel confirm)."""
    mn = np.arange(rows)[:, None]
    k = np.arange(16)[None, :]
    addr = start + (mn // 8) * sbo + (mn % 8) * 2 + (k // 8) * lbo + (k % 8) * 16
    assert addr.min() >= 0 and addr.max() + 2 <= 2 * st.size
    return st[addr // 2]


def wgrad_stage(x, dz, n, y, x0, m0, nn0, ky, BN, sw):
    """One stage of k_wgrad_tc as its boxes fill it.  sw = False: A = dz boxes
    (8 output channels x 128 pixels, groups 2048 B apart) for the groups below
    Cout, B = x boxes (8 input channels x 130 pixels of row y+ky-1, groups
    WG_BGRP apart); sw = True: A = the x boxes (input channels on M), B = the
    dz boxes.  A groups at or beyond the M channel count are zeroed once."""
    N, H, W, Cin = x.shape
    Cout = dz.shape[3]
    agrp, bgrp = (WG_BGRP, 2048) if sw else (2048, WG_BGRP)
    a_bytes = 16 * agrp
    st = np.full((a_bytes + (BN // 8) * bgrp) // 2, np.nan)
    yy = y + ky - 1

    def put_dz(o, co):
        for p in range(128):
            st[o + p * 8:o + p * 8 + 8] = dz[n, y, x0 + p, co:co + 8]

    def put_x(o, ci):
        for p in range(130):
            xi = x0 - 1 + p
            ok = 0 <= yy < H and 0 <= xi < W
            st[o + p * 8:o + p * 8 + 8] = x[n, yy, xi, ci:ci + 8] if ok else 0.0

    mch = Cin if sw else Cout
    for j in range(16):  # A
        o = j * agrp // 2
        ch = m0 + 8 * j
        if ch >= mch:
            st[o:o + agrp // 2] = 0.0  # zeroed once at the start of the kernel
        elif sw:
            put_x(o, ch)
        else:
            put_dz(o, ch)
    for j in range(BN // 8):  # B
        o = (a_bytes + j * bgrp) // 2
        (put_dz if sw else put_x)(o, nn0 + 8 * j)
    return st, a_bytes, agrp, bgrp


@pytest.mark.parametrize("BN,Cin,Cout,sw", [(32, 32, 16, False), (16, 48, 160, False), (16, 48, 16, True),
                                            (32, 144, 32, True)])
def test_wgrad_tc_layout_matches_direct_sum(BN, Cin, Cout, sw):
    rng = np.random.default_rng(3)
    N, H, W = 1, 3, 128
    x = rng.integers(-3, 4, size=(N, H, W, Cin)).astype(np.float64)
    dz = rng.integers(-2, 3, size=(N, H, W, Cout)).astype(np.float64)
    xp = np.zeros((N, H + 2, W + 2, Cin))
    xp[:, 1:-1, 1:-1] = x
    ref = np.zeros((Cout, 9, Cin))
    for tap in range(9):
        ky, kx = tap // 3, tap % 3
        ref[:, tap] = np.einsum("nhwo,nhwc->oc", dz, xp[:, ky:ky + H, kx:kx + W])
    mch, nch = (Cin, Cout) if sw else (Cout, Cin)
    for m0 in range(0, mch, 128):
        for nn0 in range(0, nch, BN):
            for ky in range(3):
                acc = np.zeros((3, 128, BN))
                for y in range(H):  # the chunks: one row segment of 128 pixels each
                    st, a_bytes, agrp, bgrp = wgrad_stage(x, dz, 0, y, 0, m0, nn0, ky, BN, sw)
                    for kx in range(3):
                        ash, bsh = (kx * 16, 0) if sw else (0, kx * 16)
                        for s in range(8):
                            a = operand_mn(st, ash + s * 256, 128, agrp, 128)
                            b = operand_mn(st, a_bytes + bsh + s * 256, 128, bgrp, BN)
                            acc[kx] += a @ b.T
                assert np.isfinite(acc).all()  # no operand read an unwritten byte
                rows = min(128, mch - m0)
                for kx in range(3):
                    got = acc[kx][:rows]
                    want = ref[m0:m0 + rows, ky * 3 + kx, nn0:nn0 + BN] if not sw else \
                        ref[nn0:nn0 + BN, ky * 3 + kx, m0:m0 + rows].T
                    np.testing.assert_array_equal(got, want)
