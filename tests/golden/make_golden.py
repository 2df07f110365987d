"""Generate the golden fixtures in this folder by running the reference itself.

Run from the repository root in a checkout where the reference is available:

    python tests/golden/make_golden.py /root/reference

The reference scripts (lattice_boltzmann/fingering_periodic.py,
fingering.py, bounce_back.py, create_block.py) are imported unmodified.  Two
modules they import are not installed and are replaced by stand-ins:

* ``matplotlib`` (plotting only) -> empty modules;
* ``cv2`` (block outlines, create_block.py:15,21,40-41) -> ``circle``,
  ``rectangle``, ``findNonZero`` and ``boundingRect`` backed by this
  package's own rasterisers, so the reference and the package see the same
  outlines.

The driver loop below replays the reference's main-loop body
(fingering_periodic.py:454-479, fingering.py:558-585) against the reference's
own ``Compute``, ``stream``, ``Bounce_back`` and ``bottom_top_wall``; module
globals are set from the fixture's parameter set before ``Compute`` is built.
Outputs are written as compressed .npz files next to this script.
"""
from __future__ import annotations

import copy
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from fingering_dynamics_gb300 import geometry as geo  # noqa: E402
from fingering_dynamics_gb300.params import (  # noqa: E402
    periodic_reference_params, walls_reference_params)


def install_stubs():
    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")
    anim = types.ModuleType("matplotlib.animation")
    mpl.pyplot = plt
    mpl.animation = anim
    sys.modules.update({"matplotlib": mpl, "matplotlib.pyplot": plt, "matplotlib.animation": anim})

    cv2 = types.ModuleType("cv2")

    def _draw(img, pts, color):
        H, W = img.shape[:2]
        for x, y in pts:
            if 0 <= x < W and 0 <= y < H:
                img[y, x] = color[0]

    def circle(img, center, radius, color, *a, **k):
        _draw(img, geo.circle_outline(center[0], center[1], radius), color)
        return img

    def rectangle(img, pt1, pt2, color, *a, **k):
        _draw(img, geo.rectangle_outline(pt1, pt2), color)
        return img

    def findNonZero(img):
        ys, xs = np.nonzero(img)
        return np.stack([xs, ys], axis=1).reshape(-1, 1, 2)

    def boundingRect(points):
        p = np.asarray(points).reshape(-1, 2)
        x, y = int(p[:, 0].min()), int(p[:, 1].min())
        return x, y, int(p[:, 0].max()) - x + 1, int(p[:, 1].max()) - y + 1

    cv2.circle, cv2.rectangle = circle, rectangle
    cv2.findNonZero, cv2.boundingRect = findNonZero, boundingRect
    sys.modules["cv2"] = cv2


def import_reference(ref_root):
    install_stubs()
    sys.path.insert(0, os.path.join(ref_root, "lattice_boltzmann"))
    import io
    import contextlib
    with contextlib.redirect_stdout(io.StringIO()):
        import fingering_periodic as fp
        import fingering as fw
        import bounce_back as bbm
        import create_block as cbm
    return fp, fw, bbm, cbm


def set_globals(mod, prm):
    mod.H, mod.W = prm.H, prm.W
    mod.tau = prm.tau
    mod.Eta_n = prm.eta_n
    mod.M = prm.M
    mod.a = prm.a
    mod.kappa = prm.kappa
    mod.gamma = prm.gamma
    mod.psi_wall = prm.psi_wall
    mod.u0 = prm.u0


def params_record(prm):
    return {k: np.array(getattr(prm, k)) for k in
            ("H", "W", "tau", "eta_n", "M", "a", "kappa", "gamma", "psi_wall", "u0",
             "outlet_coef", "slab")} | {"variant": np.array(prm.variant), "inlet_ux": prm.inlet_ux}


def snapshot(cm, H, W, tag):
    m = cm.mask
    out = {f"{tag}_f": cm.f.copy(), f"{tag}_g": cm.g.copy(), f"{tag}_psi": cm.psi.copy(),
           f"{tag}_npx": np.asarray(cm.nabla_psix).copy(), f"{tag}_npy": np.asarray(cm.nabla_psiy).copy(),
           f"{tag}_np2": np.asarray(cm.nabla_psi2).copy()}
    for name in ("rho", "ux", "uy", "p", "mu", "mix_tau"):
        full = np.full((H, W), np.nan)
        full[m] = getattr(cm, name)
        out[f"{tag}_{name}"] = full
    return out


def run_case(fp, fw, bbm, cbm, variant, prm, rects, circles, steps, snap_steps, phases_at, seed=None,
             finals_only=False):
    mod = fp if variant == "periodic" else fw
    set_globals(mod, prm)
    H, W = prm.H, prm.W
    cr = cbm.Createblock(H, W)
    bb = bbm.Bounce_back(H, W)
    rec = {}
    corner_list, lists = [], None
    bpa = np.zeros((H, W), dtype=int)
    if rects:
        b, corner_list = cr.setblock(rects)
        bpa = bpa + b
    if circles:
        b, side_list, concave_list, convex_list = cr.setCirleblock(circles)
        bpa = bpa + b
        lists = (side_list, concave_list, convex_list)
    block_mask = np.where(bpa == 1, True, False)
    mask = np.logical_not(block_mask)
    if seed is not None:
        np.random.seed(seed)
    cm = mod.Compute(mask)
    rec["block_psi_all"] = bpa
    rec["corners"] = np.array([[c["top_left"][0], c["top_left"][1], c["bottom_left"][0], c["bottom_left"][1],
                                c["top_right"][0], c["top_right"][1], c["bottom_right"][0], c["bottom_right"][1]]
                               for c in corner_list], dtype=np.int64).reshape(-1, 8)
    if lists is not None:
        rec["circle_masks"] = np.stack(list(lists[0]) + list(lists[1]) + list(lists[2]))
    if seed is not None:
        rec["rho0_full"] = np.full((H, W), np.nan)
        rec["rho0_full"][mask] = cm.rho
    if not finals_only:
        rec.update(snapshot(cm, H, W, "s0"))
    for i in range(steps):
        for j in range(9):
            cm.F[j] = cm.getLarge_F(j)
            cm.feq[j] = cm.getfeq(j)
            cm.geq[j] = cm.getgeq(j)
            cm.f[j][mask] = cm.getF(j)
            cm.g[j][mask] = cm.getG(j)
        if i in phases_at:
            rec[f"p{i}_collided_f"] = cm.f.copy(); rec[f"p{i}_collided_g"] = cm.g.copy()
        f_behind = copy.deepcopy(cm.f)
        g_behind = copy.deepcopy(cm.g)
        mod.stream(cm.f, cm.g)
        if i in phases_at:
            rec[f"p{i}_streamed_f"] = cm.f.copy(); rec[f"p{i}_streamed_g"] = cm.g.copy()
        if lists is not None:
            bb.halfway_bounceback_circle(*lists, f_behind, g_behind, cm.f, cm.g)
        if corner_list:
            bb.halfway_bounceback_rec(corner_list, f_behind, g_behind, cm.f, cm.g)
        if variant == "walls":
            mod.bottom_top_wall(f_behind[:, 1:-1], g_behind[:, 1:-1], cm.f[:, 1:-1], cm.g[:, 1:-1])
        if i in phases_at:
            rec[f"p{i}_bounced_f"] = cm.f.copy(); rec[f"p{i}_bounced_g"] = cm.g.copy()
        cm.zou_he_boundary_inlet()
        cm.zou_he_boundary_outlet()
        if i in phases_at:
            rec[f"p{i}_zouhe_f"] = cm.f.copy(); rec[f"p{i}_zouhe_g"] = cm.g.copy()
        cm.rho = cm.getRho()
        cm.udpatePsi()
        cm.nabla_psix = cm.getNabla_psix()
        cm.nabla_psiy = cm.getNabla_psiy()
        cm.nabla_psi2 = cm.getNabla_psi2()
        cm.mu = cm.getMu()
        cm.ux = cm.getUx()
        cm.uy = cm.getUy()
        cm.p = cm.getP()
        cm.mix_tau = cm.getMix_tau()
        if (i + 1) in snap_steps:
            s = snapshot(cm, H, W, f"s{i + 1}")
            if finals_only:
                s = {k: v for k, v in s.items() if not (k.endswith("_f") or k.endswith("_g"))}
                import hashlib
                rec[f"s{i + 1}_f_sha256"] = np.array(hashlib.sha256(cm.f.tobytes()).hexdigest())
                rec[f"s{i + 1}_g_sha256"] = np.array(hashlib.sha256(cm.g.tobytes()).hexdigest())
            rec.update(s)
    rec.update(params_record(prm))
    rec["steps"] = np.array(steps)
    rec["snap_steps"] = np.array(sorted(snap_steps))
    rec["phases_at"] = np.array(sorted(phases_at))
    rec["rects"] = np.array([[p0[0], p0[1], p1[0], p1[1]] for p0, p1 in rects], dtype=np.int64).reshape(-1, 4)
    rec["circles"] = np.array([[c[0][0], c[0][1], c[1]] for c in circles], dtype=np.int64).reshape(-1, 3)
    return rec


def geometry_case(cbm, bbm):
    """Reference Createblock masks for a spread of radii and an overlapping pair."""
    H, W = 96, 160
    circles = [((12, 12), 3), ((30, 14), 4), ((52, 15), 5), ((80, 17), 7), ((115, 20), 9),
               ((20, 60), 10), ((60, 62), 12), ((110, 66), 14), ((140, 40), 6), ((146, 80), 2),
               ((28, 86), 4), ((33, 88), 4)]
    rects = [((5, 30), (9, 40)), ((20, 40), (30, 44)), ((150, 5), (152, 20)), ((70, 85), (90, 93)),
             ((75, 80), (80, 88))]
    cr = cbm.Createblock(H, W)
    bpa_c, side, conc, vex = cr.setCirleblock(circles)
    bpa_r, corner_list = cr.setblock(rects)
    return {
        "H": np.array(H), "W": np.array(W),
        "circles": np.array([[c[0][0], c[0][1], c[1]] for c in circles]),
        "rects": np.array([[p0[0], p0[1], p1[0], p1[1]] for p0, p1 in rects]),
        "bpa_circles": bpa_c, "bpa_rects": bpa_r,
        "circle_masks": np.stack(list(side) + list(conc) + list(vex)),
        "corners": np.array([[c["top_left"][0], c["top_left"][1], c["bottom_left"][0], c["bottom_left"][1],
                              c["top_right"][0], c["top_right"][1], c["bottom_right"][0], c["bottom_right"][1]]
                             for c in corner_list]),
    }


def main(ref_root):
    np.seterr(all="raise")
    fp, fw, bbm, cbm = import_reference(ref_root)
    out = {}
    # periodic variant (fingering_periodic.py), circle blocks, reference constants
    prm = periodic_reference_params().with_size(24, 48)
    out["periodic_circles_24x48"] = run_case(
        fp, fw, bbm, cbm, "periodic", prm, [], [((16, 8), 3), ((30, 15), 4), ((40, 6), 2)],
        steps=40, snap_steps={1, 2, 40}, phases_at={0, 1, 39})
    # walled variant (fingering.py), rectangle blocks, seeded random initial density
    prm = walls_reference_params().with_size(24, 48)  # constants as the script defines them (gamma from H=380)
    out["walls_rects_24x48"] = run_case(
        fp, fw, bbm, cbm, "walls", prm, [((12, 5), (16, 9)), ((26, 13), (31, 17)), ((38, 4), (41, 19))], [],
        steps=40, snap_steps={1, 2, 40}, phases_at={0, 1, 39}, seed=1234)
    # 500-step runs (fields only; f/g as SHA-256 digests)
    prm = periodic_reference_params().with_size(64, 128)
    circ = [((20 + 24 * k, 12 + 20 * (k % 2)), 5 + (k % 3)) for k in range(5)]
    out["periodic_circles_64x128_500"] = run_case(
        fp, fw, bbm, cbm, "periodic", prm, [], circ, steps=500, snap_steps={500}, phases_at=set(),
        finals_only=True)
    prm = walls_reference_params().with_size(64, 128)
    rects = [((16 + 22 * k, 10 + 14 * (k % 3)), (24 + 22 * k, 20 + 14 * (k % 3))) for k in range(5)]
    out["walls_rects_64x128_500"] = run_case(
        fp, fw, bbm, cbm, "walls", prm, rects, [], steps=500, snap_steps={500}, phases_at=set(), seed=99,
        finals_only=True)
    for name, rec in out.items():
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
        print("wrote", name)
    np.savez_compressed(os.path.join(HERE, "geometry_masks.npz"), **geometry_case(cbm, bbm))
    print("wrote geometry_masks")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
