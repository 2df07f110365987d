"""Helpers shared by the tests: load golden fixtures and build the matching
oracle / package inputs."""
from __future__ import annotations

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    with np.load(os.path.join(GOLDEN, f"{name}.npz"), allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def corner_dicts(corners):
    return [{"top_left": (int(c[0]), int(c[1])), "bottom_left": (int(c[2]), int(c[3])),
             "top_right": (int(c[4]), int(c[5])), "bottom_right": (int(c[6]), int(c[7]))}
            for c in np.asarray(corners).reshape(-1, 8)]


def circle_lists(stack):
    s = [np.asarray(m, bool) for m in stack]
    return s[0:4], s[4:8], s[8:12]


def lbm_params(fx):
    """LBMParams of a fixture (the package's parameter object)."""
    from fingering_dynamics_gb300.params import LBMParams
    variant = str(fx["variant"])
    return LBMParams(
        H=int(fx["H"]), W=int(fx["W"]), variant=variant, tau=float(fx["tau"]), eta_n=float(fx["eta_n"]),
        M=float(fx["M"]), a=float(fx["a"]), kappa=float(fx["kappa"]), gamma=float(fx["gamma"]),
        psi_wall=float(fx["psi_wall"]), u0=float(fx["u0"]), outlet_coef=float(fx["outlet_coef"]),
        inlet="plug" if variant == "walls" else "gaussian", slab=int(fx["slab"]),
        init_mu=variant == "walls", init_uy=variant == "walls", inlet_ux=fx["inlet_ux"])


def oracle_params(fx):
    from oracle.lbm_oracle import OracleParams
    return OracleParams(H=int(fx["H"]), W=int(fx["W"]), variant=str(fx["variant"]), tau=float(fx["tau"]),
                        eta_n=float(fx["eta_n"]), M=float(fx["M"]), a=float(fx["a"]),
                        kappa=float(fx["kappa"]), gamma=float(fx["gamma"]), psi_wall=float(fx["psi_wall"]),
                        inlet_ux=np.asarray(fx["inlet_ux"], np.float64),
                        outlet_coef=float(fx["outlet_coef"]))


def fixture_geometry(fx):
    """(solid, rho0 or None, bb_rect corner list, bb_circle lists) of a fixture."""
    solid = np.asarray(fx["block_psi_all"]) == 1
    rho0 = None
    if "rho0_full" in fx:
        rho0 = np.where(solid, 1.0, fx["rho0_full"])
    corners = corner_dicts(fx["corners"]) if fx["corners"].size else None
    circ = circle_lists(fx["circle_masks"]) if "circle_masks" in fx else None
    return solid, rho0, corners, circ


def oracle_from_fixture(fx):
    from oracle.lbm_oracle import OracleState
    prm = oracle_params(fx)
    solid, rho0, corners, circ = fixture_geometry(fx)
    psi0 = np.full((prm.H, prm.W), -1.0)
    psi0[:, :int(fx["slab"])] = 1.0
    walls = prm.variant == "walls"
    st = OracleState(prm, solid, psi0, rho0=rho0, init_mu=walls, init_uy=walls)
    return st, corners, circ


FIELDS = ("psi", "rho", "ux", "uy", "p", "mu", "mix_tau", "npx", "npy", "np2")


def oracle_fields(st):
    out = {"f": st.f, "g": st.g, "psi": st.psi, "npx": st.npx, "npy": st.npy, "np2": st.np2}
    for n in ("rho", "ux", "uy", "p", "mu", "mix_tau"):
        out[n] = st.full(n)
    return out


def packed_planes(buf, H, W, dtype):
    """The 18 planes of a packed state buffer (a uint8 tensor) without the
    padding that rounds each plane up to 256 bytes, which nothing writes."""
    import torch
    es = 4 if dtype == "f32" else 2
    P = H * W
    bf, bg = (P * es + 255) // 256 * 256, (P * 4 + 255) // 256 * 256
    parts = [buf[i * bf:i * bf + P * es] for i in range(9)]
    parts.append(buf[9 * bf:9 * bf + P * 4])
    parts += [buf[9 * bf + bg + i * bf:9 * bf + bg + i * bf + P * es] for i in range(8)]
    return torch.cat([p.cpu() for p in parts])
