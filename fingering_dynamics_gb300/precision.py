"""Error of reduced-precision storage against the FP64 path, per configuration.

The FP64 fused kernel reproduces the reference's numpy loop bit for bit
(same operation order, no contraction), so an FP64 lattice on the GPU stands
in for the FP64 oracle over runs far longer than the numpy code could do.
Each candidate lattice (FP32, FP16 or BF16 storage) starts from the same
state and advances in lock step with it; every ``every`` iterations both
leave the fused state and are compared:

* ``max_dpsi``: max |psi - psi_64| over fluid cells (the phase-field error);
* ``mass_drift``: |m - m_64| / m_64 for the invading (r) and defending (b)
  colour masses at the same iteration, from the FP64 diagnostics reduction;
* ``sat_err`` / ``tip_err``: absolute saturation and finger-tip differences;
* ``breakthrough``: first compared iteration at which invading fluid
  (psi > 0) reaches the last five columns (``None`` if not within the run).

Pointwise differences stay at storage rounding level until the viscous
fingering instability amplifies them; afterwards fingers move and only the
integral curves (saturation, tip) remain comparable.  ``window`` marks the
early iterations over which the pointwise bound is stated.
"""
from __future__ import annotations

import numpy as np


def _fluid_max_abs(a, b, fluid):
    d = (a - b).abs()
    d = d[fluid]
    return float(d.max().item()) if d.numel() else 0.0


def _make(params, geometry, spec, device):
    from .lattice import Lattice
    d, _, rounding = spec.partition("/")
    return Lattice(params, geometry, dtype=d, device=device, rounding=rounding or "stochastic")


def precision_study(params, geometry, dtypes=("f32", "f16", "bf16"), steps: int = 20000, every: int = 500,
                    window: int = 500, device="cuda"):
    """Run the FP64 lattice and one lattice per storage spec for ``steps``
    iterations; a spec is a dtype ("f32", "f16", "bf16"), optionally with the
    store rounding ("f16/nearest"; FP16/BF16 default to stochastic rounding).
    Returns {"checkpoints": [...], "per_dtype": {spec: summary}}."""
    import torch

    from .lattice import Lattice

    ref = Lattice(params, geometry, dtype="f64", device=device)
    cands = {d: _make(params, geometry, d, device) for d in dtypes}
    fluid = ref.fluid
    curves = {d: {"iteration": [], "max_dpsi": [], "mass_drift_r": [], "mass_drift_b": [], "sat_err": [],
                  "tip_err": [], "saturation": [], "tip_x": []} for d in dtypes}
    ref_curve = {"iteration": [], "saturation": [], "tip_x": [], "mass_r": [], "mass_b": []}
    bt = {d: None for d in ("f64",) + tuple(dtypes)}
    done = 0
    while done < steps:
        n = min(every, steps - done)
        if done < window:
            n = min(n, window - done)  # always compare at the end of the window
        ref.step(n)
        for lat in cands.values():
            lat.step(n)
        done += n
        dr = ref.diagnostics()
        ref_curve["iteration"].append(done)
        for k in ("saturation", "tip_x", "mass_r", "mass_b"):
            ref_curve[k].append(dr[k])
        if bt["f64"] is None and dr["breakthrough"]:
            bt["f64"] = done
        for d, lat in cands.items():
            dc = lat.diagnostics()
            c = curves[d]
            c["iteration"].append(done)
            c["max_dpsi"].append(_fluid_max_abs(lat.psi.double(), ref.psi, fluid))
            c["mass_drift_r"].append(abs(dc["mass_r"] - dr["mass_r"]) / dr["mass_r"])
            c["mass_drift_b"].append(abs(dc["mass_b"] - dr["mass_b"]) / dr["mass_b"])
            c["sat_err"].append(abs(dc["saturation"] - dr["saturation"]))
            c["tip_err"].append(abs(dc["tip_x"] - dr["tip_x"]))
            c["saturation"].append(dc["saturation"])
            c["tip_x"].append(dc["tip_x"])
            if bt[d] is None and dc["breakthrough"]:
                bt[d] = done
    torch.cuda.synchronize()
    per = {}
    for d, c in curves.items():
        it = np.array(c["iteration"])
        early = it <= window
        sat_ref = np.array(ref_curve["saturation"])
        rel_sat = np.abs(np.array(c["saturation"]) - sat_ref) / np.maximum(sat_ref, 1e-12)
        per[d] = {
            "max_dpsi_window": float(np.max(np.array(c["max_dpsi"])[early])) if early.any() else None,
            "max_dpsi_run": float(np.max(c["max_dpsi"])),
            "finite": bool(np.all(np.isfinite(c["max_dpsi"]))),
            "mass_drift_r_max": float(np.max(c["mass_drift_r"])),
            "mass_drift_b_max": float(np.max(c["mass_drift_b"])),
            "sat_err_max": float(np.max(c["sat_err"])),
            "sat_rel_err_max": float(np.max(rel_sat)),
            "tip_err_max": int(np.max(c["tip_err"])),
            "breakthrough": bt[d],
            "breakthrough_err": (None if bt[d] is None or bt["f64"] is None else abs(bt[d] - bt["f64"])),
            "curve": {k: v for k, v in c.items()},
        }
    return {"checkpoints": ref_curve, "breakthrough_f64": bt["f64"], "per_dtype": per, "steps": steps,
            "every": every, "window": window}
