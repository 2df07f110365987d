"""The reference's own loop body (fingering_periodic.py:454-479,
fingering.py:558-585) run against the drop-in modules on the GPU in FP64
must reproduce the reference's outputs bit for bit."""
import copy

import numpy as np
import pytest

from fixtures import FIELDS, corner_dicts, circle_lists, load

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _run_reference_loop(mod, bbm, fx, steps):
    """The loop body exactly as the reference's main() writes it."""
    H, W = int(fx["H"]), int(fx["W"])
    mod.H, mod.W = H, W
    for k, n in (("tau", "tau"), ("Eta_n", "eta_n"), ("M", "M"), ("a", "a"), ("kappa", "kappa"),
                 ("gamma", "gamma"), ("psi_wall", "psi_wall"), ("u0", "u0")):
        setattr(mod, k, float(fx[n]))
    bpa = np.asarray(fx["block_psi_all"])
    block_mask = np.where(bpa == 1, True, False)
    mask = np.logical_not(block_mask)
    if "rho0_full" in fx:
        np.random.seed(99 if H == 64 else 1234)
    cm = mod.Compute(mask)
    bb = bbm.Bounce_back(H, W)
    corner_list = corner_dicts(fx["corners"]) if fx["corners"].size else []
    lists = circle_lists(fx["circle_masks"]) if "circle_masks" in fx else None
    for i in range(steps):
        for j in range(9):
            cm.F[j] = cm.getLarge_F(j)
            cm.feq[j] = cm.getfeq(j)
            cm.geq[j] = cm.getgeq(j)
            cm.f[j][mask] = cm.getF(j)
            cm.g[j][mask] = cm.getG(j)
        f_behind = copy.deepcopy(cm.f)
        g_behind = copy.deepcopy(cm.g)
        mod.stream(cm.f, cm.g)
        if lists is not None:
            bb.halfway_bounceback_circle(*lists, f_behind, g_behind, cm.f, cm.g)
        if corner_list:
            bb.halfway_bounceback_rec(corner_list, f_behind, g_behind, cm.f, cm.g)
        if str(fx["variant"]) == "walls":
            mod.bottom_top_wall(f_behind[:, 1:-1], g_behind[:, 1:-1], cm.f[:, 1:-1], cm.g[:, 1:-1])
        cm.zou_he_boundary_inlet()
        cm.zou_he_boundary_outlet()
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
    return cm, mask


@pytest.mark.parametrize("name", ["periodic_circles_24x48", "walls_rects_24x48"])
def test_reference_loop_on_dropin_is_bitwise(name):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fingering_dynamics_gb300 import build
    build.build()
    from fingering_dynamics_gb300 import bounce_back, fingering, fingering_periodic
    fx = load(name)
    mod = fingering if str(fx["variant"]) == "walls" else fingering_periodic
    cm, mask = _run_reference_loop(mod, bounce_back, fx, 40)
    assert np.array_equal(cm.f.cpu().numpy(), fx["s40_f"])
    assert np.array_equal(cm.g.cpu().numpy(), fx["s40_g"])
    assert np.array_equal(cm.psi.cpu().numpy(), fx["s40_psi"])
    for k in ("rho", "ux", "uy", "p", "mu", "mix_tau"):
        assert np.array_equal(getattr(cm, k).cpu().numpy(), fx[f"s40_{k}"][mask]), k


def test_reference_binding_stub_equals_the_fused_step():
    """The ctypes binding offered to the reference's maintainers
    (fingering_dynamics_gb300/binding/reference_gb300.py) run from a walled
    module's globals gives, bit for bit, the package's own FP64 fused state."""
    import types

    from fingering_dynamics_gb300 import build
    from fingering_dynamics_gb300 import geometry as geo
    from fingering_dynamics_gb300.binding import reference_gb300 as rb
    from fingering_dynamics_gb300.lattice import Lattice
    from fingering_dynamics_gb300.params import walls_reference_params
    lib = rb.load(build.build())
    H, W, n = 32, 64, 7
    prm = walls_reference_params().with_size(H, W)
    g = geo.build_geometry(H, W, rects=[((20, 10), (26, 16))], walls=True)
    mod = types.SimpleNamespace(__name__="fingering", H=H, W=W, tau=prm.tau, Eta_n=prm.eta_n, M=prm.M, a=prm.a,
                                kappa=prm.kappa, gamma=prm.gamma, psi_wall=prm.psi_wall, u0=float(prm.inlet_ux[0]))
    assert np.all(prm.inlet_ux == mod.u0)
    got = rb.run(lib, mod, g.mask_word, prm.initial_psi(g.solid), n)
    lat = Lattice(prm, g, dtype="f64")
    lat.enter_fused()
    lat.advance(n)
    torch.cuda.synchronize()
    assert torch.equal(got, lat.pop[lat.cur])
