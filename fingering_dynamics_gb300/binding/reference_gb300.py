"""The ctypes binding a maintainer of the reference would add to its scripts
(as ``lattice_boltzmann/gb300.py``) to drive the loop body of
``fingering_periodic.py:454-479`` / ``fingering.py:558-585`` on a GB300
through ``libfdlbm.so``.  It uses only ctypes, numpy and torch (for device
buffers); the structures mirror ``include/fdlbm.h``.
"""
import ctypes as C

import numpy as np


class fd_params(C.Structure):
    """The reference's module globals in one struct (include/fdlbm.h fd_params)."""
    _fields_ = [("H", C.c_int32), ("W", C.c_int32), ("variant", C.c_int32), ("flags", C.c_uint32),
                ("tau", C.c_double), ("eta_n", C.c_double), ("M", C.c_double), ("a", C.c_double),
                ("kappa", C.c_double), ("gamma", C.c_double), ("psi_wall", C.c_double),
                ("outlet_coef", C.c_double), ("force_x", C.c_double), ("force_y", C.c_double)]


class fd_storage(C.Structure):
    """Packed storage of the populations (include/fdlbm.h fd_storage)."""
    _fields_ = [("dtype", C.c_int32), ("f_scale_log2", C.c_int32), ("g_scale_log2", C.c_int32),
                ("rounding", C.c_int32), ("seed", C.c_uint32)]


def load(path):
    """Open libfdlbm.so at `path` and declare the return types the stub uses."""
    lib = C.CDLL(path)
    lib.fd_packed_bytes.restype = C.c_size_t
    return lib


def params_of(mod):
    """fd_params of a reference module (fingering_periodic or fingering) with its current globals."""
    walls = mod.__name__.endswith("fingering")
    return fd_params(mod.H, mod.W, int(walls), 3 if walls else 0, mod.tau, mod.Eta_n, mod.M, mod.a, mod.kappa,
                     mod.gamma, mod.psi_wall, 1.5 if walls else 2 / 3, 0.0, 0.0)


def run(lib, mod, mask_word, psi0, steps):
    """Run `steps` iterations of the loop body of module `mod` with its current
    globals in FP64 (bit for bit the reference's arithmetic); returns the
    (18, H, W) post-collision populations on the GPU."""
    import torch
    H, W = mod.H, mod.W
    prm = params_of(mod)
    dev = torch.device("cuda")
    mask = torch.from_numpy(np.ascontiguousarray(mask_word).view(np.int16)).to(dev)
    psi0_d = torch.from_numpy(np.ascontiguousarray(psi0, np.float64)).to(dev)
    pop = [torch.zeros((18, H, W), dtype=torch.float64, device=dev) for _ in range(2)]
    fields = [torch.zeros((H, W), dtype=torch.float64, device=dev) for _ in range(10)]
    side = [torch.zeros((6, H), dtype=torch.float64, device=dev) for _ in range(2)]
    ux = torch.full((H,), mod.u0, dtype=torch.float64, device=dev)  # or the Gaussian profile
    ptrs = (C.c_void_p * 12)(pop[0].data_ptr(), pop[0][9:].data_ptr(), *[t.data_ptr() for t in fields])
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.fd_compute_init(C.byref(prm), 0, C.c_void_p(mask.data_ptr()), C.c_void_p(psi0_d.data_ptr()),
                               None, ptrs, s) == 0
    # fd_boundary_fields(.. fields[0] = psi, fields[3] = np2 ..) into side[0], then fd_collide, enter the
    # fused state (post-collision populations in pop[0])
    assert lib.fd_boundary_fields(C.byref(prm), 0, C.c_void_p(mask.data_ptr()), C.c_void_p(fields[0].data_ptr()),
                                  C.c_void_p(fields[3].data_ptr()), C.c_void_p(side[0].data_ptr()), s) == 0
    assert lib.fd_collide(C.byref(prm), 0, C.c_void_p(mask.data_ptr()), ptrs, s) == 0
    assert lib.fd_fused_step(C.byref(prm), 0, C.c_void_p(mask.data_ptr()), C.c_void_p(ux.data_ptr()),
                             C.c_void_p(pop[0].data_ptr()), C.c_void_p(pop[1].data_ptr()),
                             C.c_void_p(side[0].data_ptr()), C.c_void_p(side[1].data_ptr()), steps, 0, s) == 0
    return pop[steps % 2]


def run_host_resident(lib, prm, mask, ux, host, side, steps, stream):
    """The state stays in a pinned host buffer `host` (packed FP32 layout,
    fd_packed_bytes bytes), as the reference's numpy arrays do: each call
    uploads it, advances one iteration and downloads it, with the two copy
    directions overlapping (fd_fused_step_packed_host).  `side`: two (6, H)
    float32 device tensors holding the boundary values; `mask`, `ux` device
    tensors."""
    import torch
    st = fd_storage(1, 0, 0, 0, 0)  # FD_F32 storage, first step's seed 0
    nbytes = lib.fd_packed_bytes(prm.H, prm.W, C.byref(st))
    pa, pb = (torch.empty(nbytes, dtype=torch.uint8, device=mask.device) for _ in range(2))
    for it in range(steps):  # one reference iteration per call
        assert lib.fd_fused_step_packed_host(C.byref(prm), C.byref(st), C.c_void_p(mask.data_ptr()),
                                             C.c_void_p(ux.data_ptr()), C.c_void_p(host.data_ptr()),
                                             C.c_void_p(host.data_ptr()), C.c_void_p(pa.data_ptr()),
                                             C.c_void_p(pb.data_ptr()), C.c_void_p(side[it % 2].data_ptr()),
                                             C.c_void_p(side[1 - it % 2].data_ptr()), 1, 0, stream) == 0
        st.seed += 1  # stochastic rounding: seed of the next step
