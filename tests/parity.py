"""Shared helpers of the parity tests: run matching oracle and GPU cases."""
import numpy as np

import oracle_ffi as O

try:
    import adg_gb300 as G
except Exception:  # the CUDA library may be unbuilt on a CPU-only machine
    G = None

CASES = {
    # name: (D, P, n_cell, prob_lo, prob_hi, periodic, ic, extra)
    "vortex_p1": (2, 1, (32, 32, 1), (0, 0, 0), (10, 10, 1), (1, 1, 1), "vortex", dict(u_inf=1.0, v_inf=1.0)),
    "vortex_p2": (2, 2, (16, 16, 1), (0, 0, 0), (10, 10, 1), (1, 1, 1), "vortex", dict(u_inf=1.0, v_inf=0.0)),
    "kh_p3": (2, 3, (32, 32, 1), (0, 0, 0), (1, 1, 1), (1, 1, 1), "kh_noise", dict(seed=12345, noise_amp=1e-3)),
    "kh_p3_rect": (2, 3, (24, 16, 1), (0, 0, 0), (1.5, 1, 1), (1, 1, 1), "kh_noise", dict(seed=7, noise_amp=1e-3)),
    "vortex_p3_outflow": (2, 3, (16, 12, 1), (0, 0, 0), (10, 7.5, 1), (0, 0, 1), "vortex", dict(u_inf=0.3, v_inf=0.2)),
    "blast3d_p2": (3, 2, (8, 8, 8), (0, 0, 0), (1, 1, 1), (0, 0, 0), "blast3d", dict()),
    "blast3d_p1_per": (3, 1, (8, 6, 4), (0, 0, 0), (1, 0.75, 0.5), (1, 1, 1), "blast3d", dict()),
}

ORACLE_IC = {"vortex": "vortex", "kh_noise": "kh_noise", "blast3d": "blast3d", "const": "const"}
GPU_IC = {"vortex": "isentropic_vortex", "kh_noise": "kh_noise", "blast3d": "blast3d", "const": "const"}


def make_oracle(case, c_dt=0.5, max_grid=1024):
    D, P, n, lo, hi, per, ic, extra = CASES[case]
    cfg = O.make_cfg(D=D, P=P, n=n, lo=lo, hi=hi, periodic=per, ic=ORACLE_IC[ic], c_dt=c_dt,
                     max_grid=max_grid, **extra)
    s = O.OracleSim(cfg)
    s.init()
    return s


def make_gpu(case, c_dt=0.5, **kw):
    D, P, n, lo, hi, per, ic, extra = CASES[case]
    m = G.Compressible_Euler().settings(GPU_IC[ic], **extra)
    s = G.AmrDG(P=P, D=D)
    s.setGeometrySettings(prob_lo=lo, prob_hi=hi, n_cell=n, periodic=per)
    s.settings(c_dt=c_dt, **kw)
    s.init(m)
    return s


def rel_err(a, b):
    """max |a - b| over cells and modes of each variable, relative to the
    variable's largest cell mean, maximised over variables."""
    a = np.asarray(a)
    b = np.asarray(b)
    worst = 0.0
    for q in range(a.shape[1]):
        scale = max(np.max(np.abs(b[:, q, 0])), 1e-300)
        worst = max(worst, float(np.max(np.abs(a[:, q, :] - b[:, q, :])) / scale))
    return worst
