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
    # higher degrees (plain FP64 path)
    "vortex_p4": (2, 4, (16, 12, 1), (0, 0, 0), (10, 7.5, 1), (1, 1, 1), "vortex", dict(u_inf=1.0, v_inf=0.5)),
    "kh_p5_outflow": (2, 5, (12, 12, 1), (0, 0, 0), (1, 1, 1), (0, 1, 1), "kh_noise", dict(seed=5, noise_amp=1e-3)),
    "vortex_p6": (2, 6, (8, 8, 1), (0, 0, 0), (10, 10, 1), (1, 1, 1), "vortex", dict(u_inf=1.0, v_inf=0.0)),
    "blast3d_p3": (3, 3, (6, 6, 6), (0, 0, 0), (1, 1, 1), (0, 0, 0), "blast3d", dict()),
}
HIGH_DEGREE = ("vortex_p4", "kh_p5_outflow", "vortex_p6", "blast3d_p3")

ORACLE_IC = {"vortex": "vortex", "kh_noise": "kh_noise", "blast3d": "blast3d", "const": "const"}
GPU_IC = {"vortex": "isentropic_vortex", "kh_noise": "kh_noise", "blast3d": "blast3d", "const": "const"}


def make_oracle(case, c_dt=0.5, max_grid=1024, **kw):
    D, P, n, lo, hi, per, ic, extra = CASES[case]
    cfg = O.make_cfg(D=D, P=P, n=n, lo=lo, hi=hi, periodic=per, ic=ORACLE_IC[ic], c_dt=c_dt,
                     max_grid=max_grid, **extra, **kw)
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


AMR_CASES = {
    "kh_p4_amr": (2, 4, (16, 16, 1), (1, 1, 1), (1, 1, 1), "kh_noise", dict(seed=11, noise_amp=1e-3),
                  dict(max_level=1, max_grid=8, blocking_factor=4, dtn_regrid=2, tag_kind=0, tag_threshold=0.05)),
    # name: (D, P, n_cell, hi, periodic, ic, extra, amr)
    "kh_p3_amr": (2, 3, (16, 16, 1), (1, 1, 1), (1, 1, 1), "kh_noise", dict(seed=12345, noise_amp=1e-3),
                  dict(max_level=2, max_grid=16, blocking_factor=8, dtn_regrid=4, tag_kind=0, tag_threshold=0.1)),
    "kh_p2_amr_rect": (2, 2, (24, 16, 1), (1.5, 1, 1), (1, 1, 1), "kh_noise", dict(seed=3, noise_amp=1e-3),
                       dict(max_level=1, max_grid=8, blocking_factor=4, dtn_regrid=2, tag_kind=0, tag_threshold=0.05)),
    "blast3d_p2_amr": (3, 2, (8, 8, 8), (1, 1, 1), (0, 0, 0), "blast3d", dict(),
                       dict(max_level=1, max_grid=8, blocking_factor=4, dtn_regrid=2, tag_kind=1, tag_threshold=0.05)),
}


def make_oracle_amr(case, c_dt=0.5, quirk=1, **kw):
    D, P, n, hi, per, ic, extra, amr = AMR_CASES[case]
    cfg = O.make_cfg(D=D, P=P, n=n, hi=hi, periodic=per, ic=ORACLE_IC[ic], c_dt=c_dt, reflux_box_quirk=quirk,
                     **extra, **amr, **kw)
    s = O.OracleSim(cfg)
    s.init()
    return s


def make_gpu_amr(case, c_dt=0.5, quirk=1, **kw):
    D, P, n, hi, per, ic, extra, amr = AMR_CASES[case]
    m = G.Compressible_Euler().settings(GPU_IC[ic], **extra)
    s = G.AmrDG(P=P, D=D)
    s.setGeometrySettings(prob_lo=(0, 0, 0), prob_hi=hi, n_cell=n, periodic=per, max_level=amr["max_level"],
                          max_grid=amr["max_grid"], blocking_factor=amr["blocking_factor"],
                          dtn_regrid=amr["dtn_regrid"])
    s.setAmrSettings(tag_kind=amr["tag_kind"], tag_threshold=amr["tag_threshold"], reflux_box_quirk=quirk)
    s.settings(c_dt=c_dt, **kw)
    s.init(m)
    return s


def leaf_mass(levels_u, boxes, n_cell, hi, D):
    """Integral of density over leaf cells from per-level valid data."""
    tot = 0.0
    nl = len(levels_u)
    for l in range(nl):
        n = [n_cell[d] << l for d in range(D)]
        vol = 1.0
        for d in range(D):
            vol *= hi[d] / n[d]
        mask = np.zeros(n[::-1], bool)
        for bx in boxes[l]:
            sl = tuple(slice(bx[d], bx[3 + d] + 1) for d in range(D))[::-1]
            mask[sl] = True
        idx = np.argwhere(mask)  # (k, j, i) lexicographic = x fastest
        leaf = np.ones(len(idx), bool)
        if l + 1 < nl:
            fm = np.zeros(n[::-1], bool)
            for bx in boxes[l + 1]:
                sl = tuple(slice(bx[d] // 2, bx[3 + d] // 2 + 1) for d in range(D))[::-1]
                fm[sl] = True
            leaf = ~fm[tuple(idx.T)]
        tot += levels_u[l][leaf, 0, 0].sum() * vol
    return tot
