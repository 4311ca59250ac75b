"""ctypes bindings for the CPU oracle (oracle/_build/liboracle.so).

Test infrastructure only: the oracle is the checker, never the product.
"""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
LIB_PATH = os.path.join(ORACLE_DIR, "_build", "liboracle.so")


class OracleCfg(ctypes.Structure):
    _fields_ = [
        ("D", ctypes.c_int), ("P", ctypes.c_int),
        ("gamma", ctypes.c_double), ("c_dt", ctypes.c_double),
        ("n_cell", ctypes.c_int * 3),
        ("prob_lo", ctypes.c_double * 3), ("prob_hi", ctypes.c_double * 3),
        ("periodic", ctypes.c_int * 3),
        ("ic", ctypes.c_int),
        ("u_inf", ctypes.c_double), ("v_inf", ctypes.c_double),
        ("beta", ctypes.c_double), ("xc", ctypes.c_double), ("yc", ctypes.c_double),
        ("seed", ctypes.c_uint64), ("noise_amp", ctypes.c_double),
        ("max_grid", ctypes.c_int),
        ("max_level", ctypes.c_int), ("blocking_factor", ctypes.c_int),
        ("dtn_regrid", ctypes.c_int), ("tag_kind", ctypes.c_int),
        ("tag_threshold", ctypes.c_double), ("grid_eff", ctypes.c_double),
        ("n_error_buf", ctypes.c_int), ("reflux_box_quirk", ctypes.c_int),
        ("t_limit", ctypes.c_int), ("tvb_M", ctypes.c_double), ("tvb_c", ctypes.c_double * 8),
        ("dt_regrid", ctypes.c_double), ("amr_c", ctypes.c_double * 8),
        ("tag_advect", ctypes.c_int), ("validation_mode", ctypes.c_int), ("no_reflux", ctypes.c_int),
    ]


IC = {"vortex": 0, "kh_noise": 1, "kh_ref": 2, "blast3d": 3, "const": 4}

_lib = None


def build():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        vp, dp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
        L.oracle_create.restype = vp
        L.oracle_create.argtypes = [ctypes.POINTER(OracleCfg)]
        L.oracle_destroy.argtypes = [vp]
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        L.oracle_set_threads.restype = ctypes.c_int
        for f in ("oracle_init", "oracle_get_dt", "oracle_step", "oracle_get_time"):
            getattr(L, f).restype = ctypes.c_double
            getattr(L, f).argtypes = [vp]
        L.oracle_set_dt.argtypes = [vp, ctypes.c_double]
        L.oracle_ader.argtypes = [vp]
        L.oracle_limit.argtypes = [vp]
        L.oracle_limit.restype = ctypes.c_long
        L.oracle_fill_patch.argtypes = [vp]
        L.oracle_predictor.argtypes = [vp, ctypes.c_int]
        L.oracle_num_levels.argtypes = [vp]
        L.oracle_num_levels.restype = ctypes.c_int
        L.oracle_limited_count.argtypes = [vp]
        L.oracle_limited_count.restype = ctypes.c_long
        L.oracle_layout_changes.argtypes = [vp]
        L.oracle_layout_changes.restype = ctypes.c_int
        L.oracle_get_boxes.argtypes = [vp, ctypes.c_int, ip, ctypes.c_int]
        L.oracle_get_boxes.restype = ctypes.c_int
        for f in ("oracle_get_uw", "oracle_set_uw", "oracle_get_uw_grown", "oracle_get_hw_grown"):
            getattr(L, f).argtypes = [vp, ctypes.c_int, dp]
            getattr(L, f).restype = ctypes.c_long
        L.oracle_tags.argtypes = [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int8)]
        L.oracle_tags.restype = ctypes.c_long
        L.oracle_norm.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int]
        L.oracle_norm.restype = ctypes.c_double
        L.oracle_norm_diff.argtypes = [vp, ctypes.POINTER(dp), ctypes.c_int, ctypes.c_int]
        L.oracle_norm_diff.restype = ctypes.c_double
        L.oracle_matrix.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.c_int, dp,
                                    ctypes.c_int, ip, ip]
        L.oracle_matrix.restype = ctypes.c_int
        L.oracle_gl_nodes.argtypes = [ctypes.c_int, dp, dp]
        L.oracle_gl_nodes.restype = ctypes.c_int
        _lib = L
    return _lib


def make_cfg(D=2, P=1, n=(32, 32, 1), lo=(0.0, 0.0, 0.0), hi=(10.0, 10.0, 1.0), periodic=(1, 1, 1),
             ic="vortex", u_inf=1.0, v_inf=0.0, c_dt=0.5, gamma=1.4, seed=12345, noise_amp=1e-3,
             max_grid=1024, max_level=0, blocking_factor=8, dtn_regrid=4, tag_kind=0,
             tag_threshold=0.1, grid_eff=0.7, n_error_buf=1, reflux_box_quirk=1, xc=5.0, yc=5.0, beta=5.0,
             t_limit=0, tvb_M=0.0, tvb_c=None, dt_regrid=0.0, amr_c=None, tag_advect=0,
             validation_mode=0, no_reflux=0):
    c = OracleCfg()
    c.D, c.P, c.gamma, c.c_dt = D, P, gamma, c_dt
    for d in range(3):
        c.n_cell[d] = n[d] if d < len(n) else 1
        c.prob_lo[d] = lo[d]
        c.prob_hi[d] = hi[d]
        c.periodic[d] = periodic[d]
    c.ic = IC[ic] if isinstance(ic, str) else ic
    c.u_inf, c.v_inf, c.beta, c.xc, c.yc = u_inf, v_inf, beta, xc, yc
    c.seed, c.noise_amp = seed, noise_amp
    c.max_grid, c.max_level, c.blocking_factor, c.dtn_regrid = max_grid, max_level, blocking_factor, dtn_regrid
    c.tag_kind, c.tag_threshold, c.grid_eff, c.n_error_buf = tag_kind, tag_threshold, grid_eff, n_error_buf
    c.reflux_box_quirk = reflux_box_quirk
    c.t_limit, c.tvb_M = t_limit, tvb_M
    for l in range(8):
        c.tvb_c[l] = 1.0 if tvb_c is None else tvb_c[l]
        c.amr_c[l] = 1.0 if amr_c is None or l >= len(amr_c) else amr_c[l]
    c.dt_regrid, c.tag_advect = dt_regrid, tag_advect
    c.validation_mode, c.no_reflux = validation_mode, no_reflux
    return c


class OracleSim:
    """One oracle simulation (the reference's evolve loop restated on the CPU)."""

    def __init__(self, cfg):
        self.cfg = cfg
        self.L = lib()
        self.h = self.L.oracle_create(ctypes.byref(cfg))
        if not self.h:
            raise RuntimeError("oracle_create failed")
        self.Q = cfg.D + 2
        from math import comb
        self.Np_s = comb(cfg.P + cfg.D, cfg.D)
        self.Np_st = comb(cfg.P + cfg.D + 1, cfg.D + 1)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.oracle_destroy(self.h)
            self.h = None

    def init(self):
        return self.L.oracle_init(self.h)

    @property
    def dt(self):
        return self.L.oracle_get_dt(self.h)

    @dt.setter
    def dt(self, v):
        self.L.oracle_set_dt(self.h, float(v))

    @property
    def time(self):
        return self.L.oracle_get_time(self.h)

    def step(self):
        return self.L.oracle_step(self.h)

    def ader(self):
        self.L.oracle_ader(self.h)

    def limit(self):
        """TVB limiter of the finest level; returns the cells modified."""
        return int(self.L.oracle_limit(self.h))

    def fill_patch(self):
        """Ghost cells of every level from the valid data."""
        self.L.oracle_fill_patch(self.h)

    def num_levels(self):
        return self.L.oracle_num_levels(self.h)

    def boxes(self, lev):
        buf = (ctypes.c_int * (6 * 100000))()
        n = self.L.oracle_get_boxes(self.h, lev, buf, 100000)
        a = np.frombuffer(buf, dtype=np.int32, count=6 * n).reshape(n, 6)
        return a.copy()

    def ncells_level(self, lev):
        b = self.boxes(lev)
        ext = b[:, 3:] - b[:, :3] + 1
        return int(np.prod(ext, axis=1).sum())

    def get_uw(self, lev=0):
        n = self.ncells_level(lev)
        out = np.zeros((n, self.Q, self.Np_s))
        w = self.L.oracle_get_uw(self.h, lev, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        assert w == n
        return out

    def set_uw(self, arr, lev=0):
        arr = np.ascontiguousarray(arr, dtype=np.float64)
        self.L.oracle_set_uw(self.h, lev, arr.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))

    def limited_count(self):
        """Cells the TVB limiter has modified so far."""
        return int(self.L.oracle_limited_count(self.h))

    def layout_changes(self):
        """Regrids that changed the layout, plus the first one."""
        return int(self.L.oracle_layout_changes(self.h))

    def tags(self, lev):
        n = self.ncells_level(lev)
        out = np.zeros(n, dtype=np.int8)
        w = self.L.oracle_tags(self.h, lev, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int8)))
        assert w == n
        return out

    def norm_diff(self, levels, p=2, q=0):
        """Lp norm of component q of (levels - this solution) over the leaf
        cells; levels[l] holds level l's valid cells in canonical order on
        this solution's layout."""
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in levels]
        assert len(arrs) == self.num_levels()
        for l, a in enumerate(arrs):
            assert a.size == self.ncells_level(l) * self.Q * self.Np_s
        ptrs = (ctypes.POINTER(ctypes.c_double) * len(arrs))(
            *[a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) for a in arrs])
        return self.L.oracle_norm_diff(self.h, ptrs, p, q)

    def norm(self, p=2, q=0, other=None):
        return self.L.oracle_norm(self.h, other.h if other is not None else None, p, q)


def set_threads(n):
    return lib().oracle_set_threads(n)


def matrix(D, P, name, idx=0):
    buf = np.zeros(200000)
    r, c = ctypes.c_int(), ctypes.c_int()
    rc = lib().oracle_matrix(D, P, name.encode(), idx, buf.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                             buf.size, ctypes.byref(r), ctypes.byref(c))
    if rc != 0:
        raise KeyError(name)
    return buf[: r.value * c.value].reshape(r.value, c.value).copy()
