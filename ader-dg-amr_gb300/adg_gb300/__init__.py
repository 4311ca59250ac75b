"""GB300 (sm_103a) ADER-DG element path: Python host mirror of the reference's
Solver<AmrDG<P>> / ModelEquation<Compressible_Euler> surface over the C ABI of
libadg.so (include/adg.h).

Reference surface mirrored here:
  Simulation setters      Source/Core/Simulation.h:25-176
  AmrDG<P>::settings      Source/NumericalMethod/AmrDG/AmrDG.tpp:49-59
  Solver::init            Source/Core/Solver.h:502-597
  AmrDG::evolve / ADER    Source/NumericalMethod/AmrDG/AmrDG.h:853-1165
  AmrDG::set_Dt           Source/NumericalMethod/AmrDG/AmrDG.h:1253-1357
  Compressible_Euler::settings  Source/Model/CompressibleEuler/Compressible_Euler.cpp:5-48
  Solver::PlotFile / ReadPlotFile  Source/Core/Solver.h:599-652, 922-968

The compute path is the CUDA library only; there is no CPU fallback.  Loading
fails loudly when the library is missing.
"""
import ctypes
import os
from math import comb

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_lib", "libadg.so")

ADG_OK = 0
ADG_MEM_HOST = 0
ADG_MEM_DEVICE = 1
ADG_MEM_HOST_ASYNC = 2
ADG_ALL_LEVELS = -1
IC_CODES = {"isentropic_vortex": 0, "vortex": 0, "kh_noise": 1, "kelvin_helmolz_instability": 2,
            "kh_ref": 2, "blast3d": 3, "const": 4}


class AdgConfig(ctypes.Structure):
    _fields_ = [
        ("D", ctypes.c_int), ("P", ctypes.c_int),
        ("gamma", ctypes.c_double), ("c_dt", ctypes.c_double),
        ("n_cell", ctypes.c_int * 3),
        ("prob_lo", ctypes.c_double * 3), ("prob_hi", ctypes.c_double * 3),
        ("periodic", ctypes.c_int * 3),
        ("ic", ctypes.c_int),
        ("u_inf", ctypes.c_double), ("v_inf", ctypes.c_double), ("beta", ctypes.c_double),
        ("xc", ctypes.c_double), ("yc", ctypes.c_double),
        ("seed", ctypes.c_uint64), ("noise_amp", ctypes.c_double),
        ("max_grid", ctypes.c_int),
        ("max_level", ctypes.c_int), ("blocking_factor", ctypes.c_int), ("dtn_regrid", ctypes.c_int),
        ("tag_kind", ctypes.c_int), ("tag_threshold", ctypes.c_double), ("grid_eff", ctypes.c_double),
        ("n_error_buf", ctypes.c_int), ("reflux_box_quirk", ctypes.c_int),
        ("picard_sweeps", ctypes.c_int), ("elems_per_block", ctypes.c_int),
        ("limiter_t", ctypes.c_int), ("tvb_M", ctypes.c_double), ("tvb_c", ctypes.c_double * 8),
        ("dt_regrid", ctypes.c_double), ("amr_c", ctypes.c_double * 8), ("tag_advect", ctypes.c_int),
        ("validation_mode", ctypes.c_int), ("no_reflux", ctypes.c_int),
    ]


# Refinement criteria (ADG_TAG_* of include/adg.h): this library's two
# indicators and the reference's own pde_tag_cell_refinement variants
# (Compressible_Euler.h:606-685).
TAG_KINDS = {"density_gradient": 0, "pressure_jump": 1, "isentropic_vortex": 2, "vortex": 2,
             "kelvin_helmolz_instability": 3, "kh_tvb": 3}


class AdgPatch(ctypes.Structure):
    """adg_patch: one box of the caller's per-(level, q) arrays."""
    _fields_ = [
        ("level", ctypes.c_int), ("lo", ctypes.c_int * 3), ("hi", ctypes.c_int * 3), ("nghost", ctypes.c_int),
        ("U_w", ctypes.c_void_p * 5), ("jstride", ctypes.c_int64), ("kstride", ctypes.c_int64),
        ("nstride", ctypes.c_int64),
    ]


class AdgError(RuntimeError):
    pass


_lib = None


def lib():
    """Load libadg.so (built in-tree by adg_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise AdgError(f"CUDA library not built: {LIB_PATH} (run adg_gb300.build.build())")
    L = ctypes.CDLL(LIB_PATH)
    vp, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)
    i = ctypes.c_int
    sig = {
        "adg_ctx_create": ([ctypes.POINTER(AdgConfig), ctypes.POINTER(vp)], i),
        "adg_ctx_destroy": ([vp], i),
        "adg_last_error": ([vp], ctypes.c_char_p),
        "adg_set_stream": ([vp, vp], i),
        "adg_init": ([vp], i),
        "adg_num_levels": ([vp, ctypes.POINTER(i)], i),
        "adg_level_cells": ([vp, i, ctypes.POINTER(ctypes.c_int64)], i),
        "adg_get_state": ([vp, i, vp, i], i),
        "adg_set_state": ([vp, i, vp, i], i),
        "adg_set_readback": ([vp, i, vp, ctypes.c_int64], i),
        "adg_readback_active": ([vp, i, ctypes.POINTER(i)], i),
        "adg_get_dt": ([vp, dp], i),
        "adg_set_dt": ([vp, ctypes.c_double], i),
        "adg_compute_dt": ([vp, dp], i),
        "adg_get_time": ([vp, dp], i),
        "adg_ader": ([vp], i),
        "adg_step": ([vp], i),
        "adg_advance": ([vp, i, i], i),
        "adg_predictor": ([vp, i, vp], i),
        "adg_status": ([vp, ctypes.POINTER(ctypes.c_uint32)], i),
        "adg_launch_count": ([vp, ctypes.POINTER(ctypes.c_int64)], i),
        "adg_fp64_peak_probe": ([dp], i),
        "adg_set_device": ([i], i),
        "adg_advance_timed": ([vp, i, i, dp], i),
        "adg_advance_timed_flushed": ([vp, i, i, ctypes.c_int64, dp], i),
        "adg_time_kernels": ([vp, i, dp, i], i),
        "adg_host_alloc": ([ctypes.c_size_t, ctypes.POINTER(vp)], i),
        "adg_host_free": ([vp], i),
        "adg_flops_per_element": ([i, i, dp, dp], i),
        "adg_regrid_count": ([vp, ctypes.POINTER(i)], i),
        "adg_dof_updates": ([vp, ctypes.POINTER(ctypes.c_int64), dp], i),
        "adg_regrid_profile": ([vp, dp, i], i),
        "adg_leaf_dof_updates": ([vp, ctypes.POINTER(ctypes.c_int64)], i),
        "adg_limited_count": ([vp, ctypes.POINTER(ctypes.c_int64)], i),
        "adg_lp_norm": ([vp, i, i, dp], i),
        "adg_seed_set_path": ([vp, i], i),
        "adg_seed_infer": ([vp, vp, i], i),
        "adg_seed_create": ([i, i, i, ctypes.c_uint64, ctypes.POINTER(vp)], i),
        "adg_seed_destroy": ([vp], i),
        "adg_seed_collect": ([vp, vp, i], i),
        "adg_seed_num_samples": ([vp, ctypes.POINTER(ctypes.c_int64)], i),
        "adg_seed_train": ([vp, i, i, ctypes.c_double, dp], i),
        "adg_seed_forward": ([vp, vp, i, vp], i),
        "adg_seed_gradients": ([vp, vp, vp, i, vp, dp], i),
        "adg_seed_num_params": ([vp, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)], i),
        "adg_seed_get_params": ([vp, vp], i),
        "adg_seed_set_params": ([vp, vp], i),
        "adg_seed_attach": ([vp, vp, i, i, ctypes.c_double], i),
        "adg_seed_stats": ([vp, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)], i),
        "adg_get_boxes": ([vp, i, ctypes.POINTER(i), i, ctypes.POINTER(i)], i),
        "adg_set_layout": ([vp, i, ctypes.POINTER(i), ctypes.POINTER(i)], i),
        "adg_level_cell_coords": ([vp, i, ctypes.POINTER(i)], i),
        "adg_tags": ([vp, i, ctypes.POINTER(ctypes.c_uint8)], i),
        "adg_get_step": ([vp, ctypes.POINTER(ctypes.c_int64)], i),
        "adg_synchronize": ([vp], i),
        "adg_interp_scatter": ([vp, vp, vp, ctypes.c_int64, vp, i], i),
        "adg_interp_gather": ([vp, vp, ctypes.c_int64, vp, i], i),
        "adg_average_down": ([vp], i),
        "adg_fill_ghosts": ([vp], i),
        "adg_limit": ([vp, ctypes.POINTER(ctypes.c_int64)], i),
        "adg_autotune": ([vp, i, ctypes.POINTER(i), dp, i], i),
        "adg_block_choices": ([vp, ctypes.POINTER(i), i, ctypes.POINTER(i), ctypes.POINTER(i), ctypes.POINTER(i)], i),
        "adg_set_patches": ([vp, ctypes.POINTER(AdgPatch), i], i),
        "adg_read_patches": ([vp], i),
        "adg_write_patches": ([vp], i),
        "adg_write_plotfile": ([vp, ctypes.c_char_p, i, i, ctypes.POINTER(ctypes.c_char_p)], i),
        "adg_read_plotfile": ([vp, ctypes.c_char_p, i, dp], i),
        "adg_plotfile_info": ([ctypes.c_char_p, ctypes.POINTER(i), ctypes.POINTER(i), ctypes.POINTER(i), dp,
                               ctypes.POINTER(i), ctypes.c_char_p, i], i),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def exported_symbols():
    return [n for n in ("adg_ctx_create",) if hasattr(lib(), n)]


class Compressible_Euler:
    """ModelEquation<Compressible_Euler>: model case, gamma and Q
    (Compressible_Euler.cpp:5-48)."""

    def __init__(self):
        self.model_case = "isentropic_vortex"
        self.gamma_adiab = 1.4
        self.ic_params = {}

    def settings(self, euler_case, **ic_params):
        self.model_case = euler_case
        self.gamma_adiab = 5.0 / 3.0 if euler_case == "keplerian_disc" else 1.4
        self.ic_params = dict(ic_params)
        return self

    def Q_model(self, D):
        return D + 2


class AmrDG:
    """Solver<AmrDG<P>> on one GB300.

    Typical use (mirrors Simulation::run):
        model = Compressible_Euler().settings("kh_noise", seed=12345)
        s = AmrDG(P=3, D=2)
        s.setGeometrySettings(prob_lo=(0, 0), prob_hi=(1, 1), n_cell=(256, 256))
        s.settings(T=1.0, c_dt=0.5)
        s.init(model)
        s.evolve(nsteps=100)
    """

    def __init__(self, P, D=2):
        self.P, self.D = int(P), int(D)
        self.Q = self.D + 2
        self.Np_s = comb(self.P + self.D, self.D)
        self.Np_st = comb(self.P + self.D + 1, self.D + 1)
        self.cfg = AdgConfig()
        c = self.cfg
        c.D, c.P, c.gamma, c.c_dt = self.D, self.P, 1.4, 0.5
        for d in range(3):
            c.n_cell[d] = 1
            c.prob_lo[d], c.prob_hi[d] = 0.0, 1.0
            c.periodic[d] = 1
        c.u_inf, c.v_inf, c.beta, c.xc, c.yc = 1.0, 0.0, 5.0, 5.0, 5.0
        c.seed, c.noise_amp = 12345, 1e-3
        c.max_grid, c.max_level, c.blocking_factor, c.dtn_regrid = 32, 0, 8, 4
        c.tag_kind, c.tag_threshold, c.grid_eff, c.n_error_buf = 0, 0.1, 0.7, 1
        c.reflux_box_quirk, c.picard_sweeps, c.elems_per_block = 1, 0, 0
        self.T = None
        self.ctx = None
        self.dtn_outplt, self.dt_outplt, self.data_dir, self.restart_tstep = 0, 0.0, "plt", 0
        self.restart_time = 0.0
        self._t_last_plt = 0.0
        self._L = lib()

    # ------------------------------------------------------------ settings
    def settings(self, T=None, c_dt=0.5, picard_sweeps=0, elems_per_block=0, limiter_type="", TVB_M=0.0,
                 amr_tvb_c=None, t_limit=-1):
        """AmrDG<P>::settings / Simulation::setNumericalSettings(T, c_dt,
        limiter_type, TVB_M, AMR_TVB_C, t_limit) (AmrDG.tpp:49-59,
        Source/main.cpp:147); limiter_type "TVB" with t_limit > 0 limits the
        finest level every t_limit steps."""
        self.T = T
        self.cfg.c_dt = float(c_dt)
        self.cfg.picard_sweeps = int(picard_sweeps)
        self.cfg.elems_per_block = int(elems_per_block)
        if limiter_type not in ("", "TVB"):
            raise ValueError(f"unknown limiter {limiter_type!r}")
        self.cfg.limiter_t = int(t_limit) if (limiter_type == "TVB" and t_limit > 0) else 0
        self.cfg.tvb_M = float(TVB_M)
        for l in range(8):
            self.cfg.tvb_c[l] = 1.0 if amr_tvb_c is None or l >= len(amr_tvb_c) else float(amr_tvb_c[l])
        return self

    def setNumericalSettings(self, T=None, c_dt=0.5, limiter_type="", TVB_M=0.0, amr_tvb_c=None, t_limit=-1):
        """Simulation::setNumericalSettings (Source/main.cpp:147)."""
        return self.settings(T=T, c_dt=c_dt, picard_sweeps=self.cfg.picard_sweeps,
                             elems_per_block=self.cfg.elems_per_block, limiter_type=limiter_type, TVB_M=TVB_M,
                             amr_tvb_c=amr_tvb_c, t_limit=t_limit)

    def setGeometrySettings(self, prob_lo, prob_hi, n_cell, max_level=0, periodic=None, max_grid=32,
                            blocking_factor=8, dtn_regrid=4, amr_c=None, dt_regrid=0.0):
        """Simulation::setGeometrySettings (Simulation.h:120-140): amr_c is
        the per-level coefficient of the reference's tagging criteria,
        dtn_regrid / dt_regrid the step and time cadence of the regrid
        (<= 0: off)."""
        c = self.cfg
        for l in range(8):
            c.amr_c[l] = 1.0 if amr_c is None or l >= len(amr_c) else float(amr_c[l])
        c.dt_regrid = float(dt_regrid)
        for d in range(3):
            if d < self.D:
                c.prob_lo[d], c.prob_hi[d] = float(prob_lo[d]), float(prob_hi[d])
                c.n_cell[d] = int(n_cell[d])
                c.periodic[d] = 1 if periodic is None else int(periodic[d])
            else:
                c.prob_lo[d], c.prob_hi[d], c.n_cell[d], c.periodic[d] = 0.0, 1.0, 1, 1
        c.max_level, c.max_grid = int(max_level), int(max_grid)
        c.blocking_factor, c.dtn_regrid = int(blocking_factor), int(dtn_regrid)
        return self

    def setIO(self, n_out=0, t_out=0.0, data_dir="plt", restart_tstep=0):
        """Simulation::setIO (Simulation.h:155-161): a plotfile every n_out
        steps and/or every t_out of simulated time into data_dir, and the step
        to restart from (0: start from the initial condition).  The reference
        puts data_dir under its Results tree and empties it on a fresh run;
        here it is the caller's path and nothing is deleted."""
        self.dtn_outplt, self.dt_outplt = int(n_out), float(t_out)
        self.data_dir, self.restart_tstep = str(data_dir), int(restart_tstep)
        return self

    def setAmrSettings(self, tag_kind=0, tag_threshold=0.1, grid_eff=0.7, n_error_buf=1, reflux_box_quirk=1,
                       tag_advect=0, reflux=True):
        """Refinement criterion (a TAG_KINDS name or code) and the AMReX
        clustering parameters; tag_advect moves the vortex criterion's centre
        with the free stream; reflux=False drops the coarse-fine flux
        correction."""
        c = self.cfg
        c.tag_kind = TAG_KINDS[tag_kind] if isinstance(tag_kind, str) else int(tag_kind)
        c.tag_threshold, c.grid_eff = float(tag_threshold), float(grid_eff)
        c.n_error_buf, c.reflux_box_quirk = int(n_error_buf), int(reflux_box_quirk)
        c.tag_advect, c.no_reflux = int(tag_advect), 0 if reflux else 1
        return self

    def setValidationMode(self, mode):
        """Simulation::setValidationMode (Simulation.h:51-53, Solver.h:711-734):
        False/0 projects the finer levels' initial state from the coarser
        level; True/1 takes the analytic IC on every level (then average down
        and ghost fill); 2 as 1 with the finer levels' coarse-fine ghosts left
        at the analytic IC until the first step."""
        self.cfg.validation_mode = int(mode)
        return self

    # ------------------------------------------------------------ lifecycle
    def _check(self, rc, what):
        if rc != ADG_OK:
            msg = self._L.adg_last_error(self.ctx).decode() if self.ctx else ""
            raise AdgError(f"{what} failed (status {rc}): {msg}")

    def init(self, model=None):
        """Solver::init: element matrices, layout, initial condition, first Dt."""
        if model is not None:
            self.cfg.gamma = model.gamma_adiab
            self.cfg.ic = IC_CODES[model.model_case]
            for k, v in model.ic_params.items():
                setattr(self.cfg, k, v)
        h = ctypes.c_void_p()
        rc = self._L.adg_ctx_create(ctypes.byref(self.cfg), ctypes.byref(h))
        if rc != ADG_OK:
            raise AdgError(f"adg_ctx_create failed (status {rc})")
        self.ctx = h
        self._check(self._L.adg_init(self.ctx), "adg_init")
        if self.restart_tstep > 0:  # Solver::init on restart (Solver.h:571-593)
            self.restart_time = self.ReadPlotFile(self.restart_tstep)
        self._t_last_plt = self.time
        return self

    def close(self):
        if self.ctx:
            self._L.adg_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------ stepping
    def set_Dt(self):
        """Recompute Dt from the current state (AmrDG.h:1253-1357)."""
        v = ctypes.c_double()
        self._check(self._L.adg_compute_dt(self.ctx, ctypes.byref(v)), "adg_compute_dt")
        return v.value

    @property
    def Dt(self):
        v = ctypes.c_double()
        self._check(self._L.adg_get_dt(self.ctx, ctypes.byref(v)), "adg_get_dt")
        return v.value

    @Dt.setter
    def Dt(self, value):
        self._check(self._L.adg_set_dt(self.ctx, float(value)), "adg_set_dt")

    @property
    def time(self):
        v = ctypes.c_double()
        self._check(self._L.adg_get_time(self.ctx, ctypes.byref(v)), "adg_get_time")
        return v.value

    def ADER(self):
        """One predictor-corrector step with the current Dt (AmrDG.h:1071-1165)."""
        self._check(self._L.adg_ader(self.ctx), "adg_ader")

    def time_integration(self):
        """One evolve-loop body: ADER, AMR sync, t += Dt, new Dt."""
        self._check(self._L.adg_step(self.ctx), "adg_step")

    def advance(self, nsteps, use_graph=True):
        self._check(self._L.adg_advance(self.ctx, int(nsteps), int(bool(use_graph))), "adg_advance")

    def evolve(self, nsteps=None, T=None):
        """AmrDG::evolve (AmrDG.h:853-1030): fixed step count, or until T with
        the last step clamped; plotfiles as set by setIO: the initial state on
        a fresh start, then after every step n with n % n_out == 0, else when
        t_out has passed since the last one."""
        T = T if T is not None else self.T
        out = self.dtn_outplt > 0 or self.dt_outplt > 0
        if out and self.step == 0:
            self.PlotFile(0)
        if nsteps is not None and self.dt_outplt <= 0:
            left = int(nsteps)
            while left > 0:  # graph replay between plotfile steps
                k = left
                if self.dtn_outplt > 0:
                    k = min(k, self.dtn_outplt - self.step % self.dtn_outplt)
                self.advance(k)
                left -= k
                self._maybe_plot()
            return
        n_done = 0
        while (nsteps is not None and n_done < nsteps) or (nsteps is None and self.time < T):
            if nsteps is None and T - self.time < self.Dt:
                self.Dt = T - self.time
            self.time_integration()
            n_done += 1
            self._maybe_plot()

    def _maybe_plot(self):
        n, t = self.step, self.time
        if self.dtn_outplt > 0 and n % self.dtn_outplt == 0:
            self.PlotFile(n)
        elif self.dt_outplt > 0 and t - self._t_last_plt >= self.dt_outplt - 1e-12:
            self.PlotFile(n)
            self._t_last_plt = t

    @property
    def step(self):
        """Completed steps (the evolve loop's n; continues after a restart)."""
        v = ctypes.c_int64()
        self._check(self._L.adg_get_step(self.ctx, ctypes.byref(v)), "adg_get_step")
        return v.value

    # ------------------------------------------------------------ plotfiles
    def PlotFile(self, tstep, level=-1, data_dir=None, var_names=None):
        """Solver::PlotFile (Solver.h:922-968): per conserved variable q the
        AMReX plotfile <data_dir>/tstep_<tstep>_q_<q>_plt with the modes of
        U_w as components "<name>_<m>"; level -1 writes every level."""
        d = (data_dir if data_dir is not None else self.data_dir).encode()
        names = None
        if var_names is not None:
            if len(var_names) != self.Q:
                raise ValueError(f"need {self.Q} variable names")
            names = (ctypes.c_char_p * self.Q)(*[n.encode() for n in var_names])
        self._check(self._L.adg_write_plotfile(self.ctx, d, int(tstep), int(level), names), "adg_write_plotfile")

    def ReadPlotFile(self, tstep, data_dir=None):
        """Solver::ReadPlotFile (Solver.h:599-652) + the FillPatch of Solver::init:
        boxes, state, time and step count from the plotfiles of tstep.
        Returns the time read."""
        d = (data_dir if data_dir is not None else self.data_dir).encode()
        t = ctypes.c_double()
        self._check(self._L.adg_read_plotfile(self.ctx, d, int(tstep), ctypes.byref(t)), "adg_read_plotfile")
        self._t_last_plt = t.value
        return t.value

    # ------------------------------------------------------------ state
    def num_levels(self):
        n = ctypes.c_int()
        self._check(self._L.adg_num_levels(self.ctx, ctypes.byref(n)), "adg_num_levels")
        return n.value

    def level_cells(self, lev=0):
        n = ctypes.c_int64()
        self._check(self._L.adg_level_cells(self.ctx, lev, ctypes.byref(n)), "adg_level_cells")
        return n.value

    def get_U_w(self, lev=0):
        n = self.level_cells(lev)
        out = np.empty((n, self.Q, self.Np_s))
        self._check(self._L.adg_get_state(self.ctx, lev, out.ctypes.data, ADG_MEM_HOST), "adg_get_state")
        return out

    def set_U_w(self, arr, lev=0):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        assert a.size == self.level_cells(lev) * self.Q * self.Np_s
        self._check(self._L.adg_set_state(self.ctx, lev, a.ctypes.data, ADG_MEM_HOST), "adg_set_state")

    def get_U_w_async(self, pinned, lev=0):
        """Queue the copy of level lev into a PinnedArray of shape
        (cells, Q, Np_s); valid after synchronize()."""
        assert pinned.array.shape == (self.level_cells(lev), self.Q, self.Np_s)
        self._check(self._L.adg_get_state(self.ctx, lev, pinned.array.ctypes.data, ADG_MEM_HOST_ASYNC),
                    "adg_get_state")

    def set_U_w_async(self, pinned, lev=0):
        """Queue the copy of a PinnedArray into level lev; the array must not
        change before synchronize()."""
        assert pinned.array.shape == (self.level_cells(lev), self.Q, self.Np_s)
        self._check(self._L.adg_set_state(self.ctx, lev, pinned.array.ctypes.data, ADG_MEM_HOST_ASYNC),
                    "adg_set_state")

    def set_readback(self, pinned, lev=0):
        """Register a PinnedArray of shape (capacity, Q, Np_s), capacity at
        least the level's cells, whose first level_cells(lev) rows receive
        level lev's state at the end of every step of advance(), copied beside
        the rest of the step (adg_set_readback); None clears.  Valid after
        synchronize(); see readback_active() after a regrid."""
        if pinned is None:
            self._check(self._L.adg_set_readback(self.ctx, lev, None, 0), "adg_set_readback")
            return
        assert pinned.array.shape[1:] == (self.Q, self.Np_s) and pinned.array.shape[0] >= self.level_cells(lev)
        self._check(self._L.adg_set_readback(self.ctx, lev, pinned.array.ctypes.data, pinned.array.shape[0]),
                    "adg_set_readback")

    def readback_active(self, lev=0):
        """False once a regrid removed the level or grew it past the buffer
        (the registration is then dropped)."""
        v = ctypes.c_int()
        self._check(self._L.adg_readback_active(self.ctx, lev, ctypes.byref(v)), "adg_readback_active")
        return bool(v.value)

    # ------------------------------------------------------------ L2ProjInterp
    def amr_scatter(self, coarse, child):
        """L2ProjInterp::amr_scatter on a batch: coarse [n, Q, Np_s], child [n]
        (bit D-1-d: upper half in direction d) -> fine [n, Q, Np_s]."""
        c = np.ascontiguousarray(coarse, dtype=np.float64).reshape(-1, self.Q, self.Np_s)
        ch = np.ascontiguousarray(child, dtype=np.int8)
        assert ch.shape == (c.shape[0],)
        out = np.empty_like(c)
        self._check(self._L.adg_interp_scatter(self.ctx, c.ctypes.data, ch.ctypes.data, c.shape[0],
                                               out.ctypes.data, ADG_MEM_HOST), "adg_interp_scatter")
        return out

    def amr_gather(self, fine):
        """L2ProjInterp::amr_gather on a batch: fine [n, 2^D, Q, Np_s] -> coarse [n, Q, Np_s]."""
        f = np.ascontiguousarray(fine, dtype=np.float64).reshape(-1, 1 << self.D, self.Q, self.Np_s)
        out = np.empty((f.shape[0], self.Q, self.Np_s))
        self._check(self._L.adg_interp_gather(self.ctx, f.ctypes.data, f.shape[0], out.ctypes.data, ADG_MEM_HOST),
                    "adg_interp_gather")
        return out

    def average_down(self):
        """Solver::AMR_average_fine_coarse on the context's layout."""
        self._check(self._L.adg_average_down(self.ctx), "adg_average_down")

    def set_patches(self, patches):
        """Register the caller's per-box device arrays (a list of AdgPatch)
        that tile the current layout."""
        arr = (AdgPatch * max(1, len(patches)))(*patches)
        self._check(self._L.adg_set_patches(self.ctx, arr, len(patches)), "adg_set_patches")

    def read_patches(self):
        """Queue the copy of the registered patches' valid cells into the state."""
        self._check(self._L.adg_read_patches(self.ctx), "adg_read_patches")

    def write_patches(self):
        """Queue the copy of the state into the registered patches' valid cells."""
        self._check(self._L.adg_write_patches(self.ctx), "adg_write_patches")

    def autotune(self, nsteps=3):
        """Time every elements-per-block choice of the predictor on the current
        layout (state restored), keep and record the fastest; returns
        {"E": choice, "ms": {E: per-step predictor ms}}."""
        ch = self.block_choices()["choices"]
        E = ctypes.c_int()
        ms = (ctypes.c_double * len(ch))()
        self._check(self._L.adg_autotune(self.ctx, int(nsteps), ctypes.byref(E), ms, len(ch)), "adg_autotune")
        return {"E": E.value, "ms": {c: ms[i] for i, c in enumerate(ch)}}

    def block_choices(self):
        """Built elements-per-block choices and the ones in use."""
        ch = (ctypes.c_int * 16)()
        n, ep, es = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._check(self._L.adg_block_choices(self.ctx, ch, 16, ctypes.byref(n), ctypes.byref(ep), ctypes.byref(es)),
                    "adg_block_choices")
        return {"choices": list(ch[:n.value]), "plain": ep.value, "seeded": es.value}

    def Limiter_w(self):
        """The TVB limiter of the finest level on the current state
        (AmrDG::Limiter_w, AmrDG.h:1657-1855), after ADER(); returns the
        elements it modified."""
        n = ctypes.c_int64()
        self._check(self._L.adg_limit(self.ctx, ctypes.byref(n)), "adg_limit")
        return n.value

    def fill_ghosts(self):
        """The coarse-interpolated ghost cells of FillPatchTwoLevels on the context's layout."""
        self._check(self._L.adg_fill_ghosts(self.ctx), "adg_fill_ghosts")

    def synchronize(self):
        self._check(self._L.adg_synchronize(self.ctx), "adg_synchronize")

    def get_U_w_device(self, lev, dev_ptr):
        self._check(self._L.adg_get_state(self.ctx, lev, ctypes.c_void_p(dev_ptr), ADG_MEM_DEVICE), "adg_get_state")

    def set_U_w_device(self, lev, dev_ptr):
        self._check(self._L.adg_set_state(self.ctx, lev, ctypes.c_void_p(dev_ptr), ADG_MEM_DEVICE), "adg_set_state")

    def predictor(self, lev, dev_ptr):
        """Predictor H_w of the valid cells of level lev into a device buffer."""
        self._check(self._L.adg_predictor(self.ctx, lev, ctypes.c_void_p(dev_ptr)), "adg_predictor")

    def seed_set_path(self, path):
        """1: fused tensor-core seed inference (hidden width 128), 0: SIMT kernels."""
        self._check(self._L.adg_seed_set_path(self.ctx, int(path)), "adg_seed_set_path")

    def seed_infer(self, dev_ptr, path=1):
        """Seeds H_w of every element of the layout (valid of all levels, then
        ghosts) into a device buffer of n_elem * Q * Np_st doubles."""
        self._check(self._L.adg_seed_infer(self.ctx, ctypes.c_void_p(dev_ptr), int(path)), "adg_seed_infer")

    def status(self):
        v = ctypes.c_uint32()
        self._check(self._L.adg_status(self.ctx, ctypes.byref(v)), "adg_status")
        return v.value

    def launch_count(self):
        v = ctypes.c_int64()
        self._check(self._L.adg_launch_count(self.ctx, ctypes.byref(v)), "adg_launch_count")
        return v.value

    def advance_timed_flushed(self, nsteps, flush_bytes=256 << 20, use_graph=True):
        """Device ms of nsteps steps with the L2 evicted before each (flush excluded)."""
        v = ctypes.c_double()
        self._check(self._L.adg_advance_timed_flushed(self.ctx, int(nsteps), int(bool(use_graph)), int(flush_bytes),
                                                      ctypes.byref(v)), "adg_advance_timed_flushed")
        return v.value

    def advance_timed(self, nsteps, use_graph=True):
        """n steps bracketed by CUDA events on the context's stream; returns ms."""
        v = ctypes.c_double()
        self._check(self._L.adg_advance_timed(self.ctx, int(nsteps), int(bool(use_graph)), ctypes.byref(v)),
                    "adg_advance_timed")
        return v.value

    def time_kernels(self, nsteps=3):
        """Average per-step duration (ms) of each kernel kind, CUDA events."""
        out = (ctypes.c_double * 8)()
        self._check(self._L.adg_time_kernels(self.ctx, int(nsteps), out, 8), "adg_time_kernels")
        return {"predictor": out[0], "numflux": out[1], "corrector": out[2], "dt": out[3], "amr_sync": out[4],
                "seed_inference": out[5], "seeded_predictor": out[6], "fallback": out[7]}

    def dof_updates(self):
        """(total DOF updates so far, ms of host time spent in regrids)."""
        n, ms = ctypes.c_int64(), ctypes.c_double()
        self._check(self._L.adg_dof_updates(self.ctx, ctypes.byref(n), ctypes.byref(ms)), "adg_dof_updates")
        return n.value, ms.value

    def norm(self, p=2, q=0):
        """LpNorm_DG_AMR: Lp norm of component q minus the analytic initial
        condition over the leaf cells (AmrDG.h:1399-1578)."""
        v = ctypes.c_double()
        self._check(self._L.adg_lp_norm(self.ctx, int(p), int(q), ctypes.byref(v)), "adg_lp_norm")
        return v.value

    def limited_count(self):
        """Elements the TVB limiter has modified so far."""
        n = ctypes.c_int64()
        self._check(self._L.adg_limited_count(self.ctx, ctypes.byref(n)), "adg_limited_count")
        return n.value

    def leaf_dof_updates(self):
        """DOF updates so far over leaf elements only."""
        n = ctypes.c_int64()
        self._check(self._L.adg_leaf_dof_updates(self.ctx, ctypes.byref(n)), "adg_leaf_dof_updates")
        return n.value

    def regrid_profile(self):
        """Host ms spent in regrids by phase: tags+wait, clustering, tables,
        upload, remap launches, graph update."""
        ms = (ctypes.c_double * 6)()
        self._check(self._L.adg_regrid_profile(self.ctx, ms, 6), "adg_regrid_profile")
        keys = ("tags_wait", "cluster", "tables", "upload", "remap", "graph")
        return dict(zip(keys, list(ms)))

    def regrid_count(self):
        n = ctypes.c_int()
        self._check(self._L.adg_regrid_count(self.ctx, ctypes.byref(n)), "adg_regrid_count")
        return n.value

    def boxes(self, lev):
        """Boxes of level lev: array [nbox, 6] = lo0, lo1, lo2, hi0, hi1, hi2."""
        cap = 1 << 16
        buf = (ctypes.c_int * (6 * cap))()
        n = ctypes.c_int()
        self._check(self._L.adg_get_boxes(self.ctx, lev, buf, cap, ctypes.byref(n)), "adg_get_boxes")
        return np.frombuffer(buf, dtype=np.int32, count=6 * n.value).reshape(n.value, 6).copy()

    def set_layout(self, boxes_per_level):
        """Layout from the caller: one [nbox, 6] array (lo0, lo1, lo2, hi0,
        hi1, hi2) per level; the state is remapped onto it."""
        arrs = [np.asarray(b, dtype=np.int32).reshape(-1, 6) for b in boxes_per_level]
        nbox = (ctypes.c_int * len(arrs))(*[a.shape[0] for a in arrs])
        flat = np.ascontiguousarray(np.concatenate(arrs, axis=0) if arrs else np.zeros((0, 6), np.int32))
        self._check(self._L.adg_set_layout(self.ctx, len(arrs), nbox, flat.ctypes.data_as(ctypes.POINTER(ctypes.c_int))),
                    "adg_set_layout")

    def level_cell_coords(self, lev):
        """(i, j, k) of the valid cells of level lev in state order: [n, 3]."""
        n = self.level_cells(lev)
        out = np.zeros((n, 3), dtype=np.int32)
        self._check(self._L.adg_level_cell_coords(self.ctx, lev, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int))),
                    "adg_level_cell_coords")
        return out

    def tags(self, lev):
        """Refinement tags of the valid cells of level lev (current state)."""
        n = self.level_cells(lev)
        out = np.zeros(n, dtype=np.uint8)
        self._check(self._L.adg_tags(self.ctx, lev, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))), "adg_tags")
        return out

    def set_stream(self, stream_handle):
        self._check(self._L.adg_set_stream(self.ctx, ctypes.c_void_p(stream_handle)), "adg_set_stream")


class PredictorSeed:
    """Learned predictor seed (MLP, FP32, trained on the GPU).

    Inputs: the element's Q*Np_s modal coefficients and Dt/dx (standardised);
    three hidden layers of `hidden` units with GELU; outputs the Q*Np_st
    space-time predictor coefficients (as H_w - W U_w, standardised)."""

    def __init__(self, D, P, hidden=128, rng_seed=1234):
        self.D, self.P, self.hidden = D, P, hidden
        self._L = lib()
        h = ctypes.c_void_p()
        rc = self._L.adg_seed_create(D, P, hidden, rng_seed, ctypes.byref(h))
        if rc != ADG_OK:
            raise AdgError(f"adg_seed_create failed ({rc})")
        self.h = h
        self.Q = D + 2
        self.n_in = self.Q * comb(P + D, D) + 1
        self.n_out = self.Q * comb(P + D + 1, D + 1)

    def close(self):
        if self.h:
            self._L.adg_seed_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ok(self, rc, what):
        if rc != ADG_OK:
            raise AdgError(f"{what} failed ({rc})")

    def collect(self, sim, target_sweeps=8):
        self._ok(self._L.adg_seed_collect(sim.ctx, self.h, int(target_sweeps)), "adg_seed_collect")

    def num_samples(self):
        n = ctypes.c_int64()
        self._ok(self._L.adg_seed_num_samples(self.h, ctypes.byref(n)), "adg_seed_num_samples")
        return n.value

    def train(self, epochs, batch=4096, lr=1e-3):
        v = ctypes.c_double()
        self._ok(self._L.adg_seed_train(self.h, int(epochs), int(batch), float(lr), ctypes.byref(v)), "adg_seed_train")
        return v.value

    def forward(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.zeros((X.shape[0], self.n_out), dtype=np.float32)
        self._ok(self._L.adg_seed_forward(self.h, X.ctypes.data, X.shape[0], Y.ctypes.data), "adg_seed_forward")
        return Y

    def gradients(self, X, T):
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        nw, _ = self.num_params()
        g = np.zeros(nw, dtype=np.float32)
        loss = ctypes.c_double()
        self._ok(self._L.adg_seed_gradients(self.h, X.ctypes.data, T.ctypes.data, X.shape[0], g.ctypes.data,
                                            ctypes.byref(loss)), "adg_seed_gradients")
        return g, loss.value

    def num_params(self):
        a, b = ctypes.c_int64(), ctypes.c_int64()
        self._ok(self._L.adg_seed_num_params(self.h, ctypes.byref(a), ctypes.byref(b)), "adg_seed_num_params")
        return a.value, b.value

    def get_params(self):
        _, n = self.num_params()
        out = np.zeros(n, dtype=np.float32)
        self._ok(self._L.adg_seed_get_params(self.h, out.ctypes.data), "adg_seed_get_params")
        return out

    def set_params(self, v):
        v = np.ascontiguousarray(v, dtype=np.float32)
        self._ok(self._L.adg_seed_set_params(self.h, v.ctypes.data), "adg_seed_set_params")

    def weights(self):
        """List of (W, b) per layer from the flat parameter vector."""
        p = self.get_params()
        sizes = [(self.n_in, self.hidden), (self.hidden, self.hidden), (self.hidden, self.hidden),
                 (self.hidden, self.n_out)]
        out, o = [], 0
        for (a, b) in sizes:
            W = p[o:o + a * b].reshape(a, b)
            o += a * b
            bias = p[o:o + b]
            o += b
            out.append((W, bias))
        return out

    def attach(self, sim, mode=1, sweeps=1, tol=1e-3):
        """mode 1: seeded sweeps in FP64, 2: in FP32, 0: detach."""
        self._ok(self._L.adg_seed_attach(sim.ctx, self.h if mode else None, int(mode), int(sweeps), float(tol)),
                 "adg_seed_attach")


def seed_stats(sim):
    a, b = ctypes.c_int64(), ctypes.c_int64()
    rc = lib().adg_seed_stats(sim.ctx, ctypes.byref(a), ctypes.byref(b))
    if rc != ADG_OK:
        raise AdgError("adg_seed_stats failed")
    return a.value, b.value


def plotfile_info(path):
    """Header of one plotfile directory (no context, no GPU needed):
    dict(dim, ncomp, finest_level, time, step); raises AdgError when the
    plotfile is missing or malformed."""
    i = ctypes.c_int
    dim, nc, fin, st = i(), i(), i(), i()
    t = ctypes.c_double()
    err = ctypes.create_string_buffer(512)
    rc = lib().adg_plotfile_info(str(path).encode(), ctypes.byref(dim), ctypes.byref(nc), ctypes.byref(fin),
                                 ctypes.byref(t), ctypes.byref(st), err, 512)
    if rc != ADG_OK:
        raise AdgError(f"adg_plotfile_info failed (status {rc}): {err.value.decode()}")
    return dict(dim=dim.value, ncomp=nc.value, finest_level=fin.value, time=t.value, step=st.value)


def set_device(dev):
    rc = lib().adg_set_device(int(dev))
    if rc != ADG_OK:
        raise AdgError(f"adg_set_device({dev}) failed")


class PinnedArray:
    """numpy view of a page-locked host buffer allocated by the library."""

    def __init__(self, shape):
        n = int(np.prod(shape)) * 8
        self._p = ctypes.c_void_p()
        if lib().adg_host_alloc(n, ctypes.byref(self._p)) != ADG_OK:
            raise AdgError("adg_host_alloc failed")
        buf = (ctypes.c_double * int(np.prod(shape))).from_address(self._p.value)
        self.array = np.frombuffer(buf, dtype=np.float64).reshape(shape)

    def free(self):
        if self._p:
            lib().adg_host_free(self._p)
            self._p = None


def fp64_peak_gflops():
    v = ctypes.c_double()
    rc = lib().adg_fp64_peak_probe(ctypes.byref(v))
    if rc != ADG_OK:
        raise AdgError(f"adg_fp64_peak_probe failed ({rc})")
    return v.value


def flops_per_element(D, P):
    a, b = ctypes.c_double(), ctypes.c_double()
    rc = lib().adg_flops_per_element(D, P, ctypes.byref(a), ctypes.byref(b))
    if rc != ADG_OK:
        raise AdgError("unsupported (D, P)")
    return a.value, b.value
