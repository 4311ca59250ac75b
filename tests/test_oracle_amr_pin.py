"""Pin the oracle's multi-level path to the reference's own recorded outputs.

The reference's post-processing script records the density L2 errors of its
two-level isentropic-vortex runs (p = 2, Source/PostProcessing/convergence.py,
tests/golden/vortex_amr_p2_l2.json): at t = 0 with the analytic and the
projected initial condition, and after one period (T = 10) with static
refinement.  The t = 0 errors depend on which cells are refined (the
reference's vortex criterion, AMReX clustering with blocking factor 4, the
L2 norm over leaf cells); the T = 10 errors on everything a multi-level step
does (both levels' ADER, the coarse-fine flux registers and reflux, the
average down, the ghost fill, Dt over levels), over 472 to 1942 steps.
"""
import json
import os

import pytest

import oracle_ffi as O

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "vortex_amr_p2_l2.json")))


def vortex_amr_cfg(N, validation_mode=1, dtn_regrid=0, dt_regrid=0.0, tag_advect=0, no_reflux=0):
    """The reference's vortex preset with one fine level (Source/main.cpp:62-83,
    amr_c[0] = 1.4: cells within 1.96 of the centre are refined)."""
    return O.make_cfg(D=2, P=2, n=(N, N, 1), hi=(10.0, 10.0, 1.0), ic="vortex", u_inf=1.0, v_inf=0.0, c_dt=0.9,
                      max_grid=128, max_level=1, blocking_factor=4, n_error_buf=1, grid_eff=0.7,
                      dtn_regrid=dtn_regrid, dt_regrid=dt_regrid, tag_kind=2, amr_c=[1.4],
                      tag_advect=tag_advect, validation_mode=validation_mode, no_reflux=no_reflux)


def run_to(s, T):
    n = 0
    while s.time < T:
        if T - s.time < s.dt:
            s.dt = T - s.time
        s.step()
        n += 1
    return n


def ref_value(run, N):
    return GOLD["runs"][run]["L2"][GOLD["N"].index(N)]


@pytest.mark.parametrize("run", ["t0_analytic_ic", "t0_projected_ic"])
@pytest.mark.parametrize("N", [8, 16, 32])
def test_initial_hierarchy_error_matches_reference(run, N):
    s = O.OracleSim(vortex_amr_cfg(N, validation_mode=GOLD["runs"][run]["validation_mode"]))
    s.init()
    assert s.num_levels() == 2
    # the refined disc of radius 1.96 about (5, 5), buffered by one cell and
    # coarsened by the blocking factor: one box of a quarter of the domain
    b = s.boxes(1)
    assert b.tolist() == [[N // 2, N // 2, 0, 3 * N // 2 - 1, 3 * N // 2 - 1, 0]]
    got, ref = s.norm(2, 0), ref_value(run, N)
    assert abs(got - ref) / ref < 1e-12, (got, ref)


@pytest.mark.parametrize("run,N", [("static_projected_ic", 8), ("static_projected_ic", 16),
                                   ("static_analytic_ic", 8), ("static_analytic_ic", 16),
                                   ("static_projected_ic", 32), ("static_analytic_ic", 32)])
def test_static_refinement_error_matches_reference(run, N):
    s = O.OracleSim(vortex_amr_cfg(N, validation_mode=GOLD["runs"][run]["validation_mode"]))
    s.init()
    run_to(s, 10.0)
    got, ref = s.norm(2, 0), ref_value(run, N)
    # rounding differences accumulate over up to 1942 steps
    assert abs(got - ref) / ref < 1e-11, (got, ref)


def test_validation_modes_differ_only_through_the_initial_ghost_fill():
    """Mode 1 (ghost fill of every level at t = 0, the current
    AMR_sync_initial_condition) and mode 2 (the fine ghosts keep their
    analytic projection until the first step) start from the same valid
    state; only mode 2 reproduces the recorded static run."""
    a = O.OracleSim(vortex_amr_cfg(8, validation_mode=1))
    b = O.OracleSim(vortex_amr_cfg(8, validation_mode=2))
    a.init()
    b.init()
    for l in range(2):
        assert (a.get_uw(l) == b.get_uw(l)).all()
    run_to(a, 10.0)
    run_to(b, 10.0)
    ref = ref_value("static_analytic_ic", 8)
    assert abs(b.norm(2, 0) - ref) / ref < 1e-12
    assert abs(a.norm(2, 0) - ref) / ref > 1e-5


def test_fixed_centre_criterion_keeps_the_static_boxes():
    """With the reference's fixed-centre vortex criterion a regrid every step
    keeps the initial boxes, so it reproduces the static run; the recorded
    dynamic-refinement errors therefore came from another tagging code."""
    a = O.OracleSim(vortex_amr_cfg(8, validation_mode=2))
    b = O.OracleSim(vortex_amr_cfg(8, validation_mode=2, dtn_regrid=1))
    a.init()
    b.init()
    run_to(a, 10.0)
    run_to(b, 10.0)
    assert b.layout_changes() == 1  # the first step's regrid only
    assert b.norm(2, 0) == a.norm(2, 0)
    dyn = ref_value("dynamic_every_step", 8)
    assert abs(b.norm(2, 0) - dyn) / dyn > 1.0


def test_advected_centre_moves_the_fine_level():
    s = O.OracleSim(vortex_amr_cfg(8, validation_mode=1, dt_regrid=0.5, tag_advect=1))
    s.init()
    b0 = s.boxes(1).tolist()
    run_to(s, 2.0)
    assert s.boxes(1).tolist() != b0
    assert s.layout_changes() >= 2
