"""Polynomial degrees above 3 (the reference's AmrDG<P> is a template over
P, AmrDG_NumericalFlux.tpp:42; its thesis reports p = 6): D = 2 with
P = 4, 5, 6 and D = 3 with P = 3 on the plain FP64 path against the oracle
after several steps (1e-12 relative), a two-level run with identical tags
and boxes, and the p = 6 vortex after one period against the oracle's error.
The initial condition, first Dt and one-step parity of these cases run with
the other configurations in test_gpu_single_level.py / test_gpu_amr.py."""
import numpy as np
import pytest

import oracle_ffi as O
from parity import CASES, G, HIGH_DEGREE, make_gpu, make_gpu_amr, make_oracle, make_oracle_amr, rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case,steps", [("vortex_p4", 12), ("kh_p5_outflow", 8), ("vortex_p6", 8), ("blast3d_p3", 5)])
def test_high_degree_run_matches_oracle(case, steps):
    assert case in HIGH_DEGREE
    o = make_oracle(case)
    g = make_gpu(case)
    assert rel_err(g.get_U_w(), o.get_uw()) < 1e-13
    g.set_U_w(o.get_uw())
    g.Dt = o.dt
    for _ in range(steps):
        o.step()
        g.time_integration()
        assert abs(g.Dt - o.dt) / o.dt < 1e-12
    assert rel_err(g.get_U_w(), o.get_uw()) < 1e-12
    assert g.status() == 0


def test_p4_two_levels_match_oracle():
    o = make_oracle_amr("kh_p4_amr")
    g = make_gpu_amr("kh_p4_amr")
    for l in range(o.num_levels()):
        g.set_U_w(o.get_uw(l), l)
    g.Dt = o.dt
    for s in range(6):
        for l in range(min(o.num_levels(), 1)):
            assert np.array_equal(g.tags(l), o.tags(l).astype(np.uint8)), f"tags before step {s}"
        o.step()
        g.time_integration()
        assert g.num_levels() == o.num_levels()
        for l in range(o.num_levels()):
            assert np.array_equal(g.boxes(l), o.boxes(l)), f"boxes of level {l} after step {s}"
    for l in range(o.num_levels()):
        assert rel_err(g.get_U_w(l), o.get_uw(l)) < 1e-12, f"level {l}"


def test_p6_vortex_period_error_matches_oracle():
    """p = 6, N = 8, T = 10: the density L2 error of the GPU run equals the
    oracle's (thesis Table 5.2 reports 8.3997e-5 for its own, slightly
    different set-up; the oracle's is within 0.4 % of it, as the thesis'
    p = 3 value is within 0.7 % of the reference's recorded run)."""
    cfg = O.make_cfg(D=2, P=6, n=(8, 8, 1), hi=(10, 10, 1), ic="vortex", u_inf=1.0, v_inf=0.0, c_dt=0.9)
    o = O.OracleSim(cfg)
    o.init()
    s = G.AmrDG(P=6, D=2)
    s.setGeometrySettings(prob_lo=(0, 0), prob_hi=(10, 10), n_cell=(8, 8))
    s.settings(c_dt=0.9)
    s.init(G.Compressible_Euler().settings("isentropic_vortex", u_inf=1.0, v_inf=0.0))
    T = 10.0
    while o.time < T:
        if T - o.time < o.dt:
            o.dt = T - o.time
        o.step()
    while s.time < T:
        if T - s.time < s.Dt:
            s.Dt = T - s.time
        s.time_integration()
    for p in (1, 2):
        a, b = s.norm(p, 0), o.norm(p, 0)
        assert abs(a - b) <= 1e-11 * b, (p, a, b)
    assert abs(s.norm(2, 0) - 8.3997e-5) / 8.3997e-5 < 0.01


def test_learned_seed_is_refused_above_its_degrees():
    g = make_gpu("vortex_p4")
    seed = G.PredictorSeed(2, 4, hidden=128, rng_seed=1)
    with pytest.raises(G.AdgError):
        seed.attach(g, mode=2, sweeps=2, tol=1e-3)
