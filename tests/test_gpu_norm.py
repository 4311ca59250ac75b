"""The GPU path against the reference's own recorded outputs: the density L2
error of the isentropic vortex after one period (T = 10, single level,
p = 1..3), which the reference's post-processing script records
(Source/PostProcessing/convergence.py:8-10), computed with the device Lp norm
(LpNorm_DG_AMR, AmrDG.h:1399-1578).  Also the norm itself against the
oracle's on an AMR state."""
import json
import os

import pytest

from parity import G, make_gpu_amr, make_oracle_amr

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "vortex_single_level_l2.json")))


def run_vortex_gpu(P, N, T=10.0, c_dt=0.9):
    s = G.AmrDG(P=P, D=2)
    s.setGeometrySettings(prob_lo=(0, 0), prob_hi=(10, 10), n_cell=(N, N))
    s.settings(c_dt=c_dt)
    s.init(G.Compressible_Euler().settings("isentropic_vortex", u_inf=1.0, v_inf=0.0))
    while s.time < T:
        if T - s.time < s.Dt:
            s.Dt = T - s.time
        s.time_integration()
    return s


@pytest.mark.parametrize("P,N", [(1, 8), (2, 8), (3, 8), (1, 16), (2, 16), (3, 16)])
def test_gpu_vortex_l2_matches_reference_outputs(P, N):
    s = run_vortex_gpu(P, N)
    ref = GOLD["L2"][str(P)][GOLD["N"].index(N)]
    got = s.norm(2, 0)
    assert abs(got - ref) / ref < 1e-11, (got, ref)


@pytest.mark.parametrize("p", [1, 2])
def test_norm_matches_oracle_on_amr_state(p):
    o = make_oracle_amr("kh_p3_amr")
    g = make_gpu_amr("kh_p3_amr")
    for l in range(o.num_levels()):
        g.set_U_w(o.get_uw(l), l)
    g.Dt = o.dt
    for _ in range(5):
        o.step()
        g.time_integration()
    for q in (0, 3):
        a, b = g.norm(p, q), o.norm(p, q)
        assert abs(a - b) <= 1e-12 * abs(b), (q, a, b)
