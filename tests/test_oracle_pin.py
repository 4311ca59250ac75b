"""Pin the CPU oracle to the reference's own recorded outputs.

The reference ships no tests; its post-processing script records the density
L2 errors its runs produced for the isentropic vortex (single level, p = 1..3).
The oracle restates the reference's algorithm; reproducing those numbers to
~1e-13 relative pins the restatement (matrices, predictor, corrector, LLF,
set_Dt, IC projection and the L2 norm machinery at once).
"""
import json
import os

import pytest

import oracle_ffi as O

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "vortex_single_level_l2.json")))


def run_vortex(P, N, T=10.0, c_dt=0.9):
    s = O.OracleSim(O.make_cfg(D=2, P=P, n=(N, N, 1), hi=(10.0, 10.0, 1.0), ic="vortex",
                               u_inf=1.0, v_inf=0.0, c_dt=c_dt))
    s.init()
    while s.time < T:
        if T - s.time < s.dt:
            s.dt = T - s.time
        s.step()
    return s


@pytest.mark.parametrize("P,N", [(1, 8), (2, 8), (3, 8), (1, 16), (2, 16), (3, 16)])
def test_vortex_l2_matches_reference_outputs(P, N):
    s = run_vortex(P, N)
    ref = GOLD["L2"][str(P)][GOLD["N"].index(N)]
    got = s.norm(2, 0)
    # the reference sums cell norms in a thread-dependent order
    assert abs(got - ref) / ref < 1e-11, (got, ref)


def test_p6_vortex_error_near_thesis_table():
    """p = 6 (the highest degree the thesis reports, Table 5.2 p. 40: L1
    5.4456e-5, L2 8.3997e-5 at N = 8).  The thesis runs used a slightly
    different set-up than the reference's recorded ones (its p = 3, N = 8 L2,
    2.7705e-3, is 0.6 % from the recorded 2.7878e-3), so the oracle is
    checked to the same closeness, not to rounding."""
    s = run_vortex(6, 8)
    assert abs(s.norm(1, 0) - 5.4456e-5) / 5.4456e-5 < 0.01
    assert abs(s.norm(2, 0) - 8.3997e-5) / 8.3997e-5 < 0.01
