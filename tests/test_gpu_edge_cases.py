"""Edge cases of the layout on the GPU against the oracle: one-cell and
one-cell-thick grids (periodic self-neighbours, outflow mirrors on both
sides), element counts that leave the last predictor block partly empty,
strongly stretched cells, and rejected configurations."""
import numpy as np
import pytest

import oracle_ffi as O
from parity import G

pytestmark = pytest.mark.gpu

EDGE = {
    # name: D, P, n, hi, periodic, ic, extra
    "one_cell_periodic": (2, 2, (1, 1, 1), (1.0, 1.0, 1.0), (1, 1, 1), "vortex", dict(u_inf=0.3, v_inf=0.1)),
    "strip_outflow": (2, 3, (7, 1, 1), (7.0, 0.5, 1.0), (0, 0, 1), "vortex", dict(u_inf=0.2, v_inf=0.0)),
    "odd_count_kh": (2, 3, (13, 11, 1), (1.0, 1.0, 1.0), (1, 1, 1), "kh_noise", dict(seed=5, noise_amp=1e-3)),
    "stretched": (2, 1, (40, 3, 1), (10.0, 0.1, 1.0), (1, 0, 1), "vortex", dict(u_inf=1.0, v_inf=0.0)),
    "column_3d": (3, 1, (1, 1, 9), (1.0, 1.0, 1.0), (1, 1, 0), "blast3d", dict()),
    "odd_3d": (3, 2, (5, 3, 2), (1.0, 0.6, 0.4), (0, 1, 0), "blast3d", dict()),
}
ORACLE_IC = {"vortex": "vortex", "kh_noise": "kh_noise", "blast3d": "blast3d"}
GPU_IC = {"vortex": "isentropic_vortex", "kh_noise": "kh_noise", "blast3d": "blast3d"}


def state_err(a, b):
    """max |a - b| relative to the largest cell mean of any variable (several
    of these states have variables that are zero or nearly so throughout)."""
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b[:, :, 0])))


@pytest.mark.parametrize("case", list(EDGE))
def test_edge_layout_matches_oracle(case):
    D, P, n, hi, per, ic, extra = EDGE[case]
    o = O.OracleSim(O.make_cfg(D=D, P=P, n=n, hi=hi, periodic=per, ic=ORACLE_IC[ic], c_dt=0.5, **extra))
    o.init()
    g = G.AmrDG(P=P, D=D)
    g.setGeometrySettings(prob_lo=(0, 0, 0), prob_hi=hi, n_cell=n, periodic=per)
    g.settings(c_dt=0.5)
    g.init(G.Compressible_Euler().settings(GPU_IC[ic], **extra))
    g.set_U_w(o.get_uw())
    g.Dt = o.dt
    for _ in range(6):
        o.step()
        g.time_integration()
        assert abs(g.Dt - o.dt) / o.dt < 1e-12
    assert state_err(g.get_U_w(), o.get_uw()) < 1e-12
    assert g.status() == 0


@pytest.mark.parametrize("bad", [dict(n_cell=(0, 4, 1)), dict(P=7), dict(D=4)])
def test_invalid_configurations_are_rejected(bad):
    D, P = bad.get("D", 2), bad.get("P", 2)
    g = G.AmrDG(P=P, D=min(D, 3))
    if D != min(D, 3):
        g.cfg.D = D
    g.setGeometrySettings(prob_lo=(0, 0, 0), prob_hi=(1, 1, 1), n_cell=bad.get("n_cell", (4, 4, 4)))
    g.settings(c_dt=0.5)
    with pytest.raises(G.AdgError):
        g.init(G.Compressible_Euler().settings("isentropic_vortex"))
