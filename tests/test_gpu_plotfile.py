"""Plotfiles on the GPU path: Solver::PlotFile / Solver::ReadPlotFile
(Source/Core/Solver.h:599-652, 922-968) through adg_write_plotfile /
adg_read_plotfile.

* What the library writes is read back by an independent parser
  (plotfile_py) and compared value for value with the device state.
* What an independent writer produces, in the variants the format allows
  (other box decompositions, big-endian or 4-byte reals, FABs grown by ghost
  cells, several data files per level), is read by the library into the state
  it describes.
* A restart continues bitwise: run n steps, write, run m more; a fresh context
  that reads the plotfile and runs m steps ends in the same state, layout,
  time and Dt.
* Bad plotfiles are rejected before the context changes.
"""
import os

import numpy as np
import pytest

from parity import AMR_CASES, G, GPU_IC
from plotfile_py import level_from_state, read_plotfile, write_plotfile

pytestmark = pytest.mark.gpu

NAMES = {2: ["mass_density", "momentum_x", "momentum_y", "energy_density"],
         3: ["mass_density", "momentum_x", "momentum_y", "momentum_z", "energy_density"]}


def amr_sim(case, io=None, max_level=None, n_cell=None, **kw):
    D, P, n, hi, per, ic, extra, amr = AMR_CASES[case]
    m = G.Compressible_Euler().settings(GPU_IC[ic], **extra)
    s = G.AmrDG(P=P, D=D)
    s.setGeometrySettings(prob_lo=(0, 0, 0), prob_hi=hi, n_cell=n_cell or n, periodic=per,
                          max_level=amr["max_level"] if max_level is None else max_level,
                          max_grid=amr["max_grid"], blocking_factor=amr["blocking_factor"],
                          dtn_regrid=amr["dtn_regrid"])
    s.setAmrSettings(tag_kind=amr["tag_kind"], tag_threshold=amr["tag_threshold"])
    s.settings(**kw)
    if io:
        s.setIO(**io)
    s.init(m)
    return s


def boxes_of(s, l):
    return [(tuple(b[:s.D]), tuple(b[3:3 + s.D])) for b in s.boxes(l)]


def snapshot(s):
    return dict(levels=[s.get_U_w(l) for l in range(s.num_levels())],
                boxes=[boxes_of(s, l) for l in range(s.num_levels())], time=s.time, Dt=s.Dt, step=s.step)


def assert_same(a, b):
    assert len(a["levels"]) == len(b["levels"])
    assert a["boxes"] == b["boxes"]
    for ua, ub in zip(a["levels"], b["levels"]):
        assert np.array_equal(ua, ub)
    assert a["time"] == b["time"] and a["Dt"] == b["Dt"] and a["step"] == b["step"]


def plt_dir(root, tstep, q):
    return os.path.join(str(root), f"tstep_{tstep}_q_{q}_plt")


@pytest.mark.parametrize("case", ["kh_p3_amr", "blast3d_p2_amr"])
def test_written_plotfiles_parse_independently(tmp_path, case):
    s = amr_sim(case)
    s.advance(4)
    s.PlotFile(4, data_dir=str(tmp_path))
    t, D, nl = s.time, s.D, s.num_levels()
    dx0 = [1.0 / AMR_CASES[case][2][d] * AMR_CASES[case][3][d] for d in range(D)]
    for q in range(s.Q):
        pf = read_plotfile(plt_dir(tmp_path, 4, q))
        assert pf["version"] == "HyperCLaw-V1.1"
        assert pf["names"] == [f"{NAMES[D][q]}_{m}" for m in range(s.Np_s)]
        assert pf["dim"] == D and pf["time"] == t and pf["finest_level"] == nl - 1
        assert pf["ref_ratio"] == [2] * (nl - 1) and pf["level_steps"] == [4] * nl
        assert pf["coord"] == 0 and pf["bwidth"] == 0
        assert pf["prob_lo"] == [0.0] * D and pf["prob_hi"] == list(AMR_CASES[case][3][:D])
        for l in range(nl):
            n_l = [AMR_CASES[case][2][d] << l for d in range(D)]
            assert pf["domains"][l] == ((0,) * D, tuple(x - 1 for x in n_l))
            assert pf["dx"][l] == pytest.approx([x / 2 ** l for x in dx0], rel=1e-15)
            L = pf["levels"][l]
            assert L["cellh_head"] == ["1", "1", str(s.Np_s), "0"]
            assert L["boxes"] == boxes_of(s, l) and L["step"] == 4 and L["time"] == t
            expect = level_from_state(s.get_U_w(l)[:, q, :], s.level_cell_coords(l), L["boxes"], D)
            for b, (got, want) in enumerate(zip(L["data"], expect)):
                assert np.array_equal(got, want)
                assert L["mins"][b] == [float(want[m].min()) for m in range(s.Np_s)]
                assert L["maxs"][b] == [float(want[m].max()) for m in range(s.Np_s)]
            for (lo, hi), ext in zip(L["boxes"], L["extents"]):
                for d in range(D):
                    assert ext[d] == pytest.approx((lo[d] * pf["dx"][l][d], (hi[d] + 1) * pf["dx"][l][d]), abs=1e-14)
        info = G.plotfile_info(plt_dir(tmp_path, 4, q))
        assert info == dict(dim=D, ncomp=s.Np_s, finest_level=nl - 1, time=t, step=4)


@pytest.mark.parametrize("case,n,m,kw", [
    ("kh_p3_amr", 8, 8, {}),
    ("kh_p2_amr_rect", 6, 5, {}),
    ("blast3d_p2_amr", 4, 4, dict(limiter_type="TVB", TVB_M=10.0, t_limit=1)),
])
def test_restart_continues_bitwise(tmp_path, case, n, m, kw):
    a = amr_sim(case, **kw)
    a.advance(n)
    a.PlotFile(n, data_dir=str(tmp_path))
    a.advance(m)
    b = amr_sim(case, io=dict(data_dir=str(tmp_path), restart_tstep=n), **kw)
    assert b.step == n
    b.advance(m)
    assert_same(snapshot(a), snapshot(b))
    assert a.status() == 0 and b.status() == 0


def test_single_level_plotfile(tmp_path):
    s = amr_sim("kh_p3_amr")
    s.advance(3)
    nl = s.num_levels()
    assert nl == 3
    s.PlotFile(3, level=1, data_dir=str(tmp_path))
    pf = read_plotfile(plt_dir(tmp_path, 3, 0))
    assert pf["finest_level"] == 0 and pf["domains"][0] == ((0, 0), (31, 31))
    assert pf["dx"][0] == [1.0 / 32, 1.0 / 32]
    got = pf["levels"][0]["data"]
    want = level_from_state(s.get_U_w(1)[:, 0, :], s.level_cell_coords(1), pf["levels"][0]["boxes"], 2)
    for g, w in zip(got, want):
        assert np.array_equal(g, w)


def _levels_for_writer(s, q, boxes, step):
    D = s.D
    out = []
    for l, bl in enumerate(boxes):
        n_l = [s.cfg.n_cell[d] << l for d in range(D)]
        dx = [(s.cfg.prob_hi[d] - s.cfg.prob_lo[d]) / n_l[d] for d in range(D)]
        data = level_from_state(s.get_U_w(l)[:, q, :], s.level_cell_coords(l), bl, D)
        out.append(dict(domain=((0,) * D, tuple(x - 1 for x in n_l)), dx=dx, step=step, boxes=list(bl), data=data))
    return out


def _split_x(boxes):
    """Each box cut in two along x where it is at least two cells wide."""
    out = []
    for lo, hi in boxes:
        if hi[0] > lo[0]:
            mid = (lo[0] + hi[0]) // 2
            out += [(lo, (mid,) + hi[1:]), ((mid + 1,) + lo[1:], hi)]
        else:
            out.append((lo, hi))
    return out


@pytest.mark.parametrize("variant", [dict(), dict(byte_order=">"), dict(ngrow=1), dict(boxes_per_file=2),
                                     dict(real_bytes=4)])
def test_reads_independently_written_plotfiles(tmp_path, variant):
    s = amr_sim("kh_p3_amr")
    s.advance(5)
    nl = s.num_levels()
    boxes = [_split_x(boxes_of(s, l)) for l in range(nl)]
    for q in range(s.Q):
        write_plotfile(plt_dir(tmp_path, 5, q), s.D, [f"{NAMES[2][q]}_{m}" for m in range(s.Np_s)], s.time,
                       [0.0, 0.0], [1.0, 1.0], _levels_for_writer(s, q, boxes, 5), **variant)
    r = amr_sim("kh_p3_amr")
    t = r.ReadPlotFile(5, data_dir=str(tmp_path))
    assert t == s.time and r.time == s.time and r.step == 5
    assert r.num_levels() == nl
    for l in range(nl):
        assert boxes_of(r, l) == boxes[l]
        want = s.get_U_w(l)
        if variant.get("real_bytes") == 4:
            want = want.astype(np.float32).astype(np.float64)
        assert np.array_equal(r.get_U_w(l), want)
    r.advance(2)
    assert r.status() == 0


def test_read_caps_levels_at_max_level(tmp_path):
    s = amr_sim("kh_p3_amr")
    s.advance(4)
    assert s.num_levels() == 3
    s.PlotFile(4, data_dir=str(tmp_path))
    r = amr_sim("kh_p3_amr", max_level=1)
    r.ReadPlotFile(4, data_dir=str(tmp_path))
    assert r.num_levels() == 2
    for l in range(2):
        assert boxes_of(r, l) == boxes_of(s, l)
        assert np.array_equal(r.get_U_w(l), s.get_U_w(l))


def test_evolve_writes_plotfiles_and_init_restarts(tmp_path):
    s = amr_sim("kh_p3_amr", io=dict(n_out=4, data_dir=str(tmp_path)))
    s.evolve(nsteps=9)
    for n in (0, 4, 8):
        for q in range(s.Q):
            assert os.path.isdir(plt_dir(tmp_path, n, q)), (n, q)
    assert not os.path.exists(plt_dir(tmp_path, 9, 0))
    twin = amr_sim("kh_p3_amr")
    twin.advance(8)
    assert G.plotfile_info(plt_dir(tmp_path, 8, 2)) == dict(dim=2, ncomp=10, finest_level=twin.num_levels() - 1,
                                                          time=twin.time, step=8)
    r = amr_sim("kh_p3_amr", io=dict(n_out=4, data_dir=str(tmp_path), restart_tstep=8))
    assert r.restart_time == twin.time and r.step == 8
    r.evolve(nsteps=4)
    assert r.step == 12 and os.path.isdir(plt_dir(tmp_path, 12, 3))
    twin.advance(4)
    for l in range(twin.num_levels()):
        assert np.array_equal(r.get_U_w(l), twin.get_U_w(l))


def test_time_interval_output(tmp_path):
    s = amr_sim("kh_p3_amr", io=dict(t_out=0.0015, data_dir=str(tmp_path)))
    s.evolve(nsteps=16)
    written = sorted(int(d.split("_")[1]) for d in os.listdir(tmp_path) if d.endswith("_q_0_plt"))
    assert written[0] == 0 and len(written) >= 2
    times = [G.plotfile_info(plt_dir(tmp_path, n, 0))["time"] for n in written]
    assert all(b - a >= 0.0015 - 1e-12 for a, b in zip(times[1:], times[2:]))
    assert times[1] >= 0.0015 - 1e-12


def _assert_unchanged(r, before):
    assert_same(before, snapshot(r))
    r.advance(1)
    assert r.status() == 0


def test_bad_plotfiles_leave_the_context_unchanged(tmp_path):
    r = amr_sim("kh_p3_amr")
    r.advance(2)
    before = snapshot(r)
    # missing
    with pytest.raises(G.AdgError, match="status 7"):
        r.ReadPlotFile(99, data_dir=str(tmp_path))
    assert_same(before, snapshot(r))
    # dimension
    d3 = amr_sim("blast3d_p2_amr")
    d3.PlotFile(1, data_dir=str(tmp_path / "d3"))
    with pytest.raises(G.AdgError, match="dimension"):
        r.ReadPlotFile(1, data_dir=str(tmp_path / "d3"))
    # component count (P = 2 state into a P = 3 context)
    p2 = amr_sim("kh_p2_amr_rect")
    p2.PlotFile(1, data_dir=str(tmp_path / "p2"))
    with pytest.raises(G.AdgError, match="component count"):
        r.ReadPlotFile(1, data_dir=str(tmp_path / "p2"))
    # level-0 domain
    big = amr_sim("kh_p3_amr", n_cell=(32, 32, 1))
    big.PlotFile(1, data_dir=str(tmp_path / "big"))
    with pytest.raises(G.AdgError, match="domain"):
        r.ReadPlotFile(1, data_dir=str(tmp_path / "big"))
    assert_same(before, snapshot(r))
    # level 1 without the box under a level-2 box (improper nesting): a layout error
    s = amr_sim("kh_p3_amr")
    s.advance(4)
    assert s.num_levels() == 3
    boxes = [boxes_of(s, l) for l in range(3)]
    plo = [c // 2 for c in boxes[2][0][0]]
    under = [b for b, (lo, hi) in enumerate(boxes[1]) if all(lo[d] <= plo[d] <= hi[d] for d in range(2))]
    assert len(under) == 1
    for q in range(s.Q):
        lq = _levels_for_writer(s, q, boxes, 4)
        del lq[1]["boxes"][under[0]]
        del lq[1]["data"][under[0]]
        write_plotfile(plt_dir(tmp_path / "nest", 4, q), 2, [f"v_{m}" for m in range(s.Np_s)], s.time,
                       [0.0, 0.0], [1.0, 1.0], lq)
    with pytest.raises(G.AdgError, match="status 3"):
        r.ReadPlotFile(4, data_dir=str(tmp_path / "nest"))
    assert_same(before, snapshot(r))
    # variables with different boxes
    for q in range(s.Q):
        bq = boxes if q != 2 else [boxes[0], _split_x(boxes[1]), boxes[2]]
        write_plotfile(plt_dir(tmp_path / "mixed", 4, q), 2, [f"v_{m}" for m in range(s.Np_s)], s.time,
                       [0.0, 0.0], [1.0, 1.0], _levels_for_writer(s, q, bq, 4))
    with pytest.raises(G.AdgError, match="different boxes"):
        r.ReadPlotFile(4, data_dir=str(tmp_path / "mixed"))
    _assert_unchanged(r, before)
