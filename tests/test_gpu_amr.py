"""GPU parity of the multi-level (AMR) path against the CPU oracle:
identical refinement tags and box layouts at every step, and modal
coefficients of every level within 1e-12 relative after the stated steps.
Covers the coarse->fine projection (ghost fill and regrid), fine->coarse
average down, and the coarse-fine flux correction (reflux), batched over all
levels in one launch per stage."""
import numpy as np
import pytest

from parity import AMR_CASES, G, leaf_mass, make_gpu_amr, make_oracle_amr, rel_err

pytestmark = pytest.mark.gpu

RUN_TOL = 1e-12


def sync_initial_state(o, g):
    for l in range(o.num_levels()):
        g.set_U_w(o.get_uw(l), l)
    g.Dt = o.dt


@pytest.mark.parametrize("case", list(AMR_CASES))
def test_initial_hierarchy_matches(case):
    o = make_oracle_amr(case)
    g = make_gpu_amr(case)
    assert g.num_levels() == o.num_levels()
    for l in range(o.num_levels()):
        assert np.array_equal(g.boxes(l), o.boxes(l))
        assert rel_err(g.get_U_w(l), o.get_uw(l)) < 1e-13


@pytest.mark.parametrize("case,steps", [("kh_p3_amr", 9), ("kh_p2_amr_rect", 7), ("blast3d_p2_amr", 5)])
def test_amr_run_matches_oracle(case, steps):
    o = make_oracle_amr(case)
    g = make_gpu_amr(case)
    sync_initial_state(o, g)
    for s in range(steps):
        for l in range(min(o.num_levels(), g.num_levels())):
            to = o.tags(l)
            tg = g.tags(l)
            assert np.array_equal(to.astype(np.uint8), tg), f"tags differ on level {l} before step {s}"
        o.step()
        g.time_integration()
        assert g.num_levels() == o.num_levels(), f"step {s}"
        for l in range(o.num_levels()):
            assert np.array_equal(g.boxes(l), o.boxes(l)), f"boxes differ on level {l} after step {s}"
        assert abs(g.Dt - o.dt) / o.dt < 1e-12
    for l in range(o.num_levels()):
        assert rel_err(g.get_U_w(l), o.get_uw(l)) < RUN_TOL, f"level {l}"
    assert g.regrid_count() >= 2
    assert g.status() == 0


@pytest.mark.parametrize("quirk", [0, 1])
def test_amr_conserves_mass(quirk):
    g = make_gpu_amr("kh_p3_amr", quirk=quirk)
    D, P, n, hi, per, ic, extra, amr = AMR_CASES["kh_p3_amr"]

    def mass():
        nl = g.num_levels()
        return leaf_mass([g.get_U_w(l) for l in range(nl)], [g.boxes(l) for l in range(nl)], n, hi, 2)

    g.time_integration()  # first step regrids from the full-domain start
    m0 = mass()
    for _ in range(8):
        g.time_integration()
    assert abs(mass() - m0) < 1e-13 * abs(m0)


def test_amr_graph_replay_matches_stream_launches():
    a = make_gpu_amr("kh_p3_amr")
    b = make_gpu_amr("kh_p3_amr")
    a.advance(9, use_graph=True)
    b.advance(9, use_graph=False)
    assert a.num_levels() == b.num_levels()
    for l in range(a.num_levels()):
        assert np.array_equal(a.get_U_w(l), b.get_U_w(l))


def test_caller_supplied_layout_reproduces_the_run():
    """adg_set_layout: a context given another context's boxes and state (as
    a caller that owns the hierarchy, e.g. AMReX, would) takes the same
    steps bit for bit."""
    case = "kh_p3_amr"
    a = make_gpu_amr(case)
    for _ in range(6):
        a.time_integration()
    D, P, n, hi, per, ic, extra, amr = AMR_CASES[case]
    from parity import GPU_IC
    b = G.AmrDG(P=P, D=D)
    b.setGeometrySettings(prob_lo=(0, 0, 0), prob_hi=hi, n_cell=n, periodic=per, max_level=amr["max_level"],
                          max_grid=amr["max_grid"], blocking_factor=amr["blocking_factor"], dtn_regrid=0)
    b.setAmrSettings(tag_kind=amr["tag_kind"], tag_threshold=amr["tag_threshold"], reflux_box_quirk=1)
    b.settings(c_dt=0.5)
    b.init(G.Compressible_Euler().settings(GPU_IC[ic], **extra))
    b.set_layout([a.boxes(l) for l in range(a.num_levels())])
    assert b.num_levels() == a.num_levels()
    for l in range(a.num_levels()):
        assert np.array_equal(b.boxes(l), a.boxes(l))
        assert np.array_equal(b.level_cell_coords(l), a.level_cell_coords(l))
        b.set_U_w(a.get_U_w(l), l)
    b.Dt = a.Dt
    for _ in range(2):  # a's next regrid is due at its 8th step
        a.time_integration()
        b.time_integration()
    for l in range(a.num_levels()):
        assert np.array_equal(a.get_U_w(l), b.get_U_w(l)), l
    assert a.Dt == b.Dt


@pytest.mark.parametrize("case,kw", [("kh_p3_amr", {}),
                                     ("blast3d_p2_amr", dict(limiter_type="TVB", TVB_M=10.0, t_limit=1))])
def test_overlapped_regrid_matches_synchronous_regrid(case, kw):
    """A due regrid overlaps the step (the step runs on the current boxes while
    the host clusters, and is redone on the new boxes if they differ); the
    per-stage timing path regrids first.  Both take the same steps bit for
    bit, also when a forced layout makes the clustering change the boxes
    (the rollback)."""
    a = make_gpu_amr(case, **kw)
    b = make_gpu_amr(case, **kw)
    dtn = AMR_CASES[case][7]["dtn_regrid"]
    a.advance(dtn, use_graph=True)
    b.time_kernels(dtn)
    # a layout the clustering will not keep: level 0 and one small box per finer level
    D = a.D
    for s in (a, b):
        boxes = [s.boxes(0)]
        for l in range(1, s.num_levels()):
            lo = s.boxes(l)[0][:3]
            hi = lo.copy()
            hi[:D] = lo[:D] + AMR_CASES[case][7]["blocking_factor"] - 1
            box = np.concatenate([lo, hi])
            if l > 1:  # inside the level below with a one-cell margin (its coarse-fine ghosts)
                prev = boxes[l - 1][0]
                half = AMR_CASES[case][7]["blocking_factor"] // 2
                box[:D] = 2 * prev[:D] + half
                box[3:3 + D] = 2 * prev[:D] + 3 * half - 1
            boxes.append(box.reshape(1, 6))
        s.set_layout(boxes)
    a.advance(2 * dtn, use_graph=True)
    b.time_kernels(2 * dtn)
    assert a.num_levels() == b.num_levels()
    for l in range(a.num_levels()):
        assert np.array_equal(a.boxes(l), b.boxes(l))
        assert np.array_equal(a.get_U_w(l), b.get_U_w(l)), l
    assert a.time == b.time and a.Dt == b.Dt
    assert a.regrid_count() == b.regrid_count()
    assert a.status() == 0 and b.status() == 0


def test_host_round_trip_every_step_matches_device_resident_run():
    """The end-to-end pattern on three levels: every level copied in from
    page-locked host memory (queued), one step, every level copied out, one
    synchronisation.  Setting the coarse levels leaves the finer levels'
    ghosts stale; the one deferred fill before the step reproduces what the
    previous step's own fill left, so the run equals the device-resident one
    bit for bit (layouts included)."""
    a = make_gpu_amr("kh_p3_amr")
    b = make_gpu_amr("kh_p3_amr")
    a.advance(2)
    b.advance(2)
    for _ in range(6):
        nl = b.num_levels()
        pins = [G.PinnedArray((b.level_cells(l), b.Q, b.Np_s)) for l in range(nl)]
        for l, p in enumerate(pins):
            b.get_U_w_async(p, l)
        b.synchronize()
        for l, p in enumerate(pins):
            b.set_U_w_async(p, l)
        b.advance(1)
        a.advance(1)
        b.synchronize()
        for p in pins:
            p.free()
    assert a.num_levels() == b.num_levels()
    for l in range(a.num_levels()):
        assert np.array_equal(a.boxes(l), b.boxes(l))
        assert np.array_equal(a.get_U_w(l), b.get_U_w(l))
