"""Step readback (adg_set_readback): registered page-locked host buffers
receive every level's state at the end of each step of adg_advance, copied
beside the step's tail.  The buffers must equal adg_get_state after every
step bit for bit, on one level and on AMR layouts that regrid (graph and
direct launches), with buffers sized for the level's largest layout and with
tight ones that a regrid outgrows (the registration is then dropped); the
results of the steps do not change."""
import ctypes

import numpy as np
import pytest

from parity import AMR_CASES, G, make_gpu, make_gpu_amr

pytestmark = pytest.mark.gpu


def _capacity(s, case, lev, tight):
    if tight:
        return s.level_cells(lev)
    n = AMR_CASES[case][2]
    full = 1
    for d in range(s.D):
        full *= n[d] << lev
    return full


def _run(s, case, steps, use_graph, tight):
    """Steps with readback on every level; returns how often a registration
    was found dropped (a level grown past its buffer or a new level)."""
    bufs = {}

    def register(lev):
        b = G.PinnedArray((_capacity(s, case, lev, tight), s.Q, s.Np_s))
        s.set_readback(b, lev)
        bufs[lev] = b

    for lev in range(s.num_levels()):
        register(lev)
    dropped = 0
    for _ in range(steps):
        for b in bufs.values():
            b.array[:] = np.nan
        s.advance(1, use_graph=use_graph)
        s.synchronize()
        for lev in range(s.num_levels()):
            u = s.get_U_w(lev)
            if lev in bufs and s.readback_active(lev):
                got = bufs[lev].array[: u.shape[0]]
                assert np.array_equal(got, u), lev
                assert np.all(np.isnan(bufs[lev].array[u.shape[0]:]))  # nothing past the level's cells
            else:
                assert lev not in bufs or s.level_cells(lev) > bufs[lev].array.shape[0]
                dropped += 1
                if lev in bufs:
                    bufs.pop(lev).free()  # dropped: the library no longer writes it
                register(lev)
        for lev in [l for l in bufs if l >= s.num_levels()]:
            bufs.pop(lev).free()  # a level the layout no longer has: dropped too
    for lev in range(s.num_levels()):
        if lev in bufs:
            s.set_readback(None, lev)
    s.synchronize()
    for b in bufs.values():
        b.free()
    return dropped


@pytest.mark.parametrize("case,use_graph,tight", [("kh_p3_amr", True, False), ("kh_p3_amr", False, False),
                                                  ("kh_p3_amr", True, True), ("kh_p2_amr_rect", True, True)])
def test_readback_equals_get_state_after_every_step_amr(case, use_graph, tight):
    a = make_gpu_amr(case)
    b = make_gpu_amr(case)
    dropped = _run(a, case, 12, use_graph, tight)
    if not tight:
        assert dropped == 0  # buffers for the largest layout never drop
    b.advance(12, use_graph=use_graph)  # the same steps without readback
    assert a.num_levels() == b.num_levels()
    for lev in range(a.num_levels()):
        assert np.array_equal(a.get_U_w(lev), b.get_U_w(lev)), lev
    assert a.status() == 0


@pytest.mark.parametrize("t_limit", [1, 2])
def test_readback_after_the_limiter(t_limit):
    """With the TVB limiter the finest level's last writer in a step is the
    limiter (every step, or every other step, which runs without the graph):
    the readback holds the limited state."""
    case = "blast3d_p2_amr"
    kw = dict(limiter_type="TVB", TVB_M=0.0, t_limit=t_limit)
    a = make_gpu_amr(case, **kw)
    b = make_gpu_amr(case, **kw)
    _run(a, case, 6, True, False)
    b.advance(6)
    for lev in range(a.num_levels()):
        assert np.array_equal(a.get_U_w(lev), b.get_U_w(lev)), lev
    assert a.status() == 0


def test_readback_single_level():
    a = make_gpu("kh_p3")
    b = make_gpu("kh_p3")
    assert _run(a, None, 5, True, True) == 0
    b.advance(5)
    assert np.array_equal(a.get_U_w(0), b.get_U_w(0))


def test_readback_argument_checks():
    s = make_gpu("kh_p3")
    n = s.level_cells(0)
    L, ctx = s._L, s.ctx
    pageable = np.zeros((n, s.Q, s.Np_s))
    assert L.adg_set_readback(ctx, 0, pageable.ctypes.data, n) != 0  # not page-locked
    p = G.PinnedArray((n, s.Q, s.Np_s))
    assert L.adg_set_readback(ctx, 0, p.array.ctypes.data, n - 1) != 0  # smaller than the level
    assert L.adg_set_readback(ctx, 1, p.array.ctypes.data, n) != 0  # no such level
    v = ctypes.c_int(7)
    assert L.adg_readback_active(ctx, 0, ctypes.byref(v)) == 0 and v.value == 0
    assert L.adg_set_readback(ctx, 0, p.array.ctypes.data, n) == 0
    assert s.readback_active(0)
    s.set_readback(None, 0)
    assert not s.readback_active(0)
    p.free()


def _packed(s):
    return np.concatenate([s.get_U_w(lev) for lev in range(s.num_levels())])


@pytest.mark.parametrize("tight", [False, True])
def test_packed_readback_and_packed_copies(tight):
    """ADG_ALL_LEVELS: one copy of every level packed in level order in and
    out, and one packed readback buffer filled level by level inside the
    step."""
    case = "kh_p3_amr"
    s = make_gpu_amr(case)
    ref = make_gpu_amr(case)
    L, ctx = s._L, s.ctx
    Q, Nps = s.Q, s.Np_s

    def cap():
        if tight:
            return sum(s.level_cells(lev) for lev in range(s.num_levels()))
        return sum(_capacity(s, case, lev, False) for lev in range(AMR_CASES[case][7]["max_level"] + 1))

    buf = G.PinnedArray((cap(), Q, Nps))
    assert L.adg_set_readback(ctx, G.ADG_ALL_LEVELS, buf.array.ctypes.data, buf.array.shape[0]) == 0
    v = ctypes.c_int()
    drops = 0
    for _ in range(12):
        buf.array[:] = np.nan
        # the packed state goes in with one copy (a no-op round trip here)
        n = sum(s.level_cells(lev) for lev in range(s.num_levels()))
        packed = np.ascontiguousarray(_packed(s))
        assert packed.shape[0] == n
        assert L.adg_set_state(ctx, G.ADG_ALL_LEVELS, packed.ctypes.data, G.ADG_MEM_HOST) == 0
        s.advance(1)
        ref.advance(1)
        s.synchronize()
        want = _packed(s)
        got = np.empty_like(want)
        assert L.adg_get_state(ctx, G.ADG_ALL_LEVELS, got.ctypes.data, G.ADG_MEM_HOST) == 0
        assert np.array_equal(got, want)
        assert L.adg_readback_active(ctx, G.ADG_ALL_LEVELS, ctypes.byref(v)) == 0
        if v.value:
            assert np.array_equal(buf.array[: want.shape[0]], want)
            assert np.all(np.isnan(buf.array[want.shape[0]:]))
        else:
            assert tight and want.shape[0] > buf.array.shape[0]
            drops += 1
            buf.free()
            buf = G.PinnedArray((cap(), Q, Nps))
            assert L.adg_set_readback(ctx, G.ADG_ALL_LEVELS, buf.array.ctypes.data, buf.array.shape[0]) == 0
    if not tight:
        assert drops == 0
    assert L.adg_set_readback(ctx, G.ADG_ALL_LEVELS, None, 0) == 0
    s.synchronize()
    buf.free()
    # the packed round trips and the readback left the steps unchanged
    for lev in range(ref.num_levels()):
        assert np.array_equal(s.get_U_w(lev), ref.get_U_w(lev)), lev
