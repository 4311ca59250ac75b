"""L2ProjInterp transfer entry points on the GPU (AmrDG_Interpolater.tpp:283-398):
adg_interp_scatter / adg_interp_gather on caller batches against the
reference's matrices as the oracle builds them (Minv, P_cf, P_fc), the
gather-after-scatter identity (AmrDG_Level.tpp:96-98), device-memory calls,
and adg_average_down / adg_fill_ghosts on a context's own layout."""
import ctypes

import numpy as np
import pytest

import oracle_ffi as O
from parity import CASES, G, make_gpu, make_gpu_amr

pytestmark = pytest.mark.gpu

CONFIGS = {(2, 1): "vortex_p1", (2, 2): "vortex_p2", (2, 3): "kh_p3", (3, 1): "blast3d_p1_per", (3, 2): "blast3d_p2"}


def _sim(D, P):
    return make_gpu(CONFIGS[(D, P)])


@pytest.mark.parametrize("D,P", list(CONFIGS))
def test_scatter_and_gather_match_the_reference_matrices(D, P):
    s = _sim(D, P)
    Q, Ns, nov = s.Q, s.Np_s, 1 << D
    rng = np.random.default_rng(D * 10 + P)
    n = 37
    coarse = rng.standard_normal((n, Q, Ns))
    child = rng.integers(0, nov, n).astype(np.int8)
    Minv = O.matrix(D, P, "Minv")
    Pcf = [O.matrix(D, P, "P_cf", l) for l in range(nov)]
    Pfc = [O.matrix(D, P, "P_fc", l) for l in range(nov)]
    fine = s.amr_scatter(coarse, child)
    want = np.stack([(Minv @ Pcf[child[i]] @ coarse[i].T).T for i in range(n)])
    assert np.max(np.abs(fine - want)) < 1e-13 * np.max(np.abs(want))
    kids = rng.standard_normal((n, nov, Q, Ns))
    got = s.amr_gather(kids)
    want = np.stack([(Minv @ sum(Pfc[l] @ kids[i, l].T for l in range(nov))).T / nov for i in range(n)])
    assert np.max(np.abs(got - want)) < 1e-13 * np.max(np.abs(want))


@pytest.mark.parametrize("D,P", list(CONFIGS))
def test_gather_after_scatter_is_the_identity(D, P):
    s = _sim(D, P)
    nov = 1 << D
    rng = np.random.default_rng(7)
    coarse = rng.standard_normal((11, s.Q, s.Np_s))
    rep = np.repeat(coarse, nov, axis=0)
    child = np.tile(np.arange(nov, dtype=np.int8), 11)
    fine = s.amr_scatter(rep, child).reshape(11, nov, s.Q, s.Np_s)
    back = s.amr_gather(fine)
    assert np.max(np.abs(back - coarse)) < 1e-13 * np.max(np.abs(coarse))


def test_device_memory_batches_match_host_batches():
    torch = pytest.importorskip("torch")
    s = _sim(2, 3)
    Q, Ns = s.Q, s.Np_s
    rng = np.random.default_rng(3)
    coarse = rng.standard_normal((19, Q, Ns))
    child = rng.integers(0, 4, 19).astype(np.int8)
    host = s.amr_scatter(coarse, child)
    c_dev = torch.from_numpy(coarse).cuda()
    ch_dev = torch.from_numpy(child).cuda()
    f_dev = torch.empty_like(c_dev)
    L = s._L
    assert L.adg_interp_scatter(s.ctx, c_dev.data_ptr(), ch_dev.data_ptr(), 19, f_dev.data_ptr(), 1) == 0
    assert np.array_equal(f_dev.cpu().numpy(), host)
    kids = torch.from_numpy(rng.standard_normal((19, 4, Q, Ns))).cuda()
    out = torch.empty_like(c_dev)
    assert L.adg_interp_gather(s.ctx, kids.data_ptr(), 19, out.data_ptr(), 1) == 0
    assert np.array_equal(out.cpu().numpy(), s.amr_gather(kids.cpu().numpy()))


def test_bad_arguments_are_rejected():
    s = _sim(2, 3)
    with pytest.raises(G.AdgError, match="child index"):
        s.amr_scatter(np.zeros((2, s.Q, s.Np_s)), np.array([0, 4], dtype=np.int8))
    c = np.zeros((1, s.Q, s.Np_s))
    assert s._L.adg_interp_scatter(s.ctx, c.ctypes.data, c.ctypes.data, 1, c.ctypes.data, 5) == 1
    assert s._L.adg_interp_gather(s.ctx, None, 3, None, 0) == 1
    assert s._L.adg_interp_gather(s.ctx, None, 0, None, 0) == 0  # an empty batch is a no-op


def _children_of(s, l):
    """[covered cells of level l, 2^D] indices into level l+1's state, and the covered cells."""
    D = s.D
    fine = {tuple(c[:D]): i for i, c in enumerate(s.level_cell_coords(l + 1))}
    rows, cells = [], []
    for i, c in enumerate(s.level_cell_coords(l)):
        kids = []
        for k in range(1 << D):
            f = tuple(2 * c[d] + ((k >> (D - 1 - d)) & 1) for d in range(D))
            kids.append(fine.get(f, -1))
        if all(x >= 0 for x in kids):
            rows.append(kids)
            cells.append(i)
    return np.array(rows), np.array(cells)


def test_average_down_is_the_gather_of_the_children():
    s = make_gpu_amr("kh_p3_amr")
    s.advance(4)
    assert s.num_levels() == 3
    rng = np.random.default_rng(5)
    for l in (2, 1):  # perturb the finer levels, then average down on the layout
        u = s.get_U_w(l)
        s.set_U_w(u * (1.0 + 1e-3 * rng.standard_normal(u.shape)), l)
    s.average_down()
    for l in (1, 0):
        kids, cells = _children_of(s, l)
        assert len(cells) > 0
        uf = s.get_U_w(l + 1)
        want = s.amr_gather(uf[kids])
        assert np.array_equal(s.get_U_w(l)[cells], want)


def test_fill_ghosts_is_idempotent_within_a_step():
    a = make_gpu_amr("kh_p3_amr")
    b = make_gpu_amr("kh_p3_amr")
    a.advance(5)
    b.advance(5)
    a.fill_ghosts()  # the step already left the ghosts filled
    a.average_down()  # and the covered cells averaged
    a.advance(2)
    b.advance(2)
    for l in range(a.num_levels()):
        assert np.array_equal(a.get_U_w(l), b.get_U_w(l))
