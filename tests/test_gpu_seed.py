"""Learned predictor seed: the GPU FP32 training kernels against a float64
restatement (forward, gradients, finite differences), training on Picard
data, the residual fallback, and what the trained network buys over the
method without it (same single sweep from the reference's initial guess)."""
import numpy as np
import pytest

import mlp_ref
from parity import G, make_gpu, rel_err

pytestmark = pytest.mark.gpu


def _layers64(seed):
    return [(W.astype(np.float64), b.astype(np.float64)) for W, b in seed.weights()]


def test_forward_matches_float64_restatement():
    s = G.PredictorSeed(2, 3, hidden=64, rng_seed=7)
    rng = np.random.default_rng(0)
    X = rng.standard_normal((300, s.n_in)).astype(np.float32)
    Y = s.forward(X)
    Yr, _, _ = mlp_ref.forward(_layers64(s), X.astype(np.float64))
    assert np.max(np.abs(Y - Yr)) < 1e-4 * max(1.0, np.max(np.abs(Yr)))


def test_gradients_match_float64_restatement_and_finite_differences():
    s = G.PredictorSeed(2, 1, hidden=32, rng_seed=11)
    rng = np.random.default_rng(1)
    X = rng.standard_normal((257, s.n_in)).astype(np.float32)
    T = rng.standard_normal((257, s.n_out)).astype(np.float32)
    g, loss = s.gradients(X, T)
    layers = _layers64(s)
    lr, gr = mlp_ref.loss_and_grads(layers, X.astype(np.float64), T.astype(np.float64))
    gref = mlp_ref.flatten(gr)
    assert abs(loss - lr) < 1e-5 * lr
    assert np.max(np.abs(g - gref)) < 1e-4 * np.max(np.abs(gref))
    # the float64 restatement itself against central differences
    for (li, which, idx) in [(0, 0, (3, 5)), (1, 1, (7,)), (3, 0, (10, 2)), (2, 0, (0, 31))]:
        W, b = layers[li]
        arr = W if which == 0 else b
        h = 1e-6
        old = arr[idx]
        arr[idx] = old + h
        lp, _ = mlp_ref.loss_and_grads(layers, X.astype(np.float64), T.astype(np.float64))
        arr[idx] = old - h
        lm, _ = mlp_ref.loss_and_grads(layers, X.astype(np.float64), T.astype(np.float64))
        arr[idx] = old
        fd = (lp - lm) / (2 * h)
        an = gr[li][which][idx]
        assert abs(fd - an) < 1e-6 * max(1.0, abs(an)) + 1e-9


def _kh(n=64, seed=12345, amp=1e-3, **kw):
    s = G.AmrDG(P=3, D=2)
    s.setGeometrySettings(prob_lo=(0, 0), prob_hi=(1, 1), n_cell=(n, n))
    s.settings(c_dt=0.5, **kw)
    s.init(G.Compressible_Euler().settings("kh_noise", seed=seed, noise_amp=amp))
    return s


_SEED = {}


def _trained_seed():
    """Seed trained on Picard pairs (converged predictor, 8 sweeps) of KH runs
    with perturbed initial conditions; cached for the module."""
    if "s" not in _SEED:
        seed = G.PredictorSeed(2, 3, hidden=128, rng_seed=5)
        for ic_seed in (1, 2, 3, 4):
            s = _kh(seed=ic_seed, amp=1e-3 * ic_seed)
            for k in range(24):
                if k % 2 == 0:
                    seed.collect(s, target_sweeps=8)
                s.time_integration()
        l0 = seed.train(1, batch=4096, lr=1e-3)
        l1 = seed.train(60, batch=4096, lr=1e-3)
        _SEED["s"] = (seed, l0, l1)
    return _SEED["s"]


def _predictor(sim):
    torch = pytest.importorskip("torch")
    n = sim.level_cells(0)
    buf = torch.zeros(n * sim.Q * sim.Np_st, dtype=torch.float64, device="cuda")
    sim.predictor(0, buf.data_ptr())
    torch.cuda.synchronize()
    return buf.cpu().numpy().reshape(n, sim.Q, sim.Np_st)


def _state_after(steps, seed=42):
    s = _kh(seed=seed)
    for _ in range(steps):
        s.time_integration()
    return s.get_U_w(), s.Dt


def _err(H, Hc, U):
    scale = np.max(np.abs(U[:, :, 0]), axis=0)
    return max(float(np.max(np.abs(H[:, q] - Hc[:, q])) / scale[q]) for q in (0, 1, 3))


def test_training_reduces_loss_and_seed_beats_unseeded_single_sweep():
    seed, l0, l1 = _trained_seed()
    assert l1 < 0.1 * l0
    U, dt = _state_after(15)

    def run(**kw):
        s = _kh(**kw)
        s.set_U_w(U)
        s.Dt = dt
        return s

    Hc = _predictor(run(picard_sweeps=10))  # converged Picard
    e_plain = _err(_predictor(run()), Hc, U)
    e_one = _err(_predictor(run(picard_sweeps=1)), Hc, U)
    sd = run()
    seed.attach(sd, mode=1, sweeps=1, tol=1e9)
    e_seed1 = _err(_predictor(sd), Hc, U)
    sd2 = run()
    seed.attach(sd2, mode=2, sweeps=2, tol=1e9)
    e_seed2_f32 = _err(_predictor(sd2), Hc, U)
    # what the network buys: one sweep from the seed against one sweep from
    # the reference's initial guess, and two FP32 sweeps from the seed
    # against the reference's three FP64 sweeps
    assert e_seed1 < 0.1 * e_one, (e_seed1, e_one)
    assert e_seed2_f32 < 10 * e_plain, (e_seed2_f32, e_plain)


def test_training_is_reproducible_bit_for_bit():
    """Collection, standardisation and training reduce in a fixed order
    (split-K slices and column-sum blocks added in order, no atomics on the
    parameters' path): two seeds trained alike on the same pairs end with
    the same parameters, bit for bit."""
    params = []
    for _ in range(2):
        seed = G.PredictorSeed(2, 3, hidden=128, rng_seed=9)
        s = _kh(seed=6, amp=2e-3)
        for k in range(6):
            if k % 2 == 0:
                seed.collect(s, target_sweeps=8)
            s.time_integration()
        seed.train(3, batch=4096, lr=1e-3)
        params.append(np.asarray(seed.get_params()).copy())
    assert np.array_equal(params[0], params[1])


def test_zero_tolerance_falls_back_everywhere_to_the_plain_path():
    seed, _, _ = _trained_seed()
    a = _kh(n=32, seed=9)
    b = _kh(n=32, seed=9)
    seed.attach(b, mode=1, sweeps=1, tol=1e-300)
    for _ in range(3):
        a.time_integration()
        b.time_integration()
    assert np.array_equal(a.get_U_w(), b.get_U_w())
    fb, n = G.seed_stats(b)
    assert fb == n == 3 * 32 * 32


def test_fp32_path_fallback_is_the_fp64_picard_with_split_traces():
    """Mode 2 with a zero tolerance: every element takes the FP64 Picard
    fallback, whose final stage (volume term and split face traces, H = U +
    FP32 change) is the seeded path's; against the plain FP64 path it
    differs only by the FP32 rounding of the change of H."""
    seed, _, _ = _trained_seed()
    a = _kh(n=32, seed=9)
    b = _kh(n=32, seed=9)
    seed.attach(b, mode=2, sweeps=2, tol=1e-300)
    for _ in range(3):
        a.time_integration()
        b.time_integration()
    fb, n = G.seed_stats(b)
    assert fb == n == 3 * 32 * 32
    assert b.status() == 0
    ua, ub = a.get_U_w(), b.get_U_w()
    # relative to each variable's largest cell mean (the y momentum of this
    # flow is only its 1e-3 noise, so its bound is the loosest)
    scale = np.max(np.abs(ua[:, :, 0]), axis=0)
    err = np.max(np.abs(ua - ub), axis=(0, 2)) / scale
    assert np.all(err < 1e-7), err
    assert np.any(ua != ub)  # the split path ran (not bitwise the plain one)


def test_fp32_path_conserves_mass_and_tracks_the_plain_path():
    """Mode 2 with its working tolerance on a periodic domain: the mean
    density is conserved to rounding (the split numerical flux is one value
    per face, shared by both sides), and the state stays closer to the plain
    FP64 path (three sweeps) than two FP64 sweeps without the seed do."""
    seed, _, _ = _trained_seed()
    a = _kh(seed=5)
    b = _kh(seed=5)
    c = _kh(seed=5, picard_sweeps=2)
    seed.attach(b, mode=2, sweeps=2, tol=1e-3)
    m0 = b.get_U_w()[:, 0, 0].sum()
    for _ in range(10):
        for s in (a, b, c):
            s.time_integration()
    ub = b.get_U_w()
    assert abs(ub[:, 0, 0].sum() - m0) < 1e-12 * abs(m0)
    ua = a.get_U_w()
    scale = np.max(np.abs(ua[:, :, 0]), axis=0)

    def dist(u):
        return float(np.max(np.max(np.abs(u - ua), axis=(0, 2)) / scale))

    assert dist(ub) < 0.1 * dist(c.get_U_w()), (dist(ub), dist(c.get_U_w()))


@pytest.mark.parametrize("quirk", [0, 1])
def test_fp32_path_on_amr_conserves_mass_and_tracks_the_plain_path(quirk):
    """Mode 2 on the three-level KH hierarchy: the split numerical flux also
    feeds the coarse-fine corrections (its face moments), so the leaf mass is
    conserved to rounding; level 0 (the whole field after the average down)
    stays closer to the plain FP64 run than two FP64 sweeps without the seed."""
    from parity import AMR_CASES, leaf_mass, make_gpu_amr
    seed, _, _ = _trained_seed()
    D, P, n, hi, per, ic, extra, amr = AMR_CASES["kh_p3_amr"]
    a = make_gpu_amr("kh_p3_amr", quirk=quirk)
    b = make_gpu_amr("kh_p3_amr", quirk=quirk)
    c = make_gpu_amr("kh_p3_amr", quirk=quirk, picard_sweeps=2)
    seed.attach(b, mode=2, sweeps=2, tol=1e-3)

    def mass(g):
        nl = g.num_levels()
        return leaf_mass([g.get_U_w(l) for l in range(nl)], [g.boxes(l) for l in range(nl)], n, hi, 2)

    for g in (a, b, c):
        g.time_integration()  # the first step regrids from the full-domain start
    m0 = mass(b)
    for _ in range(8):
        for g in (a, b, c):
            g.time_integration()
    assert b.num_levels() == 3 and b.status() == 0
    assert abs(mass(b) - m0) < 1e-13 * abs(m0)
    ua = a.get_U_w(0)
    scale = np.max(np.abs(ua[:, :, 0]), axis=0)

    def dist(g):
        return float(np.max(np.max(np.abs(g.get_U_w(0) - ua), axis=(0, 2)) / scale))

    assert dist(b) < 0.1 * dist(c), (dist(b), dist(c))


@pytest.mark.parametrize("case", ["vortex_p1", "vortex_p2", "kh_p3", "vortex_p3_outflow", "blast3d_p1_per",
                                  "blast3d_p2"])
def test_fp32_path_runs_on_every_configuration(case):
    """Mode 2 on every compiled (D, P), with an untrained network (its
    corrections stay near W U, so the three FP32 sweeps carry the predictor):
    the split final stage, split traces and split numerical flux give a
    finite state, conserve mass on periodic domains, and stay as close to a
    converged Picard run (8 FP64 sweeps) as the plain path's P sweeps from
    the reference's initial guess do (closer where P < 3)."""
    from parity import CASES
    per = CASES[case][5]
    a = make_gpu(case)                   # plain: P sweeps
    c = make_gpu(case, picard_sweeps=8)  # converged predictor
    b = make_gpu(case)
    seed = G.PredictorSeed(b.D, b.P, hidden=128, rng_seed=3)
    seed.attach(b, mode=2, sweeps=3, tol=1e9)
    m0 = b.get_U_w()[:, 0, 0].sum()
    for _ in range(3):
        for s in (a, b, c):
            s.time_integration()
    ua, ub, uc = a.get_U_w(), b.get_U_w(), c.get_U_w()
    assert np.all(np.isfinite(ub)) and b.status() == 0
    if all(per[:b.D]):
        assert abs(ub[:, 0, 0].sum() - m0) < 1e-12 * abs(m0)
    scale = np.max(np.abs(uc[:, :, 0]))  # largest cell mean of any variable
    d_seed = np.max(np.abs(ub - uc)) / scale
    d_plain = np.max(np.abs(ua - uc)) / scale
    assert d_seed <= 2.0 * d_plain + 1e-9, (d_seed, d_plain)


def _seed_correction(H, U, s, seed):
    """(H - W U) / (rho_mean Dt/dx): the network's share of the seed."""
    import oracle_ffi as O
    W = O.matrix(2, 3, "Mk_h_w_inv") @ O.matrix(2, 3, "Mk_pred")  # a 0/1 selection
    scale = U[:, 0, 0] * (s.Dt * 64.0)
    return (H - np.einsum("kn,eqn->eqk", W, U)) / scale[:, None, None]


def test_tensor_core_seed_matches_float64_restatement():
    """The fused tcgen05 inference (TF32 operands, FP32 accumulation) and the
    SIMT path (FP32) against the float64 restatement of features, network
    and assembly, on the same state."""
    torch = pytest.importorskip("torch")
    seed, _, _ = _trained_seed()
    s = _kh(seed=31)
    for _ in range(3):
        s.time_integration()
    seed.attach(s, mode=2, sweeps=2, tol=1e-3)
    U = s.get_U_w()
    n, Q, Ns = U.shape
    Nst = s.Np_st
    out = {}
    for path in (0, 1):
        b = torch.full((n * Q * Nst,), float("nan"), dtype=torch.float64, device="cuda")
        s.seed_infer(b.data_ptr(), path)
        torch.cuda.synchronize()
        out[path] = b.cpu().numpy().reshape(n, Q, Nst)
    assert s.status() == 0
    p = seed.get_params()
    nw, _ = seed.num_params()
    nin, nout = seed.n_in, seed.n_out
    x_mean, x_istd = p[nw:nw + nin], p[nw + nin:nw + 2 * nin]
    y_mean, y_std = p[nw + 2 * nin:nw + 2 * nin + nout], p[nw + 2 * nin + nout:]
    X = np.concatenate([(U.reshape(n, -1) / U[:, :1, 0]).astype(np.float32),
                        np.full((n, 1), s.Dt * 64.0, dtype=np.float32)], axis=1)
    X = (X - x_mean) * x_istd
    layers = _layers64(seed)
    Y, _, _ = mlp_ref.forward(layers, X.astype(np.float64))
    # compare in the network's standardised output space
    y0 = (_seed_correction(out[0], U, s, seed).reshape(n, -1) - y_mean) / y_std
    y1 = (_seed_correction(out[1], U, s, seed).reshape(n, -1) - y_mean) / y_std
    assert np.all(np.isfinite(y0)) and np.all(np.isfinite(y1))
    rms = np.sqrt(np.mean(Y ** 2))

    def err(a, b):
        return np.max(np.abs(a - b)) / np.max(np.abs(Y)), np.sqrt(np.mean((a - b) ** 2)) / rms

    # SIMT path: FP32 throughout
    e_max, e_rms = err(y0, Y)
    assert e_max < 1e-5 and e_rms < 1e-5, (e_max, e_rms)
    # tensor cores: operands rounded to TF32 (10 mantissa bits, nearest) and
    # FP32 accumulation; the restatement that rounds its operands likewise
    # leaves FP32 rounding and the odd activation that lands on the other
    # side of a TF32 rounding boundary (one TF32 ulp, 1e-3 of it)
    e_max, e_rms = err(y1, mlp_ref.forward_tf32(layers, X.astype(np.float64), "rna"))
    assert e_max < 3e-3 and e_rms < 5e-4, (e_max, e_rms)
    # and what TF32 costs against FP32: about 1e-3 of the outputs
    e_max, e_rms = err(y1, Y)
    assert e_max < 1e-2 and e_rms < 3e-3, (e_max, e_rms)


@pytest.mark.parametrize("case", ["vortex_p1", "vortex_p2", "blast3d_p1_per", "blast3d_p2"])
def test_tensor_core_seed_matches_simt_path_on_every_configuration(case):
    """The fused tcgen05 inference against the SIMT FP32 path on the other
    compiled (D, P): output widths that are not a multiple of four (D = 3),
    a partial last tile (192 elements) and the FP64 output.  Both paths give
    H = W U + rho_mean Dt/dx Y(x); their network parts H - W U differ by the
    TF32 rounding of the operands only."""
    torch = pytest.importorskip("torch")
    import oracle_ffi as O
    s = make_gpu(case)
    seed = G.PredictorSeed(s.D, s.P, hidden=128, rng_seed=19)
    seed.attach(s, mode=2, sweeps=2, tol=1e-3)
    s.time_integration()
    U = s.get_U_w()
    n, Q, Ns = U.shape
    Nst = s.Np_st
    out = {}
    for path in (0, 1):
        b = torch.full((n * Q * Nst,), float("nan"), dtype=torch.float64, device="cuda")
        s.seed_infer(b.data_ptr(), path)
        torch.cuda.synchronize()
        out[path] = b.cpu().numpy().reshape(n, Q, Nst)
    assert s.status() == 0
    assert np.all(np.isfinite(out[0])) and np.all(np.isfinite(out[1]))
    W = O.matrix(s.D, s.P, "Mk_h_w_inv") @ O.matrix(s.D, s.P, "Mk_pred")  # a 0/1 selection
    WU = np.einsum("kn,eqn->eqk", W, U)
    net0, net1 = out[0] - WU, out[1] - WU
    scale = np.max(np.abs(net0))
    assert scale > 0.0
    e_max = np.max(np.abs(net1 - net0)) / scale
    e_rms = np.sqrt(np.mean((net1 - net0) ** 2)) / np.sqrt(np.mean(net0 ** 2))
    assert e_max < 1e-2 and e_rms < 3e-3, (e_max, e_rms)


@pytest.mark.parametrize("mode", [1, 2])
def test_seeded_run_stays_close_to_plain_run(mode):
    seed, _, _ = _trained_seed()
    a = _kh(seed=77)
    b = _kh(seed=77)
    seed.attach(b, mode=mode, sweeps=2, tol=1e-3)
    for _ in range(10):
        a.time_integration()
        b.time_integration()
    ua, ub = a.get_U_w(), b.get_U_w()
    # density and energy, relative to their largest cell means (the
    # y-momentum of this flow is ~1e-2 and is checked against the density scale)
    for q in range(4):
        scale = np.max(np.abs(ua[:, 0 if q == 2 else q, 0]))
        assert np.max(np.abs(ub[:, q] - ua[:, q])) < 1e-5 * scale, q
    assert b.status() == 0
