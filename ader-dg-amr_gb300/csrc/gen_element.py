#!/usr/bin/env python3
"""Build-time generator of the per-element FP64 operators of the ADER-DG path.

For one (D, P) it computes every element matrix the method needs, exactly
(rational arithmetic on the double-valued Gauss-Legendre tables, one rounding
at the end), factorises each operator into a chain of sparse tensor-product
stages (sum factorisation over the total-degree Legendre basis), checks every
chain against the dense operator, and emits straight-line CUDA device code in
which every structural zero is skipped and every coefficient is an exact
double literal.  One thread of a kernel runs one operator on one
(element, conserved variable) column, so all 32 lanes of a warp issue the
same FP64 instruction stream.

Operators (reference definitions, Source/NumericalMethod/AmrDG/...):
  V            space-time modes -> space-time GL points   (AmrDG_ElementMatrix.tpp:7-19)
  Vinv         unweighted pseudo-inverse of V              (AmrDG_ElementMatrix.tpp:21-25)
  Mk_h_w, Mk_pred, Sk_pred[d]                               (AmrDG_ElementMatrix.tpp:32-58)
  Sk_corr[d], Mkbdm/Mkbdp[d], quadmat                       (AmrDG_ElementMatrix.tpp:63-197)
  P_cf, P_fc, Minv                                          (AmrDG_Interpolater.tpp:157-231)
  P_flux_fc_low/high                                        (AmrDG_Interpolater.tpp:85-155)
Predictor update (AmrDG.tpp:744-827) is folded as
  H_w <- W U_w - sum_d (Dt/dx_d) A_d F_d,  W = Mk_h_w^-1 Mk_pred,
  A_d = Mk_h_w^-1 Sk_pred[d] Vinv = C_d V^T,  C_d = Mk_h_w^-1 Sk_pred[d] (V^T V)^-1.
"""
import argparse
import itertools
import math
import os
import sys
from fractions import Fraction

# ----------------------------------------------------------------------------
# Gauss-Legendre rule, same arithmetic as the reference (AmrDG.h:151-318)
# ----------------------------------------------------------------------------


def cx_cos(x):
    result, term = 1.0, 1.0
    for n in range(1, 31):
        term *= -x * x / ((2 * n - 1) * (2 * n))
        result += term
    return result


def cx_legendre(n, x):
    if n == 0:
        return 1.0
    if n == 1:
        return x
    p0, p1 = 1.0, x
    for k in range(2, n + 1):
        p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k
        p0, p1 = p1, p2
    return p1


def cx_dlegendre(n, x):
    if n == 0:
        return 0.0
    p0, p1, dp1 = 1.0, x, 1.0
    for k in range(2, n + 1):
        p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k
        dp2 = k * p1 + x * dp1
        p0, p1, dp1 = p1, p2, dp2
    return dp1


def gl_rule(P):
    N = P + 1
    nodes = [0.0] * N
    idx = 0
    for i in range(1, N // 2 + 1):
        theta = 3.14159265358979323846 * (i - 0.25) / (N + 0.5)
        x = cx_cos(theta)
        for _ in range(30):
            dx = cx_legendre(N, x) / cx_dlegendre(N, x)
            x -= dx
            if abs(dx) < 1e-16:
                break
        nodes[idx] = x
        nodes[idx + 1] = -x
        idx += 2
    if N % 2:
        nodes[idx] = 0.0
    weights = []
    for q in range(N):
        x = nodes[q]
        dp = cx_dlegendre(N, x)
        weights.append(2.0 / ((1.0 - x * x) * dp * dp))
    return nodes, weights


def multi_index(P, Dtot):
    out = []

    def rec(prefix, left, depth):
        if depth == Dtot:
            out.append(tuple(prefix))
            return
        for v in range(0, left + 1):
            rec(prefix + [v], left - v, depth + 1)

    rec([], P, 0)
    return out


# ----------------------------------------------------------------------------
# Small exact linear algebra on Fractions
# ----------------------------------------------------------------------------

def fr(x):
    return Fraction(x) if not isinstance(x, Fraction) else x


def mat_mul(A, B):
    n, k, m = len(A), len(B), len(B[0])
    out = [[Fraction(0)] * m for _ in range(n)]
    for i in range(n):
        Ai = A[i]
        for t in range(k):
            a = Ai[t]
            if a == 0:
                continue
            Bt = B[t]
            row = out[i]
            for j in range(m):
                if Bt[j]:
                    row[j] += a * Bt[j]
    return out


def transpose(A):
    return [list(r) for r in zip(*A)]


def mat_inv(A):
    n = len(A)
    M = [list(map(fr, r)) + [Fraction(int(i == j)) for j in range(n)] for i, r in enumerate(A)]
    for c in range(n):
        p = next(r for r in range(c, n) if M[r][c] != 0)
        M[c], M[p] = M[p], M[c]
        pv = M[c][c]
        M[c] = [v / pv for v in M[c]]
        for r in range(n):
            if r != c and M[r][c] != 0:
                f = M[r][c]
                M[r] = [a - f * b for a, b in zip(M[r], M[c])]
    return [r[n:] for r in M]


def to_float(A):
    return [[float(v) for v in r] for r in A]


# ----------------------------------------------------------------------------
# Element definition
# ----------------------------------------------------------------------------


class Element:
    def __init__(self, D, P):
        self.D, self.P, self.N = D, P, P + 1
        self.nodes, self.weights = gl_rule(P)
        N = self.N
        self.val = [[cx_legendre(k, self.nodes[q]) for q in range(N)] for k in range(P + 1)]
        self.dval = [[cx_dlegendre(k, self.nodes[q]) for q in range(N)] for k in range(P + 1)]
        self.bd = [[cx_legendre(k, -1.0), cx_legendre(k, 1.0)] for k in range(P + 1)]
        self.slo = [[cx_legendre(k, 0.5 * self.nodes[q] - 0.5) for q in range(N)] for k in range(P + 1)]
        self.shi = [[cx_legendre(k, 0.5 * self.nodes[q] + 0.5) for q in range(N)] for k in range(P + 1)]
        self.mi_s = multi_index(P, D)
        self.mi_st = multi_index(P, D + 1)
        self.Np_s, self.Np_st = len(self.mi_s), len(self.mi_st)
        self.pts_st = list(itertools.product(range(N), repeat=D + 1))  # d=0 slowest
        self.pts_s = list(itertools.product(range(N), repeat=D))
        self.pts_bd = list(itertools.product(range(N), repeat=D))  # free dims: spatial != d, then time
        self._build_matrices()

    # 1D exact integrals of Legendre polynomials on [-1, 1]
    @staticmethod
    def int_pp(a, b):
        return Fraction(2, 2 * a + 1) if a == b else Fraction(0)

    @staticmethod
    def int_p_dp(a, b):  # int P_a P_b'
        return Fraction(2) if (b > a and (a + b) % 2 == 1) else Fraction(0)

    def ms(self, j):  # diagonal spatial mass of a (space or space-time) mode, spatial part only
        m = Fraction(1)
        for d in range(self.D):
            m *= Fraction(2, 2 * j[d] + 1)
        return m

    def _build_matrices(self):
        D, P = self.D, self.P
        st, s = self.mi_st, self.mi_s
        nst, ns = self.Np_st, self.Np_s
        # V with double entries formed as the reference does (product d = 0..D in order)
        V = []
        for pt in self.pts_st:
            row = []
            for n in st:
                phi = 1.0
                for d in range(D + 1):
                    phi *= self.val[n[d]][pt[d]]
                row.append(phi)
            V.append(row)
        self.V = V
        Vf = [[fr(v) for v in r] for r in V]
        G = mat_mul(transpose(Vf), Vf)
        Ginv = mat_inv(G)
        self.Ginv = Ginv
        Vinv = mat_mul(Ginv, transpose(Vf))
        # Mk_h_w, Mk_pred, Sk_pred (exact)
        Mkhw = [[Fraction(0)] * nst for _ in range(nst)]
        Sk = [[[Fraction(0)] * nst for _ in range(nst)] for _ in range(D)]
        Mkpred = [[Fraction(0)] * ns for _ in range(nst)]
        for jj, j in enumerate(st):
            for ii, i in enumerate(st):
                if j[:D] == i[:D]:
                    Mkhw[jj][ii] = self.ms(j) * (1 - self.int_p_dp(i[D], j[D]))
                if j[D] == i[D]:
                    tm = Fraction(2, 2 * j[D] + 1)
                    for d in range(D):
                        ok = all(j[a] == i[a] for a in range(D) if a != d)
                        if not ok:
                            continue
                        v = Fraction(1)
                        for a in range(D):
                            if a != d:
                                v *= Fraction(2, 2 * j[a] + 1)
                        v *= self.int_p_dp(j[d], i[d])
                        Sk[d][jj][ii] = tm * v
            for ii, i in enumerate(s):
                if j[:D] == i[:D]:
                    Mkpred[jj][ii] = (-1) ** j[D] * self.ms(j)
        Mkhw_inv = mat_inv(Mkhw)
        self.W = to_float(mat_mul(Mkhw_inv, Mkpred))
        self.A = []
        self.C = []
        for d in range(D):
            KS = mat_mul(Mkhw_inv, Sk[d])
            self.A.append(to_float(mat_mul(KS, Vinv)))
            self.C.append(to_float(mat_mul(KS, Ginv)))
        self.Mdiag = [float(self.ms(n)) for n in s]
        self.Minv = [float(1 / self.ms(n)) for n in s]

    # ---- dense reference operators (rows = outputs) for chain verification
    def dense_vol_eval(self):
        return self.V

    def dense_sk_corr(self, d):
        D, N = self.D, self.N
        out = []
        for n in self.mi_s:
            row = []
            for pt in self.pts_st:
                w = 1.0
                for a in range(D + 1):
                    w *= self.weights[pt[a]]
                ph = 1.0
                for a in range(D):
                    ph *= (self.dval if a == d else self.val)[n[a]][pt[a]]
                row.append(ph * w)
            out.append(row)
        return out

    def bd_point_coords(self, d, pt):
        """face point pt (free dims: spatial dims != d in order, then time) ->
        dict dim -> node index"""
        free = [a for a in range(self.D) if a != d] + [self.D]
        return {a: pt[i] for i, a in enumerate(free)}

    def dense_face_eval(self, d, side):
        out = []
        for pt in self.pts_bd:
            c = self.bd_point_coords(d, pt)
            row = []
            for n in self.mi_st:
                phi = 1.0
                for a in range(self.D + 1):
                    phi *= self.bd[n[a]][side] if a == d else self.val[n[a]][c[a]]
                row.append(phi)
            out.append(row)
        return out

    def dense_bd_term(self, d, side):
        out = []
        for n in self.mi_s:
            row = []
            for pt in self.pts_bd:
                c = self.bd_point_coords(d, pt)
                w = 1.0
                for a in c:
                    w *= self.weights[c[a]]
                phi = 1.0
                for a in range(self.D):
                    phi *= self.bd[n[a]][side] if a == d else self.val[n[a]][c[a]]
                row.append(phi * w)
            out.append(row)
        return out


# ----------------------------------------------------------------------------
# Sparse stage chains over tuple index spaces
# ----------------------------------------------------------------------------


class Stage:
    """out[r] = sum_c coef * in[c]; rows: list of lists of (col, coef)."""

    def __init__(self, n_in, n_out, rows):
        self.n_in, self.n_out, self.rows = n_in, n_out, rows

    def nnz(self):
        return sum(len(r) for r in self.rows)


def stage_from_map(in_keys, out_keys, fn):
    """fn(out_key) -> list of (in_key, coef)"""
    pos = {k: i for i, k in enumerate(in_keys)}
    rows = []
    for ok in out_keys:
        terms = [(pos[ik], c) for ik, c in fn(ok) if ik in pos and c != 0.0]
        rows.append(terms)
    return Stage(len(in_keys), len(out_keys), rows)


def chain_dense(stages):
    """The dense matrix of a chain of stages (float64 products)."""
    import numpy as np

    M = None
    for st in stages:
        S = np.zeros((st.n_out, st.n_in))
        for r, terms in enumerate(st.rows):
            for c, v in terms:
                S[r, c] += v
        M = S if M is None else S @ M
    return M.tolist()


def check_chain(stages, dense, name, tol=1e-12, scale=None):
    """The chain's product equals the dense operator to tol relative to
    scale (default: the dense operator's largest entry; an operator that is
    zero up to rounding is checked against the scale of the operator it
    derives from)."""
    M = chain_dense(stages)
    if scale is None:
        scale = max(abs(v) for r in dense for v in r) or 1.0
    err = max(abs(M[i][j] - dense[i][j]) for i in range(len(dense)) for j in range(len(dense[0])))
    if err > tol * scale:
        raise SystemExit(f"chain check failed for {name}: {err / scale}")


def prefixes(P, length):
    return [t for t in itertools.product(range(P + 1), repeat=length) if sum(t) <= P]


class Chains:
    def __init__(self, el):
        self.el = el

    # keys are tuples with entries ('m', a) mode or ('q', k) point index
    def eval_chain(self, order, start_keys, dim_tables, n_dims):
        """Evaluate a modal expansion at tensor points by contracting
        positions in `order`; dim_tables[pos] = table T[a][k] (k may be a
        single pseudo point 0 for a fixed face dimension)."""
        stages = []
        keys = start_keys
        for pos in order:
            T = dim_tables[pos]
            npts = len(T[0])
            new_keys = sorted({tuple(('q', k) if i == pos else e for i, e in enumerate(key))
                               for key in keys for k in range(npts)})

            def fn(ok, pos=pos, T=T):
                k = ok[pos][1]
                terms = []
                for a in range(self.el.P + 1):
                    ik = tuple(('m', a) if i == pos else e for i, e in enumerate(ok))
                    terms.append((ik, T[a][k]))
                return terms

            stages.append(stage_from_map(keys, new_keys, fn))
            keys = new_keys
        return stages, keys

    def project_chain(self, order, start_keys, dim_tables, mode_ok):
        """Transposed contraction: point indices -> mode indices.  mode_ok(key)
        filters partially contracted keys (total degree <= P)."""
        stages = []
        keys = start_keys
        for pos in order:
            T = dim_tables[pos]  # T[a][k]
            new_keys = sorted({tuple(('m', a) if i == pos else e for i, e in enumerate(key))
                               for key in keys for a in range(len(T))})
            new_keys = [k for k in new_keys if mode_ok(k)]

            def fn(ok, pos=pos, T=T):
                a = ok[pos][1]
                return [(tuple(('q', k) if i == pos else e for i, e in enumerate(ok)), T[a][k])
                        for k in range(len(T[0]))]

            stages.append(stage_from_map(keys, new_keys, fn))
            keys = new_keys
        return stages, keys


def degree_ok(P):
    def ok(key):
        return sum(e[1] for e in key if e[0] == 'm') <= P
    return ok


def build_ops(el):
    D, P, N = el.D, el.P, el.N
    ch = Chains(el)
    ops = {}
    st_keys = [tuple(('m', a) for a in n) for n in el.mi_st]
    pt_keys_st = [tuple(('q', k) for k in pt) for pt in el.pts_st]
    # ---- vol_eval: st modes -> st points; contract time first, then D-1..0
    order = list(range(D, -1, -1))
    stages, keys = ch.eval_chain(order, st_keys, {p: el.val for p in range(D + 1)}, D + 1)
    stages.append(stage_from_map(keys, pt_keys_st, lambda ok: [(ok, 1.0)]))
    check_chain(stages, el.dense_vol_eval(), "vol_eval")
    ops["vol_eval"] = (stages, el.Np_st, len(pt_keys_st))

    # ---- vol_eval_init: U_w placed in st modes 0..Np_s-1 (the reference's
    # predictor initial guess, AmrDG.tpp:520-533).  Those are exactly the
    # st modes with a_0 == 0, so the expansion does not depend on x_0 and is
    # evaluated on the (x_1.., t) grid only.
    init_modes = el.mi_st[:el.Np_s]
    assert all(n[0] == 0 for n in init_modes)
    init_keys = [tuple(('m', a) for a in n[1:]) for n in init_modes]
    order = list(range(D - 1, -1, -1))  # positions in the reduced tuple (x_1.., t)
    tabs = {p: el.val for p in range(D)}
    stages, keys = ch.eval_chain(order, init_keys, tabs, D)
    grid_keys = [tuple(('q', k) for k in pt) for pt in itertools.product(range(N), repeat=D)]
    stages.append(stage_from_map(keys, grid_keys, lambda ok: [(ok, 1.0)]))
    dense = [[el.V[el.pts_st.index((0,) + pt)][i] for i in range(el.Np_s)]
             for pt in itertools.product(range(N), repeat=D)]
    check_chain(stages, dense, "vol_eval_init")
    ops["vol_eval_init"] = (stages, el.Np_s, len(grid_keys))

    # ---- proj[d]: F at st points -> st modes, A_d = C_d V^T
    order = list(range(0, D + 1))
    vt_stages, keys = ch.project_chain(order, pt_keys_st, {p: el.val for p in range(D + 1)}, degree_ok(P))
    mode_pos = {tuple(('m', a) for a in n): i for i, n in enumerate(el.mi_st)}
    perm = stage_from_map(keys, [tuple(('m', a) for a in n) for n in el.mi_st], lambda ok: [(ok, 1.0)])
    for d in range(D):
        Cd = el.C[d]
        cst = Stage(el.Np_st, el.Np_st, [[(c, Cd[r][c]) for c in range(el.Np_st) if Cd[r][c] != 0.0]
                                         for r in range(el.Np_st)])
        stages = vt_stages + [perm, cst]
        check_chain(stages, el.A[d], f"proj{d}", tol=1e-11)
        dense_A = Stage(len(pt_keys_st), el.Np_st,
                        [[(c, el.A[d][r][c]) for c in range(len(pt_keys_st)) if el.A[d][r][c] != 0.0]
                         for r in range(el.Np_st)])
        f_nnz = sum(s.nnz() for s in stages)
        ops[f"proj{d}"] = (stages if f_nnz < dense_A.nnz() else [dense_A], len(pt_keys_st), el.Np_st)

    # ---- proj_init[d]: F given on the (x_1.., t) grid (x_0-independent)
    Ssum = [sum(el.val[a][k] for k in range(N)) for a in range(P + 1)]
    # stage 1: replicate + contract x_0: g[(a0, q1.., qt)] = Ssum[a0] * F[(q1.., qt)]
    g1_keys = sorted({(('m', a),) + k for a in range(P + 1) for k in grid_keys if Ssum[a] != 0.0})
    st1 = stage_from_map(grid_keys, g1_keys, lambda ok: [(ok[1:], Ssum[ok[0][1]])])
    rest, keys = ch.project_chain(list(range(1, D + 1)), g1_keys, {p: el.val for p in range(D + 1)}, degree_ok(P))
    mode_keys_all = [tuple(('m', a) for a in n) for n in el.mi_st]
    perm_i = stage_from_map(keys, mode_keys_all, lambda ok: [(ok, 1.0)])
    for d in range(D):
        Cd = el.C[d]
        cst = Stage(el.Np_st, el.Np_st, [[(c, Cd[r][c]) for c in range(el.Np_st) if Cd[r][c] != 0.0]
                                         for r in range(el.Np_st)])
        stages = [st1] + rest + [perm_i, cst]
        dense = [[sum(el.A[d][r][el.pts_st.index((i,) + pt)] for i in range(N))
                  for pt in itertools.product(range(N), repeat=D)] for r in range(el.Np_st)]
        # proj_init[0] is zero up to rounding (the x_0 projection of an
        # x_0-independent flux): checked on the scale of A_d
        check_chain(stages, dense, f"proj_init{d}", tol=1e-11,
                    scale=max(abs(v) for r in el.A[d] for v in r))
        ops[f"proj_init{d}"] = (stages, len(grid_keys), el.Np_st)

    # ---- W U: (Np_s) -> (Np_st)
    ops["wu"] = ([Stage(el.Np_s, el.Np_st, [[(c, el.W[r][c]) for c in range(el.Np_s) if el.W[r][c] != 0.0]
                                           for r in range(el.Np_st)])], el.Np_s, el.Np_st)

    # ---- vol_term[d]: Sk_corr[d] (st points -> s modes)
    for d in range(D):
        tabs = {}
        for p in range(D):
            base = el.dval if p == d else el.val
            tabs[p] = [[base[a][k] * el.weights[k] for k in range(N)] for a in range(P + 1)]
        tabs[D] = [[el.weights[k] for k in range(N)]]  # time: weighted sum to a single "mode"
        order = [D] + list(range(0, D))
        stages, keys = ch.project_chain(order, pt_keys_st, tabs, degree_ok(P))
        s_keys = [tuple(('m', a) for a in n) + (('m', 0),) for n in el.mi_s]
        stages.append(stage_from_map(keys, s_keys, lambda ok: [(ok, 1.0)]))
        check_chain(stages, el.dense_sk_corr(d), f"vol_term{d}")
        ops[f"vol_term{d}"] = (stages, len(pt_keys_st), el.Np_s)

    # ---- vol_eval_slice[k]: st modes -> the spatial GL points of time node k
    # (one time slice of vol_eval's points, pts_s order).  Together with
    # vol_term_sp this lets a kernel hold one slice of point values at a time:
    # the same stages as vol_eval restricted to one time column.
    sp_keys = [tuple(('q', k) for k in pt) for pt in el.pts_s]
    for k in range(N):
        tabs = {p: el.val for p in range(D)}
        tabs[D] = [[el.val[a][k]] for a in range(P + 1)]
        stages, keys = ch.eval_chain(list(range(D, -1, -1)), st_keys, tabs, D + 1)
        stages.append(stage_from_map(keys, sp_keys, lambda ok: [(ok + (('q', 0),), 1.0)]))
        dense = [el.V[el.pts_st.index(tuple(pt) + (k,))] for pt in el.pts_s]
        check_chain(stages, dense, f"vol_eval_slice{k}")
        ops[f"vol_eval_slice{k}"] = (stages, el.Np_st, len(sp_keys))

    # ---- face_slice[d][side]: the face values of one time slice from the
    # slice's spatial point values, by Lagrange extrapolation along d (H is a
    # polynomial of degree <= P in x_d, so N nodes determine it exactly):
    # point x of the face (free dims != d in order) <- sum_i l_i(+-1) H(x with x_d = node i)
    def lagrange_at(xe):
        out = []
        for i in range(N):
            v = Fraction(1)
            for j in range(N):
                if j != i:
                    v *= (Fraction(xe) - Fraction(el.nodes[j])) / (Fraction(el.nodes[i]) - Fraction(el.nodes[j]))
            out.append(float(v))
        return out
    lag = [lagrange_at(-1.0), lagrange_at(1.0)]
    sp_index = {tuple(pt): i for i, pt in enumerate(el.pts_s)}
    for d in range(D):
        free = [a for a in range(D) if a != d]
        free_pts = list(itertools.product(range(N), repeat=D - 1))
        for side in range(2):
            rows = []
            for fp in free_pts:
                terms = []
                for i in range(N):
                    full = [0] * D
                    full[d] = i
                    for a, v in zip(free, fp):
                        full[a] = v
                    terms.append((sp_index[tuple(full)], lag[side][i]))
                rows.append(terms)
            st_face = Stage(len(el.pts_s), len(free_pts), rows)
            name = f"face_slice{d}{side}"
            ref_full = el.dense_face_eval(d, side)
            for k in range(N):  # face_slice o vol_eval_slice[k] == face_eval at time node k
                ev = chain_dense(ops[f"vol_eval_slice{k}"][0])
                got = chain_dense([st_face])
                comp = [[sum(got[r][c] * ev[c][m] for c in range(len(el.pts_s))) for m in range(el.Np_st)]
                        for r in range(len(free_pts))]
                ref = [ref_full[el.pts_bd.index(tuple(fp) + (k,))] for fp in free_pts]
                scale = max(abs(v) for r in ref for v in r)
                err = max(abs(comp[i][j] - ref[i][j]) for i in range(len(ref)) for j in range(el.Np_st))
                if err > 1e-12 * scale:
                    raise SystemExit(f"{name} does not reproduce face_eval{d}{side} at time node {k}: {err / scale}")
            ops[name] = ([st_face], len(el.pts_s), len(free_pts))

    # ---- vol_term_sp[d]: the spatial stages of vol_term[d], applied to the
    # time-integrated flux sum_k w_k F_d(x, t_k) at the spatial points
    for d in range(D):
        tabs = {}
        for p in range(D):
            base = el.dval if p == d else el.val
            tabs[p] = [[base[a][k] * el.weights[k] for k in range(N)] for a in range(P + 1)]
        stages, keys = ch.project_chain(list(range(D)), sp_keys, tabs, degree_ok(P))
        s_keys = [tuple(('m', a) for a in n) for n in el.mi_s]
        stages.append(stage_from_map(keys, s_keys, lambda ok: [(ok, 1.0)]))
        dsk = el.dense_sk_corr(d)
        dense = [[dsk[r][el.pts_st.index(tuple(pt) + (0,))] / el.weights[0] for pt in el.pts_s]
                 for r in range(el.Np_s)]
        check_chain(stages, dense, f"vol_term_sp{d}")
        ops[f"vol_term_sp{d}"] = (stages, len(sp_keys), el.Np_s)

    # ---- face_eval[d][side]: st modes -> face points (free spatial dims, time)
    bd_pt_keys = [tuple(('q', k) for k in pt) for pt in el.pts_bd]
    for d in range(D):
        for side in range(2):
            tabs = {p: el.val for p in range(D + 1)}
            tabs[d] = [[el.bd[a][side]] for a in range(P + 1)]
            order = [d] + [p for p in range(D, -1, -1) if p != d]
            stages, keys = ch.eval_chain(order, st_keys, tabs, D + 1)
            # drop the singleton point of dim d; order free dims as (spatial != d, time)
            free = [a for a in range(D) if a != d] + [D]

            def fn(ok, free=free):
                full = [None] * (D + 1)
                full[d] = ('q', 0)
                for i, a in enumerate(free):
                    full[a] = ok[i]
                return [(tuple(full), 1.0)]

            stages.append(stage_from_map(keys, bd_pt_keys, fn))
            check_chain(stages, el.dense_face_eval(d, side), f"face_eval{d}{side}")
            ops[f"face_eval{d}{side}"] = (stages, el.Np_st, len(bd_pt_keys))

    # ---- bd_term[d][side]: Mkbd{m,p}[d] (face points -> s modes)
    for d in range(D):
        for side in range(2):
            free = [a for a in range(D) if a != d] + [D]
            # contract time (weights), then free spatial dims with val*w, then expand dim d with bd
            nf = len(free)
            tabs = {}
            for i, a in enumerate(free):
                if a == D:
                    tabs[i] = [[el.weights[k] for k in range(N)]]
                else:
                    tabs[i] = [[el.val[m][k] * el.weights[k] for k in range(N)] for m in range(P + 1)]
            order = [nf - 1] + list(range(0, nf - 1))
            stages, keys = ch.project_chain(order, bd_pt_keys, tabs, degree_ok(P))
            s_keys = [tuple(('m', a) for a in n) for n in el.mi_s]

            def fn(ok, free=free, side=side, d=d):
                sub = tuple(ok[a] for a in free if a != D) + (('m', 0),)
                return [(sub, el.bd[ok[d][1]][side])]

            stages.append(stage_from_map(keys, s_keys, fn))
            check_chain(stages, el.dense_bd_term(d, side), f"bd_term{d}{side}")
            ops[f"bd_term{d}{side}"] = (stages, len(bd_pt_keys), el.Np_s)

    # ---- spatial modes at spatial GL point 0 (set_Dt, AmrDG.h:1275,1306)
    row = []
    for n in el.mi_s:
        phi = 1.0
        for d in range(D):
            phi *= el.val[n[d]][0]
        row.append(phi)
    ops["u_pt0"] = ([Stage(el.Np_s, 1, [[(c, row[c]) for c in range(el.Np_s) if row[c] != 0.0]])], el.Np_s, 1)

    # ---- sp_eval: spatial modes -> the spatial GL points (pts_s order).
    # W U, the space-time expansion the Picard update starts from, is U
    # constant in time (checked below), so a predictor H_w = W U + dlt is
    # U(x) + dlt(x, t) at the space-time points: the seeded path evaluates
    # the first term with this operator and the second one in its own
    # precision.
    s_keys = [tuple(('m', a) for a in n) for n in el.mi_s]

    def phi_s(n, coord):  # coord: dim -> table row (val at a node, or bd at a face)
        v = 1.0
        for a in range(D):
            v *= coord[a][n[a]]
        return v

    stages, keys = ch.eval_chain(list(range(D - 1, -1, -1)), s_keys, {p: el.val for p in range(D)}, D)
    stages.append(stage_from_map(keys, sp_keys, lambda ok: [(ok, 1.0)]))
    dense_sp = [[phi_s(n, {a: [el.val[m][pt[a]] for m in range(P + 1)] for a in range(D)}) for n in el.mi_s]
                for pt in el.pts_s]
    check_chain(stages, dense_sp, "sp_eval")
    ops["sp_eval"] = (stages, el.Np_s, len(sp_keys))
    VW = [[sum(el.V[i][k] * el.W[k][j] for k in range(el.Np_st)) for j in range(el.Np_s)]
          for i in range(len(el.pts_st))]
    for i, pt in enumerate(el.pts_st):
        want = dense_sp[el.pts_s.index(tuple(pt[:D]))]
        if max(abs(VW[i][j] - want[j]) for j in range(el.Np_s)) > 1e-12:
            raise SystemExit("W U is not U constant in time")

    # ---- the projections A_d = C_d V^T one time slice at a time:
    #   A_d F = C_d sum_k T_k vt_sp(F(., t_k)),
    # vt_sp = V_s^T (spatial points -> spatial modes, no weights), T_k the
    # expansion of spatial mode b to the space-time modes (b, a_t) with the
    # factor val[a_t][k] (st_time / st_space / time_val tables), cproj_d = C_d.
    stages, keys = ch.project_chain(list(range(D)), sp_keys, {p: el.val for p in range(D)}, degree_ok(P))
    stages.append(stage_from_map(keys, s_keys, lambda ok: [(ok, 1.0)]))
    dense_vts = [[dense_sp[m][b] for m in range(len(el.pts_s))] for b in range(el.Np_s)]
    check_chain(stages, dense_vts, "vt_sp")
    ops["vt_sp"] = (stages, len(sp_keys), el.Np_s)
    st_space = [el.mi_s.index(tuple(n[:D])) for n in el.mi_st]
    st_time = [n[D] for n in el.mi_st]
    for d in range(D):
        Cd = el.C[d]
        ops[f"cproj{d}"] = ([Stage(el.Np_st, el.Np_st, [[(c, Cd[r][c]) for c in range(el.Np_st) if Cd[r][c] != 0.0]
                                                      for r in range(el.Np_st)])], el.Np_st, el.Np_st)
        # the sliced form against A_d
        for r in range(el.Np_st):
            for i, pt in enumerate(el.pts_st):
                k, m = pt[D], el.pts_s.index(tuple(pt[:D]))
                v = sum(Cd[r][n] * el.val[st_time[n]][k] * dense_vts[st_space[n]][m] for n in range(el.Np_st))
                if abs(v - el.A[d][r][i]) > 1e-11 * max(1.0, abs(el.A[d][r][i])):
                    raise SystemExit(f"sliced projection {d} does not reproduce A_{d}")
    el.st_space, el.st_time = st_space, st_time

    # ---- face_eval_sp[d][side]: spatial modes -> the face's spatial points
    # (free dims != d in order, face_slice's point order)
    for d in range(D):
        free = [a for a in range(D) if a != d]
        free_pts = list(itertools.product(range(N), repeat=D - 1))
        fkeys = [tuple(('q', 0) if a == d else ('q', fp[free.index(a)]) for a in range(D)) for fp in free_pts]
        for side in range(2):
            tabs = {p: el.val for p in range(D)}
            tabs[d] = [[el.bd[a][side]] for a in range(P + 1)]
            order = [d] + [p for p in range(D - 1, -1, -1) if p != d]
            stages, keys = ch.eval_chain(order, s_keys, tabs, D)
            stages.append(stage_from_map(keys, fkeys, lambda ok: [(ok, 1.0)]))
            dense = [[phi_s(n, {a: ([el.bd[m][side] for m in range(P + 1)] if a == d else
                                    [el.val[m][fp[free.index(a)]] for m in range(P + 1)]) for a in range(D)})
                      for n in el.mi_s] for fp in free_pts]
            check_chain(stages, dense, f"face_eval_sp{d}{side}")
            ops[f"face_eval_sp{d}{side}"] = (stages, el.Np_s, len(free_pts))
    return ops


# ----------------------------------------------------------------------------
# CUDA emission
# ----------------------------------------------------------------------------


def lit(v):
    r = repr(float(v))
    if "e" not in r and "." not in r and "inf" not in r and "nan" not in r:
        r += ".0"
    return r


def fp64_ops(stage):
    """FP64 instructions one stage issues per column (a term with coefficient
    +-1 at the head of a row is a move, every further term one DADD/DFMA)."""
    n = 0
    for terms in stage.rows:
        if not terms:
            continue
        n += len(terms) - 1
        if terms[0][1] not in (1.0, -1.0):
            n += 1
    return n


def emit_stage(lines, st, src, dst, indent="    "):
    for r, terms in enumerate(st.rows):
        d = dst(r)
        if not terms:
            lines.append(f"{indent}{d} = T(0);")
            continue
        expr = None
        for c, v in terms:
            x = src(c)
            if expr is None:
                if v == 1.0:
                    expr = f"{x}"
                elif v == -1.0:
                    expr = f"(-{x})"
                else:
                    expr = f"T({lit(v)}) * {x}"
            else:
                if v == 1.0:
                    expr = f"({expr} + {x})"
                elif v == -1.0:
                    expr = f"({expr} - {x})"
                else:
                    expr = f"fma(T({lit(v)}), {x}, {expr})"
        lines.append(f"{indent}{d} = {expr};")


def emit_op(name, op):
    stages, n_in, n_out = op
    nops = sum(fp64_ops(s) for s in stages)
    lines = [f"  // {name}: {n_in} -> {n_out}, {nops} FP64 instructions per column",
             f"  template <class T = double, class In, class Out>",
             f"  static __device__ __forceinline__ void {name}(const In& in, Out out) {{"]
    for si, st in enumerate(stages):
        last = si == len(stages) - 1
        if not last:
            lines.append(f"    T t{si}[{st.n_out}];")
        src = (lambda c: f"T(in({c}))") if si == 0 else (lambda c, p=si - 1: f"t{p}[{c}]")
        dst = (lambda r: f"out({r})") if last else (lambda r, s=si: f"t{s}[{r}]")
        emit_stage(lines, st, src, dst)
    lines.append("  }")
    return "\n".join(lines), nops


def add_ic_proj(el, ops):
    """quadmat (AmrDG_ElementMatrix.tpp:154-168): spatial points -> spatial modes."""
    D, P, N = el.D, el.P, el.N
    ch = Chains(el)
    pt_keys = [tuple(('q', k) for k in pt) for pt in el.pts_s]
    tabs = {p: [[el.val[a][k] * el.weights[k] for k in range(N)] for a in range(P + 1)] for p in range(D)}
    stages, keys = ch.project_chain(list(range(D)), pt_keys, tabs, degree_ok(P))
    s_keys = [tuple(('m', a) for a in n) for n in el.mi_s]
    stages.append(stage_from_map(keys, s_keys, lambda ok: [(ok, 1.0)]))
    dense = []
    for n in el.mi_s:
        row = []
        for pt in el.pts_s:
            w = 1.0
            for d in range(D):
                w *= el.weights[pt[d]]
            phi = 1.0
            for d in range(D):
                phi *= el.val[n[d]][pt[d]]
            row.append(phi * w)
        dense.append(row)
    check_chain(stages, dense, "ic_proj")
    ops["ic_proj"] = (stages, len(pt_keys), el.Np_s)


def add_amr_ops(el, ops):
    """L2ProjInterp operators (AmrDG_Interpolater.tpp:85-231), each an exact
    sum of products of the double-valued tables, rounded once:
      pcf{l}      = Minv P_cf[l]              coarse -> fine child l (amr_scatter)
      pfc{l}      = P_fc[l]                   fine child l -> coarse (amr_gather)
      pflux{d}{s}{k} = P_flux_fc_{low,high}[d][k]  fine face points -> coarse face modes
    Child l of P_cf / P_fc: bit (D-1-d) of l is the upper half in direction d.
    Face child k of P_flux: bit i of k is the upper half in the i-th direction != d."""
    D, P, N = el.D, el.P, el.N
    ms = el.mi_s
    quad = [[Fraction(0)] * len(el.pts_s) for _ in ms]  # quadmat (exact products of doubles)
    for j, n in enumerate(ms):
        for qi, pt in enumerate(el.pts_s):
            w = Fraction(1)
            ph = Fraction(1)
            for d in range(D):
                w *= Fraction(el.weights[pt[d]])
                ph *= Fraction(el.val[n[d]][pt[d]])
            quad[j][qi] = ph * w
    minv = [Fraction(1) / el.ms(n) for n in ms]
    for l in range(1 << D):
        up = [(l >> (D - 1 - d)) & 1 for d in range(D)]

        def phi_child(n, pt):
            v = Fraction(1)
            for d in range(D):
                tbl = el.shi if up[d] else el.slo
                v *= Fraction(tbl[n[d]][pt[d]])
            return v

        Pcf = [[sum(quad[j][qi] * phi_child(ms[m], pt) for qi, pt in enumerate(el.pts_s)) for m in range(len(ms))]
               for j in range(len(ms))]
        Pfc = [[sum(quad[m][qi] * phi_child(ms[j], pt) for qi, pt in enumerate(el.pts_s)) for m in range(len(ms))]
               for j in range(len(ms))]
        cf = [[float(minv[j] * Pcf[j][m]) for m in range(len(ms))] for j in range(len(ms))]
        fc = [[float(Pfc[j][m]) for m in range(len(ms))] for j in range(len(ms))]
        ops[f"pcf{l}"] = ([Stage(len(ms), len(ms), [[(c, r[c]) for c in range(len(ms)) if r[c] != 0.0] for r in cf])],
                          len(ms), len(ms))
        ops[f"pfc{l}"] = ([Stage(len(ms), len(ms), [[(c, r[c]) for c in range(len(ms)) if r[c] != 0.0] for r in fc])],
                          len(ms), len(ms))
    nfc = 1 << (D - 1)
    for d in range(D):
        free = [a for a in range(D) if a != d] + [D]
        for k in range(nfc):
            upper = {}
            bit = 0
            for a in range(D):
                if a == d:
                    continue
                upper[a] = (k >> bit) & 1
                bit += 1
            for side in range(2):
                rows = []
                for n in ms:
                    row = []
                    for pt in el.pts_bd:
                        c = {a: pt[i] for i, a in enumerate(free)}
                        w = Fraction(1)
                        for a in free:
                            w *= Fraction(el.weights[c[a]])
                        ph = Fraction(el.bd[n[d]][side])
                        for a in range(D):
                            if a == d:
                                continue
                            tbl = el.shi if upper[a] else el.slo
                            ph *= Fraction(tbl[n[a]][c[a]])
                        row.append(float(ph * w))
                    rows.append(row)
                ops[f"pflux{d}{side}{k}"] = ([Stage(len(el.pts_bd), len(ms),
                                                    [[(c, r[c]) for c in range(len(el.pts_bd)) if r[c] != 0.0]
                                                     for r in rows])], len(el.pts_bd), len(ms))


def legendre_monomial(n):
    """Exact monomial coefficients of P_n (index = power)."""
    p0, p1 = [Fraction(1)], [Fraction(0), Fraction(1)]
    if n == 0:
        return p0
    for k in range(2, n + 1):
        xp1 = [Fraction(0)] + p1
        p2 = [Fraction(0)] * (k + 1)
        for i, v in enumerate(xp1):
            p2[i] += Fraction(2 * k - 1, k) * v
        for i, v in enumerate(p0):
            p2[i] -= Fraction(k - 1, k) * v
        p0, p1 = p1, p2
    return p1


def legendre_shift_coeffs(P, upper):
    """c[n][j]: P_n((x + s) / 2) = sum_j c[n][j] P_j(x), s = +1 (upper half of
    a coarse interval) or -1 (lower half), exact."""
    s = Fraction(1 if upper else -1)
    out = []
    for n in range(P + 1):
        a = legendre_monomial(n)
        # sum_i a_i ((x + s) / 2)^i in monomials of x
        poly = [Fraction(0)] * (n + 1)
        for i, ai in enumerate(a):
            for r in range(i + 1):  # binomial term x^r s^(i-r)
                poly[r] += ai * Fraction(math.comb(i, r)) * s ** (i - r) / Fraction(2) ** i
        row = []
        for j in range(P + 1):
            pj = legendre_monomial(j)
            integ = Fraction(0)
            for r, pr in enumerate(poly):
                for t, pt in enumerate(pj):
                    if (r + t) % 2 == 0:
                        integ += pr * pt * Fraction(2, r + t + 1)
            row.append(Fraction(2 * j + 1, 2) * integ)
        out.append(row)
    return out


def add_face_moment_ops(el, ops):
    """Face moments of the numerical flux.  For a face of direction d the
    corrector's boundary operators only see the flux through its tangential
    Legendre moments
      M[j] = sum_pts w_t prod_a (w_a P_ja(x_a)) fnum(pt),  |j| <= P,
    (a over the spatial dims != d), because
      Mkbd{m,p}[d][n] fnum = P_nd(+-1) M[n without d]          (bd_mom)
      P_flux_fc[k][n] fnum  = P_nd(+-1) sum_j prod_a c[n_a][j_a] M_fine[j]  (pflux_mom)
    with c the exact Legendre coefficients of P_n((x -+ 1)/2) on a half face.
    face_mom is the same operator for every direction (the free dims use the
    same tables)."""
    D, P, N = el.D, el.P, el.N
    ch = Chains(el)
    nfree = D - 1
    mom = multi_index(P, nfree)
    mom_keys = [tuple(('m', a) for a in j) for j in mom]
    bd_pt_keys = [tuple(('q', k) for k in pt) for pt in el.pts_bd]
    tabs = {i: [[el.val[a][k] * el.weights[k] for k in range(N)] for a in range(P + 1)] for i in range(nfree)}
    tabs[nfree] = [[el.weights[k] for k in range(N)]]
    stages, keys = ch.project_chain([nfree] + list(range(nfree)), bd_pt_keys, tabs, degree_ok(P))
    stages.append(stage_from_map(keys, mom_keys, lambda ok: [(ok + (('m', 0),), 1.0)]))
    dense_mom = []
    for j in mom:
        row = []
        for pt in el.pts_bd:
            w = el.weights[pt[nfree]]
            for i in range(nfree):
                w *= el.weights[pt[i]] * el.val[j[i]][pt[i]]
            row.append(w)
        dense_mom.append(row)
    check_chain(stages, dense_mom, "face_mom")
    ops["face_mom"] = (stages, len(bd_pt_keys), len(mom))
    # face_mom_sp: the tangential stages alone, on the time integral of the
    # flux at the NQ_BD / N spatial face points (free dims in order)
    sp_face = list(itertools.product(range(N), repeat=nfree))
    sp_keys = [tuple(('q', k) for k in pt) for pt in sp_face]
    tabs_sp = {i: tabs[i] for i in range(nfree)}
    st_sp, keys_sp = ch.project_chain(list(range(nfree)), sp_keys, tabs_sp, degree_ok(P))
    st_sp.append(stage_from_map(keys_sp, mom_keys, lambda ok: [(ok, 1.0)]))
    dense_sp = [[dense_mom[r][el.pts_bd.index(tuple(pt) + (0,))] / el.weights[0] for pt in sp_face]
                for r in range(len(mom))]
    check_chain(st_sp, dense_sp, "face_mom_sp")
    ops["face_mom_sp"] = (st_sp, len(sp_keys), len(mom))
    pos = {j: i for i, j in enumerate(mom)}

    def composed(rows):
        """(Np_s x NM) rows times the dense moment operator."""
        return [[sum(v * dense_mom[c][p] for c, v in r) for p in range(len(el.pts_bd))] for r in rows]

    def dense_of(name):
        st = ops[name][0]
        return chain_dense(st)

    for d in range(D):
        free = [a for a in range(D) if a != d]
        for side in range(2):
            rows = [[(pos[tuple(n[a] for a in free)], el.bd[n[d]][side])] for n in el.mi_s]
            name = f"bd_mom{d}{side}"
            ref = el.dense_bd_term(d, side)
            got = composed(rows)
            scale = max(abs(v) for r in ref for v in r)
            err = max(abs(got[i][p] - ref[i][p]) for i in range(len(ref)) for p in range(len(ref[0])))
            if err > 1e-12 * scale:
                raise SystemExit(f"{name} does not reproduce bd_term{d}{side}: {err / scale}")
            ops[name] = ([Stage(len(mom), el.Np_s, rows)], len(mom), el.Np_s)
    c_lo, c_hi = legendre_shift_coeffs(P, False), legendre_shift_coeffs(P, True)
    nfc = 1 << (D - 1)
    for d in range(D):
        free = [a for a in range(D) if a != d]
        for k in range(nfc):
            up = {a: (k >> i) & 1 for i, a in enumerate(free)}
            for side in range(2):
                rows = []
                for n in el.mi_s:
                    terms = []
                    for j in mom:
                        v = Fraction(1)
                        for i, a in enumerate(free):
                            v *= (c_hi if up[a] else c_lo)[n[a]][j[i]]
                            if v == 0:
                                break
                        if v != 0:
                            terms.append((pos[j], float(v * Fraction(el.bd[n[d]][side]))))
                    rows.append(terms)
                name = f"pflux_mom{d}{side}{k}"
                ref = dense_of(f"pflux{d}{side}{k}")
                got = composed(rows)
                scale = max(abs(v) for r in ref for v in r)
                err = max(abs(got[i][p] - ref[i][p]) for i in range(len(ref)) for p in range(len(ref[0])))
                if err > 1e-12 * scale:
                    raise SystemExit(f"{name} does not reproduce pflux{d}{side}{k}: {err / scale}")
                ops[name] = ([Stage(len(mom), el.Np_s, rows)], len(mom), el.Np_s)
    return len(mom)


# Coefficients below DENOISE_REL of a stage's largest are the rounding residue
# of exact zeros: the matrices built by quadrature on the double-valued node
# and weight tables (P_cf, P_fc, the Gram inverse inside C_d) carry entries of
# 1e-17 .. 1e-34 where the exact projections between Legendre bases are zero
# (their true entries are rationals of order 1e-3 .. 1e2).  They are dropped,
# and an operator whose whole product is below DENOISE_REL of its norm bound
# (the product of its stages' largest row sums) is zero: it is emitted with no
# arithmetic and reported in ZERO_OPS.  Every operator is checked against its
# dense matrix again, to DENOISE_REL of the norm bound.
DENOISE_REL = 1e-13


def norm_bound(stages):
    b = 1.0
    for st in stages:
        b *= max((sum(abs(v) for _, v in r) for r in st.rows), default=0.0)
    return b


def denoise(ops):
    zero = set()
    for name, (stages, n_in, n_out) in list(ops.items()):
        before = chain_dense(stages)
        bound = norm_bound(stages)
        if bound > 0 and max(abs(x) for r in before for x in r) < DENOISE_REL * bound:
            ops[name] = ([Stage(n_in, n_out, [[] for _ in range(n_out)])], n_in, n_out)
            zero.add(name)
            continue
        clean = []
        for st in stages:
            mx = max((abs(v) for r in st.rows for _, v in r), default=0.0)
            clean.append(Stage(st.n_in, st.n_out, [[(c, v) for c, v in r if abs(v) >= DENOISE_REL * mx]
                                                   for r in st.rows]))
        after = chain_dense(clean)
        err = max(abs(after[i][j] - before[i][j]) for i in range(len(before)) for j in range(len(before[0])))
        if err > DENOISE_REL * bound:
            raise SystemExit(f"denoised {name} moved by {err} (bound {bound})")
        ops[name] = (clean, n_in, n_out)
    return zero


def generate(D, P, out_path):
    el = Element(D, P)
    ops = build_ops(el)
    add_ic_proj(el, ops)
    add_amr_ops(el, ops)
    n_mom = add_face_moment_ops(el, ops)
    zero_ops = denoise(ops)
    N = P + 1
    qst = N ** (D + 1)
    qbd = N ** D
    ns = f"gen_D{D}P{P}"
    hdr = [
        "// Generated by gen_element.py -- do not edit.",
        f"// Element operators for D={D}, P={P} (ADER-DG, modal Legendre, FP64).",
        "#pragma once",
        f"namespace adg {{ namespace {ns} {{",
        "__device__ __constant__ const double MDIAG_[] = {" + ", ".join(lit(v) for v in el.Mdiag) + "};",
        "__device__ __constant__ const double MINV_[] = {" + ", ".join(lit(v) for v in el.Minv) + "};",
        "__device__ __constant__ const double NODES_[] = {" + ", ".join(lit(v) for v in el.nodes) + "};",
        "__device__ __constant__ const double WEIGHTS_[] = {" + ", ".join(lit(v) for v in el.weights) + "};",
        "__device__ __constant__ const float WEIGHTS_F_[] = {" + ", ".join(lit(v) for v in el.weights) + "};",
        "struct Ops {",
        f"  static constexpr int D = {D};",
        f"  static constexpr int P = {P};",
        f"  static constexpr int N = {N};",
        f"  static constexpr int Q = {D + 2};",
        f"  static constexpr int NP_S = {el.Np_s};",
        f"  static constexpr int NP_ST = {el.Np_st};",
        f"  static constexpr int NQ_ST = {qst};",
        f"  static constexpr int NQ_BD = {qbd};",
        f"  static constexpr int NQ_S = {N ** D};",
        f"  static constexpr int NQ_INIT = {N ** D};",
        f"  static constexpr int NM = {n_mom};  // tangential flux moments per face and variable",
        f"  static constexpr double CFL = {lit((1.0 / (2.0 * P + 1.0)) * (1.0 / D))};",
        "  static __device__ __forceinline__ double mdiag(int n) { return MDIAG_[n]; }",
        "  static __device__ __forceinline__ double minv(int n) { return MINV_[n]; }",
        "  static __device__ __forceinline__ double node(int k) { return NODES_[k]; }",
        "  static __device__ __forceinline__ double weight(int k) { return WEIGHTS_[k]; }",
        "  static __device__ __forceinline__ float weight_f(int k) { return WEIGHTS_F_[k]; }",
        f"  static constexpr double WEIGHT_SUM = {lit(sum(el.weights))};  // sum of the GL weights",
    ]
    counts = {}
    for name, op in ops.items():
        code, nops = emit_op(name, op)
        hdr.append(code)
        counts[name] = nops
    # compile-time dispatchers
    def disp(fname, names, params):
        lines = [f"  template <{', '.join('int ' + p for p in params)}, class T = double, class In, class Out>",
                 f"  static __device__ __forceinline__ void {fname}(const In& in, Out out) {{"]
        first = True
        for key, nm in names:
            cond = " && ".join(f"{p} == {v}" for p, v in zip(params, key))
            lines.append(f"    {'if' if first else 'else if'} constexpr ({cond}) {nm}<T>(in, out);")
            first = False
        lines.append("  }")
        return "\n".join(lines)
    hdr.append(disp("proj", [((d,), f"proj{d}") for d in range(D)], ["d"]))
    hdr.append(disp("proj_init", [((d,), f"proj_init{d}") for d in range(D)], ["d"]))
    hdr.append(disp("vol_term", [((d,), f"vol_term{d}") for d in range(D)], ["d"]))
    hdr.append(disp("vol_term_sp", [((d,), f"vol_term_sp{d}") for d in range(D)], ["d"]))
    hdr.append(disp("vol_eval_slice", [((k,), f"vol_eval_slice{k}") for k in range(N)], ["k"]))
    hdr.append(disp("face_slice", [((d, s), f"face_slice{d}{s}") for d in range(D) for s in range(2)], ["d", "s"]))
    hdr.append(disp("face_eval", [((d, s), f"face_eval{d}{s}") for d in range(D) for s in range(2)], ["d", "s"]))
    hdr.append(disp("face_eval_sp", [((d, s), f"face_eval_sp{d}{s}") for d in range(D) for s in range(2)],
                    ["d", "s"]))
    hdr.append(disp("cproj", [((d,), f"cproj{d}") for d in range(D)], ["d"]))
    # proj_init[d] is zero when the flux of the first sweep's initial guess
    # (independent of x_0) is projected with the x_0 derivative: A_0 F = 0
    hdr.append("  static constexpr __host__ __device__ bool proj_init_zero(int d) { return "
               + " || ".join([f"d == {d}" for d in range(D) if f"proj_init{d}" in zero_ops] or ["false"]) + "; }")
    # space-time mode n = (spatial mode st_space(n), time degree st_time(n));
    # time_val(a, k) = P_a(t_k)
    # (constexpr selections rather than arrays, which device code cannot
    # read; called with compile-time arguments inside unrolled loops)
    def select(var, vals, fmt):
        expr = fmt(vals[-1])
        for i in range(len(vals) - 2, -1, -1):
            expr = f"{var} == {i} ? {fmt(vals[i])} : ({expr})"
        return expr
    hdr.append("  static constexpr __host__ __device__ int st_space(int n) { return "
               + select("n", el.st_space, str) + "; }")
    hdr.append("  static constexpr __host__ __device__ int st_time(int n) { return "
               + select("n", el.st_time, str) + "; }")
    tv = [el.val[a][k] for a in range(P + 1) for k in range(N)]
    hdr.append(f"  static constexpr __host__ __device__ float time_val_f(int a, int k) {{ return "
               + select(f"(a * {N} + k)", tv, lambda v: lit(v) + "f") + "; }")
    hdr.append(disp("bd_term", [((d, s), f"bd_term{d}{s}") for d in range(D) for s in range(2)], ["d", "s"]))
    hdr.append(disp("pcf", [((l,), f"pcf{l}") for l in range(1 << D)], ["l"]))
    hdr.append(disp("pfc", [((l,), f"pfc{l}") for l in range(1 << D)], ["l"]))
    hdr.append(disp("pflux", [((d, s, k), f"pflux{d}{s}{k}") for d in range(D) for s in range(2)
                              for k in range(1 << (D - 1))], ["d", "s", "k"]))
    hdr.append(disp("bd_mom", [((d, s), f"bd_mom{d}{s}") for d in range(D) for s in range(2)], ["d", "s"]))
    hdr.append(disp("pflux_mom", [((d, s, k), f"pflux_mom{d}{s}{k}") for d in range(D) for s in range(2)
                                  for k in range(1 << (D - 1))], ["d", "s", "k"]))
    # FP64 instruction counts of the linear stages per column and step: the
    # first sweep from the initial guess, the remaining sweeps, the corrector
    # volume term, the face values (from the slices or from the modes,
    # whichever is cheaper), the face moments (once per face, D faces per
    # element, time integral then face_mom_sp; the boundary terms of the
    # corrector are sign copies of them) and the update
    sweeps = P
    slices_cost = N * sum(counts[f"face_slice{d}{s}"] for d in range(D) for s in range(2))
    modes_cost = sum(counts[f"face_eval{d}{s}"] for d in range(D) for s in range(2))
    nsb = N ** (D - 1)
    nz_init = sum(1 for d in range(D) if f"proj_init{d}" not in zero_ops)  # projections the first sweep runs
    per_col = (counts["wu"] + counts["vol_eval_init"] + sum(counts[f"proj_init{d}"] for d in range(D))
               + 2 * nz_init * el.Np_st
               + (sweeps - 1) * (counts["vol_eval"] + sum(counts[f"proj{d}"] for d in range(D)) + 2 * D * el.Np_st)
               + counts["vol_eval"] + sum(counts[f"vol_term{d}"] for d in range(D))
               + min(slices_cost, modes_cost)
               + D * (counts["face_mom_sp"] + nsb * (N - 1)) + 4 * el.Np_s)
    hdr.append(f"  static constexpr int LINEAR_FP64_PER_COLUMN = {per_col};")
    # face values: extrapolated from the time slices when that is cheaper
    # than evaluating the face traces from the modes
    hdr.append(f"  static constexpr bool FACE_FROM_SLICES = {'true' if slices_cost < modes_cost else 'false'};"
               f"  // {slices_cost} vs {modes_cost} FP64 per column")
    # spatial mode of degree 1 in direction d and 0 in the others (the TVB
    # limiter's slope modes, lin_mode_idx of AmrDG.tpp:174-183)
    lin = []
    for d in range(D):
        lin.append(next(n for n, mi in enumerate(el.mi_s)
                        if mi[d] == 1 and all(mi[a] == 0 for a in range(D) if a != d)))
    hdr.append("  static __device__ __forceinline__ int lin_mode(int d) { return "
               + " : ".join(f"d == {d} ? {lin[d]}" for d in range(D - 1)) + f" : {lin[D - 1]}; }}")
    hdr.append("};")
    hdr.append("}}  // namespace")
    hdr.append("")
    with open(out_path, "w") as f:
        f.write("\n".join(hdr))
    return counts


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out-dir", required=True)
    ap.add_argument("--configs", default="2:1,2:2,2:3,3:1,3:2")
    args = ap.parse_args()
    os.makedirs(args.out_dir, exist_ok=True)
    for cfg in args.configs.split(","):
        D, P = map(int, cfg.split(":"))
        path = os.path.join(args.out_dir, f"elem_D{D}P{P}.cuh")
        counts = generate(D, P, path)
        print(f"D={D} P={P}: " + ", ".join(f"{k}={v}" for k, v in counts.items()), file=sys.stderr)


if __name__ == "__main__":
    main()
