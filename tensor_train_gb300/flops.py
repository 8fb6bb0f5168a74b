"""Algorithmic FLOP model of the rounding sweeps.

Counts the flops of the reference's algorithm (not of any particular
implementation), from shapes and ranks:
  qr(m, c)     = 4 m c^2 - (4/3) c^3     Householder R + explicit thin Q (m >= c)
  svd_sq(c)    = 21 c^3                  Golub-Reinsch U, S, V of a c x c matrix
  svd(m, c)    = 4 m^2 c + 8 m c^2 + 9 c^3 (m >= c; swapped when m < c)
  gemm(m,k,n)  = 2 m k n
R->L QR sweep (orthogonalize.hpp:63-100), norm, L->R truncated-SVD sweep
(truncate.hpp:61-99) with QR-condense when rows >= 2 cols, norm balancing
(tt_round.hpp:65-124) counted as 4 flops per output entry.
"""
from __future__ import annotations


def qr(m, c):
    return 4.0 * m * c * c - (4.0 / 3.0) * c ** 3


def svd_sq(c):
    return 21.0 * c ** 3


def svd(m, c):
    if m < c:
        m, c = c, m
    return 4.0 * m * m * c + 8.0 * m * c * c + 9.0 * c ** 3


def gemm(m, k, n):
    return 2.0 * m * k * n


def round_steps(modes, ranks_in, ranks_out):
    """The step shapes of one round, in sweep order: ("rqr", m, c, r_eff,
    h_prev) for the R->L QR steps and ("svd", rows, cols, r_new, w_next) for
    the L->R truncation steps (the shapes the reference's sweep meets)."""
    d = len(modes)
    steps = []
    if d <= 1:
        return steps
    n = list(modes)
    r = list(ranks_in)
    for k in range(d - 1, 0, -1):
        m, c = n[k] * r[k + 1], r[k]
        e = min(m, c)
        steps.append(("rqr", m, c, e, r[k - 1] * n[k - 1]))
        r[k] = e
    for k in range(d - 1):
        rows, cols = r[k] * n[k], r[k + 1]
        rnew = ranks_out[k + 1]
        steps.append(("svd", rows, cols, rnew, n[k + 1] * r[k + 2]))
        r[k + 1] = rnew
    return steps


def round_flops(modes, ranks_in, ranks_out):
    """F_round of one TT with mode sizes `modes`, input ranks and output ranks."""
    d = len(modes)
    if d <= 1:
        return 0.0
    F = 0.0
    for kind, a, b, c, w in round_steps(modes, ranks_in, ranks_out):
        if kind == "rqr":
            F += qr(max(a, b), min(a, b)) + gemm(w, b, c)
        else:
            rows, cols, rnew = a, b, c
            if rows >= 2 * cols:
                F += qr(rows, cols) + svd_sq(cols) + gemm(rows, cols, cols)
            else:
                F += svd(rows, cols)
            F += gemm(rnew, cols, w)
    F += 2.0 * _norm_entries(modes, ranks_in)
    F += 4.0 * sum(ranks_out[k] * modes[k] * ranks_out[k + 1] for k in range(d))
    return F


def _norm_entries(modes, ranks_in):
    """Entries of core 0 after the R->L sweep: n_0 * r_1' with r_1' the
    (possibly shrunk) first bond."""
    r = list(ranks_in)
    n = list(modes)
    for k in range(len(n) - 1, 0, -1):
        r[k] = min(n[k] * r[k + 1], r[k])
    return r[0] * n[0] * r[1]


def matvec_flops(A_ranks, x_ranks, m, n):
    """Sum_k gemm(rA_k m_k rA_{k+1}, n_k, rx_k rx_{k+1}) (tt_matrix_apply.hpp:40-125)."""
    return sum(gemm(A_ranks[k] * m[k] * A_ranks[k + 1], n[k], x_ranks[k] * x_ranks[k + 1])
               for k in range(len(m)))


def eval_flops(ranks, M):
    """M * sum_{k>=1} 2 r_k r_{k+1} (tt_eval.hpp:32-77)."""
    return M * sum(2.0 * ranks[k] * ranks[k + 1] for k in range(1, len(ranks) - 1))
