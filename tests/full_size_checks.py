"""Size-independent checks shared by the full-size GPU tests
(tests/test_zzz_full_size.py) and their reduced-size CPU twins
(tests/test_full_size_logic.py, which run the same code with the oracle as
the backend).

At full size the oracle's own rel_err (a CPU QR sweep of the rank-2r
difference) would take minutes, so the error of a rounding is measured on
the device: ||y - t|| is the norm the R->L QR sweep of round(sub(y, t))
reports (round_result.norm), rounded with max_rank = 1 so that the
left-to-right sweep after it is cheap.  A QR-based norm of the difference
carries an error of ~1e-16 ||t|| (no cancellation of squared norms), so it
resolves relative errors far below the 1e-8 bound.
"""
import numpy as np


def feasible_ranks(modes, cap):
    """Bond ranks of a TT with no truncation: min(prod left modes, prod right
    modes, cap), 1 at both ends."""
    d = len(modes)
    out = []
    for k in range(d + 1):
        left = int(np.prod(modes[:k], dtype=np.float64)) if k else 1
        right = int(np.prod(modes[k:], dtype=np.float64)) if k < d else 1
        out.append(int(min(left, right, cap)))
    return out


def config3(T, d=40, n=8, r=128):
    """round(a + b + ones): a, b random rank r (seeds 46/47), cores scaled
    1/sqrt(r_k n_k); ones scaled 1/sqrt(n) per core; interior rank 2r + 1."""
    a = T.random([n] * d, r, 46, fan_in_scale=True)
    b = T.random([n] * d, r, 47, fan_in_scale=True)
    ones = [c / np.sqrt(n) for c in T.ones([n] * d)]
    return T.add(T.add(a, b), ones)


def qr_norms(T, ts, schedule=0):
    """||t_i|| of each TT from one batched R->L QR sweep (max_rank = 1 keeps
    the truncation sweep after it cheap).  schedule: the library's schedule
    code (0 = automatic, 1 = one CTA per TT)."""
    res = []
    T.round_batch(ts, T.RoundOptions(eps=0.0, max_rank=1, schedule=schedule), res)
    assert all(r.status == 0 for r in res)
    return [r.norm for r in res]


def diff_norms(T, ys, ts, schedule=0):
    """||y_i - t_i|| for each pair."""
    return qr_norms(T, [T.sub(y, t) for y, t in zip(ys, ts)], schedule)


def check_round_keeps_tensor(T, t, eps, precision, expected_ranks):
    """round(t) with no truncation possible: the expected ranks, and
    ||round(t) - t|| <= eps ||t||.  Returns the relative error."""
    info = T.RoundResult()
    y = T.round(t, T.RoundOptions(eps=eps, precision=precision), info)
    ranks = [y[0].shape[0]] + [c.shape[-1] for c in y]
    assert ranks == expected_ranks, (ranks, expected_ranks)
    assert info.status == 0 and info.norm > 0.0
    rel = diff_norms(T, [y], [t])[0] / info.norm
    assert rel <= eps, rel
    return rel


def check_batch(T, ts, eps, precision, every=16):
    """A batch round: every status clean, every rank <= the input's, and
    ||y - t|| <= eps ||t|| on every `every`-th member.  Returns (ys, worst)."""
    res = []
    ys = T.round_batch(ts, T.RoundOptions(eps=eps, precision=precision), res)
    assert len(ys) == len(ts)
    for y, t, r in zip(ys, ts, res):
        assert r.status == 0
        ry = [y[0].shape[0]] + [c.shape[-1] for c in y]
        rt = [t[0].shape[0]] + [c.shape[-1] for c in t]
        assert len(ry) == len(rt) and all(1 <= a <= b for a, b in zip(ry, rt))
    sel = list(range(0, len(ts), every))
    norms = diff_norms(T, [ys[i] for i in sel], [ts[i] for i in sel], schedule=1)
    worst = max(n / res[i].norm for n, i in zip(norms, sel))
    assert worst <= eps, worst
    return ys, worst
