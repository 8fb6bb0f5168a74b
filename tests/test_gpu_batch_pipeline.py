"""Host-buffer batches of at least 1024 TTs (ttg_round_batch) run as a
pipeline of 2-4 plans whose packing, copies and sweeps overlap, split by
estimated cost (two chunks at 1100 TTs, four at 4200, which reuse the two
buffer slots).  The results must be those of the same TTs rounded in
batches below that size, TT by TT and in input order, with every status
clean."""
import pytest

from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("count", [1100, 4200])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_pipelined_batch_matches_small_batches(ttg, prec, count):
    tts = [O.random_uneven(5000 + i, 4, 12, 2, 24) for i in range(count)]
    opts = ttg.RoundOptions(eps=1e-8, precision=ttg.precision[prec])
    res = []
    ys = ttg.round_batch(tts, opts, res)
    assert len(ys) == len(tts) and len(res) == len(tts)
    small = []
    for c in range(0, len(tts), 500):
        small += ttg.round_batch(tts[c:c + 500], opts)
    for i, (a, b) in enumerate(zip(ys, small)):
        assert O.ranks(a) == O.ranks(b), i
        assert O.rel_err(a, b) <= 1e-12, i
        assert res[i].status == 0 and res[i].converged, i
    for i in (0, 537, count - 1):
        ref = O.round(tts[i], 1e-8)
        assert O.ranks(ys[i]) == O.ranks(ref) and O.rel_err(ys[i], ref) <= 1e-10, i
