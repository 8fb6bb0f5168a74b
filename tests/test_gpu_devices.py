"""The multi-device batch entries on the GPU (ttg_round_batch_devices,
ttg_eval_batch_devices).  On a one-GPU host the device list repeats device
0: the partition, the per-part calls from their own host threads and the
gather in input order are the same code as on several GPUs."""
import numpy as np
import pytest

from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_round_batch_devices_matches_one_device(ttg, prec):
    tts = [O.random_uneven(3000 + i, 8, 16, 4, 48) for i in range(40)]
    opts = ttg.RoundOptions(eps=1e-8, precision=ttg.precision[prec], schedule=ttg.schedule.per_tt)
    res1, res2 = [], []
    ys1 = ttg.round_batch(tts, opts, res1)
    ys2 = ttg.round_batch(tts, opts, res2, devices=[0, 0, 0])
    part_of, _ = ttg.shard_plan(tts, 3)
    assert set(part_of.tolist()) == {0, 1, 2}
    for i, (a, b) in enumerate(zip(ys1, ys2)):
        assert O.ranks(a) == O.ranks(b), i
        assert O.rel_err(b, a) <= 1e-12, i
        assert res2[i].status == 0 and res2[i].converged
        assert abs(res2[i].norm - res1[i].norm) <= 1e-13 * res1[i].norm
    # against the oracle on a few members
    for i in (0, 17, 39):
        ref = O.round(tts[i], 1e-8)
        assert O.ranks(ys2[i]) == O.ranks(ref) and O.rel_err(ys2[i], ref) <= 1e-10


def test_eval_batch_devices_matches_one_device(ttg):
    t = O.random([4] * 12, 16, 48, fan_in_scale=True)
    idx = np.random.default_rng(5).integers(0, 4, size=(10007, 12)).astype(np.int32)
    v1 = ttg.eval_batch(t, idx)
    v3 = ttg.eval_batch(t, idx, devices=[0, 0, 0])
    assert np.array_equal(v1, v3)
    ref = O.eval_batch(t, idx[:257])
    assert np.max(np.abs(v3[:257] - ref)) <= 1e-12 * max(1.0, np.max(np.abs(ref)))
    # fewer samples than devices: empty slices are fine
    assert np.array_equal(ttg.eval_batch(t, idx[:2], devices=[0, 0, 0]), v1[:2])


def test_devices_argument_errors(ttg):
    tts = [O.random_uneven(3000 + i, 8, 10, 4, 8) for i in range(3)]
    with pytest.raises(ttg.TTGError) as e:
        ttg.round_batch(tts, ttg.RoundOptions(eps=1e-8), devices=[0, 4096])
    assert e.value.status == 1
    with pytest.raises(ttg.TTGError):
        ttg.eval_batch(tts[0], np.zeros((4, len(tts[0])), np.int32), devices=[-1])
