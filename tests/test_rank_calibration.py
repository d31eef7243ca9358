"""Host logic of the learned-rank predictor (no GPU): the level-by-level
calibration of CalibratedRankPredictor, the rank target and its inverse."""
import numpy as np

from skelfmm_gb300.rank_model import CalibratedRankPredictor, rank_from_target, rank_target


class _Build:
    """The two attributes of a build the predictor reads."""

    def __init__(self, nboxes):
        self.rank_list = np.zeros(nboxes, dtype=np.int64)


class _Fixed(CalibratedRankPredictor):
    """Estimate taken from a table set per level by the test."""

    def __init__(self, est, **kw):
        super().__init__(**kw)
        self.est = est

    def estimate(self, fmm, lev, boxes, x_lev, off):
        return self.est[lev]


def _off(bs):
    o = np.zeros(len(bs) + 1, dtype=np.int64)
    np.cumsum(bs, out=o[1:])
    return o


def test_rank_target_round_trip():
    bs = np.array([1, 10, 100, 1000, 37])
    r = np.array([0, 3, 57, 200, 37])
    assert np.array_equal(rank_from_target(rank_target(r, bs), bs), r)
    # targets above 0 (rank above the box size) are capped at the box size
    assert np.array_equal(rank_from_target(np.full(5, 0.5), bs), bs)


def test_first_level_takes_the_estimate_plus_margin():
    bs = np.array([200, 300, 50, 0])
    y = rank_target(np.array([100, 150, 40, 0]), bs)
    p = _Fixed({5: y}, margin=16)
    k = p(_Build(10), 5, np.arange(6, 10), None, _off(bs))
    want = np.clip(rank_from_target(y, bs) + 16, 1, np.maximum(bs, 1))
    assert np.array_equal(k, want)
    assert p.shifts[5] == 0.0


def test_calibration_from_the_finished_level():
    rng = np.random.default_rng(0)
    n1 = 400
    bs1 = rng.integers(40, 600, n1)
    y1 = rank_target(np.maximum(bs1 // 3, 1), bs1)
    fmm = _Build(n1 + 100)
    boxes1 = np.arange(100, 100 + n1)
    p = _Fixed({6: y1}, margin=16, calibrate=0.9, calibrate_big=0.995, big_box=256)
    p(fmm, 6, boxes1, None, _off(bs1))
    # level 6 came out with ranks larger than estimated, more so for small y
    actual = np.minimum(np.rint((bs1 + 1) * np.exp2(y1 + 0.3 - 0.2 * y1 + rng.normal(0, 0.05, n1)) - 1), bs1 - 1)
    fmm.rank_list[boxes1] = actual.astype(np.int64)
    fmm.rank_list[boxes1[:7]] = bs1[:7]  # full-rank boxes: left out of the fit
    keep = np.ones(n1, bool)
    keep[:7] = False
    err = rank_target(fmm.rank_list[boxes1], bs1) - y1
    A = np.stack([np.ones(keep.sum()), y1[keep]], 1)
    coef = np.linalg.lstsq(A, err[keep], rcond=None)[0]
    res = err[keep] - A @ coef
    q, qb = np.quantile(res, 0.9), np.quantile(res, 0.995)

    bs0 = np.array([100, 255, 256, 900, 30])
    y0 = rank_target(np.array([30, 80, 80, 250, 29]), bs0)
    p.est[5] = y0
    k = p(fmm, 5, np.arange(5), None, _off(bs0))
    shift = np.maximum(coef[0] + coef[1] * y0 + np.where(bs0 >= 256, qb, q), 0.0)
    want = np.clip(rank_from_target(y0 + shift, bs0) + 16, 1, np.maximum(bs0, 1))
    assert np.array_equal(k, want)
    assert shift[:4].min() > 0.0  # boxes like the fitted ones are raised
    # large boxes take the upper quantile
    assert shift[2] > shift[1]


def test_calibration_needs_the_level_just_below():
    bs = np.array([100, 200, 300])
    y = rank_target(np.array([20, 40, 60]), bs)
    fmm = _Build(20)
    p = _Fixed({7: y, 5: y}, margin=0)
    p(fmm, 7, np.arange(3), None, _off(bs))
    fmm.rank_list[:3] = [90, 190, 290]
    # level 5 does not follow level 7: no correction
    k = p(fmm, 5, np.arange(3, 6), None, _off(bs))
    assert np.array_equal(k, rank_from_target(y, bs))
    # nor for another build
    p2 = _Fixed({7: y, 6: y}, margin=0)
    p2(fmm, 7, np.arange(3), None, _off(bs))
    k2 = p2(_Build(20), 6, np.arange(3, 6), None, _off(bs))
    assert np.array_equal(k2, rank_from_target(y, bs))
