"""The schedule autotuner on CPU, with a model of the timings in place of the
GPU timer: which candidates it times, in which order, what it keeps, and how
its choices are cached and turned back into configs."""
import json

import numpy as np
import pytest

from wavefiber3d_gb300 import api, autotune


def make(depth, prec):
    return api.Config(depth, [24] * (depth + 1), [48] * (depth + 1), [-1e-6] * 3, [1e-6] * 3, precision=prec)


def samples(n):
    return np.zeros((7, n), np.float32)


def illum(n_inc=1, pol=api.PO_POL_TM, lams=(500e-9,)):
    return api.Illumination(list(lams), [0.1] * n_inc, [0.2] * n_inc, pol)


class Model:
    """ms = base(depth, precision) + leaf(kernel, slots) + tile term; records every config timed."""

    def __init__(self, base, leaf=None, tile=None):
        self.base, self.leaf, self.tile = base, leaf or {}, tile or {}
        self.seen = []

    def __call__(self, cfg, samples, il):
        self.seen.append(cfg)
        return (self.base[(cfg.max_depth, cfg.precision)] + self.leaf.get((cfg.leaf_kernel, cfg.leaf_slots), 0.0)
                + self.tile.get(cfg.interp_tile, 0.0))


F32, BF = api.PO_PREC_FP32, api.PO_PREC_SPLIT_BF16
WARP, TC = api.PO_LEAF_WARP, api.PO_LEAF_TCGEN05


def test_heuristic_depth_and_class_key():
    assert autotune.heuristic_depth(48) == 0 and autotune.heuristic_depth(48 * 8 ** 3) == 3
    assert autotune.heuristic_depth(10 ** 12) == autotune.MAX_DEPTH
    # patterns per wavelength are part of the class: the leaf schedule depends on them
    assert autotune.class_key(20000, 4e-6, 5e-7, 1) != autotune.class_key(20000, 4e-6, 5e-7, 64)
    assert autotune.class_key(20000, 4e-6, 5e-7, 1) == autotune.class_key(21000, 4.1e-6, 5e-7, 1)
    assert autotune.patterns_per_lambda(illum(5, api.PO_POL_TM | api.PO_POL_TE, (4e-7, 5e-7))) == 10


@pytest.mark.parametrize("g,expect", [
    (1, [(WARP, 0), (TC, 8)]),
    (8, [(WARP, 0), (TC, 8)]),
    (20, [(WARP, 0), (TC, 16), (TC, 24)]),
    (64, [(WARP, 0), (TC, 16), (TC, 32), (TC, 64)]),
    (128, [(WARP, 0), (TC, 16), (TC, 32), (TC, 64)]),
])
def test_leaf_schedules(g, expect):
    assert autotune.leaf_schedules(g) == expect


def test_search_order_and_choice():
    """Depth/precision first (heuristic depth 2 and its neighbours), then the
    leaf schedules of the split-BF16 winner, then the theta tiles."""
    base = {(1, F32): 9.0, (1, BF): 8.0, (2, F32): 7.0, (2, BF): 5.0, (3, F32): 6.0, (3, BF): 5.5}
    m = Model(base, leaf={(WARP, 0): 0.5, (TC, 16): -0.2, (TC, 32): -0.6, (TC, 64): -0.4}, tile={16: -0.1})
    t = autotune.Autotuner(timer=m)
    n = 48 * 64
    ch = t.choose(samples(n), illum(32, api.PO_POL_TM | api.PO_POL_TE), make, 4e-6)
    assert ch == {"depth": 2, "precision": BF, "tile": 16, "leaf_kernel": TC, "leaf_slots": 32,
                  "ms": pytest.approx(5.0 - 0.6 - 0.1)}
    stage1 = [(c.max_depth, c.precision) for c in m.seen[:6]]
    assert stage1 == [(1, F32), (1, BF), (2, F32), (2, BF), (3, F32), (3, BF)]
    assert all(c.leaf_kernel == api.PO_LEAF_AUTO and c.interp_tile == 0 for c in m.seen[:6])
    stage2 = [(c.leaf_kernel, c.leaf_slots) for c in m.seen[6:10]]
    assert stage2 == autotune.leaf_schedules(64)
    assert all((c.max_depth, c.precision) == (2, BF) for c in m.seen[6:])
    assert [(c.interp_tile, c.leaf_kernel, c.leaf_slots) for c in m.seen[10:]] == [(8, TC, 32), (16, TC, 32)]
    assert t.trials == len(m.seen) == 12
    cfg = autotune.apply(make(ch["depth"], ch["precision"]), ch)
    assert (cfg.interp_tile, cfg.leaf_kernel, cfg.leaf_slots) == (16, TC, 32)
    assert cfg.to_c().leaf_slots == 32 and cfg.to_c().leaf_kernel == TC


def test_fp32_winner_keeps_automatic_leaves():
    """An FP32 tree winner is not offered leaf schedules (they apply to split
    BF16 only); a slower schedule never replaces the best."""
    base = {(0, F32): 9.0, (1, F32): 3.0, (1, BF): 4.0, (2, F32): 5.0, (2, BF): 6.0}
    m = Model(base, tile={8: 1.0, 16: 2.0})
    ch = autotune.Autotuner(timer=m).choose(samples(48 * 8), illum(), make, 1e-6)
    assert (ch["depth"], ch["precision"], ch["tile"], ch["leaf_kernel"]) == (1, F32, 0, api.PO_LEAF_AUTO)
    assert all(c.leaf_kernel == api.PO_LEAF_AUTO for c in m.seen)
    assert len(m.seen) == 5 + 2


def test_depth0_winner_tries_nothing_else():
    m = Model({(0, F32): 1.0, (1, F32): 2.0, (1, BF): 3.0})
    ch = autotune.Autotuner(timer=m).choose(samples(40), illum(), make, 1e-6)
    assert ch["depth"] == 0 and len(m.seen) == 3


def test_cache_per_class_and_json_round_trip(tmp_path):
    base = {(d, p): 10.0 - d - p for d in range(4) for p in (F32, BF)}
    m = Model(base)
    path = tmp_path / "tune.json"
    t = autotune.Autotuner(cache_path=path, timer=m)
    a = t.choose(samples(48 * 64), illum(), make, 4e-6)
    n1 = len(m.seen)
    assert t.choose(samples(48 * 66), illum(), make, 4.05e-6) == a  # same class: cached
    assert len(m.seen) == n1
    t.choose(samples(48 * 64), illum(16), make, 4e-6)  # 16 patterns per wavelength: a new class
    assert len(m.seen) > n1
    t.save()
    saved = json.loads(path.read_text())
    assert len(saved) == 2
    t2 = autotune.Autotuner(cache_path=path, timer=lambda *a: pytest.fail("timed a cached class"))
    assert t2.choose(samples(48 * 64), illum(), make, 4e-6) == a
