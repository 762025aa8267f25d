"""The autotuner's search (host logic, no GPU): greedy coordinate descent over
engine options against a fake engine whose step time is a known function of
the options."""

from knightking_gb300 import tuning


class FakeEngine:
    def __init__(self, cost):
        self.opts = {}
        self.cost = cost
        self.calls = 0

    def set_option(self, name, value):
        self.opts[name] = value

    def last_timing(self):
        return self.cost(self.opts), 0.0


def test_autotune_picks_the_fastest_value_per_option():
    def cost(o):
        return (10.0 + (2.0 if o.get("alias_layout") == 0 else 0.0) + abs(o.get("walk_block", 256) - 128) / 64.0 +
                (1.0 if o.get("walk_schedule") == 1 else 0.0))
    e = FakeEngine(cost)
    best, table = tuning.autotune(e, lambda: None, (("alias_layout", (0, 1)), ("walk_block", (256, 128, 64)),
                                                   ("walk_schedule", (0, 1))))
    assert best == {"alias_layout": 1, "walk_block": 128, "walk_schedule": 0}
    assert e.opts == best
    assert len(table) == 7


def test_space_for_apps():
    names = lambda sp: [n for n, _ in sp]
    assert "alias_layout" not in names(tuning.space_for("ppr", False))
    assert "node2vec_adjacency" in names(tuning.space_for("node2vec", True))
    assert "node2vec_adjacency" not in names(tuning.space_for("deepwalk", True))
    # parking applies to first-order rejection walks (metapath), alias stream
    # splits only to walks with alias tables
    assert "walk_park" in names(tuning.space_for("metapath", True))
    assert "walk_park" not in names(tuning.space_for("node2vec", True))
    assert "walk_park" not in names(tuning.space_for("deepwalk", True))
    assert "alias_streams" in names(tuning.space_for("deepwalk", True))
    assert "alias_streams" not in names(tuning.space_for("ppr", False))


def test_space_for_batches_leaves_out_single_walk_options():
    names = lambda sp: [n for n, _ in sp]
    assert "regroup_interval" in names(tuning.space_for("deepwalk", True))
    assert "regroup_interval" in names(tuning.space_for("node2vec", True))
    assert "regroup_interval" not in names(tuning.space_for("node2vec", True, batch=True))
    assert "walk_multi" not in names(tuning.space_for("deepwalk", True, batch=True))
    # the first value of every option is the engine's default (off for regrouping)
    assert dict(tuning.space_for("ppr", False))["regroup_interval"][0] == 0
