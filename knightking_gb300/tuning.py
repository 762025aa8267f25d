"""Autotuner of the engine's speed options.

The options (kk_engine_set_option) never change a path, only how fast it is
produced: alias-table layout, the alias build's stream split, node2vec
adjacency test, walk block size, the parking threshold of rejection walks,
walkers per thread, the context's L2 fetch-granularity hint, the walk schedule,
the cursor adjacency of uniform walks and the regroup interval (walkers sorted
by the vertex they stand on every k steps).  The tuner runs a
caller-supplied step (one walk call on the real workload) under candidate
settings and keeps, option by option, the value with the shortest alias-build
plus walk time as the engine's CUDA events measure it (greedy coordinate
descent: each option in turn, the others held at their best so far).
"""

DEFAULT_SPACE = (
    ("alias_layout", (2, 0, 1)),
    ("alias_streams", (3, 4, 2, 1)),
    ("alias_small_lanes", (0, 1)),
    ("node2vec_adjacency", (0, 1)),
    ("walk_block", (256, 128, 64)),
    ("walk_multi", (1, 2, 4)),
    ("walk_park", (20, 0, 12, 28)),
    ("l2_fetch_bytes", (0, 64)),
    ("walk_schedule", (0, 1)),
    ("cursor_adjacency", (0, 1)),
    ("regroup_interval", (0, 16, 4)),
)


def space_for(app, weighted, batch=False):
    """The options that matter for a built-in app: the alias layout only with
    alias tables, the adjacency test only for node2vec; batched walks
    (walk_batch_kernel) neither regroup nor run several walkers per thread."""
    out = []
    for name, vals in DEFAULT_SPACE:
        if name in ("regroup_interval", "walk_multi") and batch:
            continue
        if name in ("alias_layout", "alias_streams", "alias_small_lanes") and not weighted:
            continue
        if name == "node2vec_adjacency" and app != "node2vec":
            continue
        if name == "walk_multi" and app not in ("deepwalk", "ppr"):
            continue
        if name == "walk_park" and app != "metapath":
            continue
        if name == "cursor_adjacency" and weighted:
            continue
        out.append((name, vals))
    return tuple(out)


def autotune(engine, step, space=DEFAULT_SPACE, repeats=2):
    """Tunes `engine` on `step()` (one walk call).  Returns (best, table):
    best maps option -> value (already set on the engine), table lists
    (settings, ms) for every setting timed."""
    best = {name: vals[0] for name, vals in space}
    for name, v in best.items():
        engine.set_option(name, v)
    table = []
    for name, vals in space:
        if len(vals) < 2:
            continue
        timed = {}
        for v in vals:
            engine.set_option(name, v)
            ms = []
            for _ in range(repeats):
                step()
                ms.append(sum(engine.last_timing()[:2]))
            timed[v] = min(ms)
            table.append((dict(best, **{name: v}), timed[v]))
        best[name] = min(timed, key=timed.get)
        engine.set_option(name, best[name])
    return best, table
