"""Deterministic append sets for add-haplotypes (shared by the golden
generator tests/golden/make_append_golden.py and the tests that read its
fixtures).

Randomness is gfaz_gb300.synthetic.rng_u64 (integer splitmix64 over
counters), so a set is the same on every machine and numpy version.

Path sets (appended to a container of P-lines): an exact copy of a stored
path, a 1%-mutated copy, a reversed copy, a concatenation of six paths,
random steps, a single step, and repetitive paths - (a,b) x 6000, a 7-step
motif x 3000, (5,6) x 9000 - whose pairings cascade through the rulebook's
layers.  Walk sets (appended to a container with W-lines): a copy of a
stored walk under new fields, a mutated copy, a reversed copy, a repetitive
walk and a one-step walk.  Entries whose delta-coded values would reach the
rule-id region are dropped, as the reference rejects them
(add_haplotypes_workflow.cpp:447-465)."""
from __future__ import annotations

import numpy as np

from gfaz_gb300.synthetic import rng_u64


def p_line(name: str, steps) -> str:
    return "P\t%s\t%s\t*\n" % (name, ",".join("%d%s" % (abs(int(v)), "+" if v > 0 else "-") for v in steps))


def w_line(sample: str, hap: int, seqid: str, start: int, end: int, steps) -> str:
    st = "*" if start < 0 else str(start)
    en = "*" if end < 0 else str(end)
    return "W\t%s\t%d\t%s\t%s\t%s\t%s\n" % (sample, hap, seqid, st, en,
                                            "".join(("<" if v < 0 else ">") + str(abs(int(v))) for v in steps))


def fits(p, delta_round: int, min_id: int) -> bool:
    """Whether the delta-coded traversal stays below the rule id region."""
    x = np.asarray(p, np.int64)
    if len(x) == 0:
        return True
    for _ in range(delta_round):
        x = np.concatenate([x[:1], np.diff(x)])
    return int(np.abs(x).max()) < min_id


def _mutate(p, hi: int, seed: int, stream: int, per: int = 100):
    m = np.asarray(p, np.int32).copy()
    k = max(1, len(m) // per)
    u = rng_u64(seed, stream, 2 * k)
    idx = (u[:k] % np.uint64(len(m))).astype(np.int64)
    m[idx] = (1 + u[k:] % np.uint64(max(1, hi // 2))).astype(np.int32)
    return m


def _random_steps(n: int, hi: int, seed: int, stream: int):
    u = rng_u64(seed, stream, n)
    v = (1 + (u >> np.uint64(1)) % np.uint64(max(1, hi // 2))).astype(np.int32)
    return np.where((u & np.uint64(1)) == 1, -v, v).astype(np.int32)


def path_set(raw, off, n_paths: int, seed: int = 11):
    """The appended P-line traversals for a container whose first n_paths
    traversals (raw[off[t]:off[t+1]]) are its paths."""
    paths = [np.asarray(raw[int(off[i]):int(off[i + 1])], np.int32) for i in range(n_paths)]
    paths = [p for p in paths if len(p) >= 8] or paths
    hi = int(np.abs(np.asarray(raw)).max())
    out = [paths[0].copy(),
           _mutate(paths[1 % len(paths)], hi, seed, 1),
           -paths[2 % len(paths)][::-1],
           np.concatenate(paths[:6]),
           _random_steps(5000, hi, seed, 2),
           np.array([7], np.int32),
           np.tile(paths[3 % len(paths)][:2], 6000),
           np.tile(paths[4 % len(paths)][:7], 3000),
           np.tile(np.array([5, 6], np.int32), 9000)]
    return [np.ascontiguousarray(p, np.int32) for p in out]


def walk_set(raw, off, n_paths: int, seed: int = 13):
    """The appended W-line traversals, each (steps, sample, hap, seqid,
    start, end), for a container whose traversals after the first n_paths
    are its walks."""
    walks = [np.asarray(raw[int(off[i]):int(off[i + 1])], np.int32) for i in range(n_paths, len(off) - 1)]
    walks = [w for w in walks if len(w) >= 2] or walks
    hi = int(np.abs(np.asarray(raw)).max())
    w0 = walks[0]
    w1 = walks[1 % len(walks)]
    w2 = walks[2 % len(walks)]
    out = [(w0.copy(), "appS0", 0, "chrA", 0, 30 * len(w0)),
           (_mutate(w1, hi, seed, 1, per=10), "appS1", 1, "chrA", -1, -1),
           (-w2[::-1], "appS1", 2, "chrB", 5, 5 + 30 * len(w2)),
           (np.tile(w0[:3], 500), "appS2", 0, "chrC", -1, -1),
           (np.array([2], np.int32), "appS3", 0, "chrD", 0, 1)]
    return [(np.ascontiguousarray(s, np.int32), a, h, q, st, en) for s, a, h, q, st, en in out]


# (case, kind) of the golden append fixtures (tests/golden/append.*): P-line
# sets on the path containers of every delta_round / rounds setting, W-line
# sets on the containers that hold walks.
GOLDEN_CASES = [("cfg1", "P"), ("cfg1_mini_d0", "P"), ("cfg1_mini_d2_r3", "P"), ("cfg1_mini_r1", "P"),
                ("rich", "W"), ("tiny", "W")]


def golden_append(case: str, kind: str, manifest: dict):
    """The append set of a golden case: (text of the append file, list of
    appended traversals as int32 arrays, the container's pre-entropy arrays
    from its golden .npz)."""
    from conftest import golden_raw
    meta = manifest["cases"][case]
    raw, off, z = golden_raw(case, meta)
    npaths = int(z["n_paths"][0])
    dr = int(z["delta_round"][0])
    min_id = int(z["layers"][0, 1])
    if kind == "P":
        steps = [p for p in path_set(raw, off, npaths) if fits(p, dr, min_id)]
        text = "".join(p_line("app%d" % i, p) for i, p in enumerate(steps))
    else:
        rows = [w for w in walk_set(raw, off, npaths) if fits(w[0], dr, min_id)]
        steps = [r[0] for r in rows]
        text = "".join(w_line(a, h, q, st, en, s) for s, a, h, q, st, en in rows)
    return text, steps, z
