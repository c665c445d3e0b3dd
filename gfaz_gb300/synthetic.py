"""Seeded synthetic pangenome graphs of the benchmark shapes.

The published datasets (chr1, chr6, HPRC ...) are not available, so seeded
synthetic graphs with their shapes stand in for them:

* ``cfg1`` - linear backbone with a 2-allele bubble every 10 segments, 16
  P-lines, 2% of bubbles traversed in reverse (small, CPU-runnable case).
* ``cfg2`` - chromosome-scale: bubbles every 6 segments with 2-4 alleles
  chosen Zipf(1.2), 5% of bubbles carry a structural-variant detour of
  10-200 segments, 90 haplotypes of ~6M steps, 1% reversed alleles.
* ``cfg3`` - 2M-segment bubble graph with 2,000 W-lines whose step counts
  are lognormal (median 50k, sigma 2, clamped to [100, 20M]).
* ``cfg4`` - whole-genome shape: 24 independent components built by the
  config-1 rules, 180 haplotypes each walking every component once (4,320
  W-lines), 3.6B steps in all.  The shape's stated 40M segments and ~20M
  steps per haplotype cannot both hold for a config-1 graph (a haplotype
  takes 11 of every 12 segments); the step count is kept, which gives ~21.8M
  segments.

Randomness is integer-only (splitmix64 over counters, comparisons against
exact integer thresholds) so that the same seed yields the same graph on
every machine and numpy version.  Only the Zipf and lognormal thresholds
are derived from floating point once, at 2**32 granularity.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from fractions import Fraction

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        x = (x + np.uint64(0x9E3779B97F4A7C15)) & _M64
        z = x
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M64
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M64
        return z ^ (z >> np.uint64(31))


def rng_u64(seed: int, stream: int, n: int) -> np.ndarray:
    """n pseudo-random uint64 values for (seed, stream)."""
    base = _splitmix(np.array([(seed * 0x632BE59BD9B4E019 + stream * 0xD1B54A32D192ED03)
                               & 0xFFFFFFFFFFFFFFFF], dtype=np.uint64))[0]
    with np.errstate(over="ignore"):
        ctr = (np.arange(n, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15) + base) & _M64
    return _splitmix(ctr)


def _bernoulli(u: np.ndarray, num: int, den: int) -> np.ndarray:
    return (u % np.uint64(den)) < np.uint64(num)


_GEOM_CACHE: dict = {}


def _geometric(u: np.ndarray, mean: int, kmax: int = 2000) -> np.ndarray:
    """Geometric lengths >= 1 with the given mean (p = 1/mean), integer-only:
    thresholds are the exact CDF (1 - (1-p)^k) scaled to 2**53."""
    key = (mean, kmax)
    if key not in _GEOM_CACHE:
        q = Fraction(mean - 1, mean)
        thr = []
        acc = Fraction(1)
        for _ in range(kmax):
            acc *= q
            thr.append(((Fraction(1) - acc) * (1 << 53)).__floor__())
        _GEOM_CACHE[key] = np.array(thr, dtype=np.uint64)
    thr = _GEOM_CACHE[key]
    v = u >> np.uint64(11)
    return (np.searchsorted(thr, v, side="right") + 1).astype(np.int64)


def _zipf_thresholds(k: int, s: float) -> np.ndarray:
    w = [1.0 / (i ** s) for i in range(1, k + 1)]
    tot = sum(w)
    acc, thr = 0.0, []
    for x in w[:-1]:
        acc += x
        thr.append(int(acc / tot * (1 << 32)))
    return np.array(thr, dtype=np.uint64)


@dataclass
class Graph:
    """Host-side synthetic graph; traversals are 1-based signed node IDs."""

    seq_lengths: np.ndarray            # per segment (index 0 = node 1)
    seq_seed: int
    links: np.ndarray                  # (L, 2) from/to node IDs, both '+'
    paths: list = field(default_factory=list)   # list of int32 arrays
    path_names: list = field(default_factory=list)
    walks: list = field(default_factory=list)
    walk_meta: list = field(default_factory=list)  # (sample, hap, seqid, start, end)
    header: str = "H\tVN:Z:1.1"

    @property
    def num_segments(self) -> int:
        return int(self.seq_lengths.shape[0])

    def flat(self):
        """(steps int32, offsets uint64) over paths then walks."""
        seqs = list(self.paths) + list(self.walks)
        lens = np.array([len(s) for s in seqs], dtype=np.uint64)
        off = np.zeros(len(seqs) + 1, dtype=np.uint64)
        np.cumsum(lens, out=off[1:])
        steps = np.concatenate(seqs).astype(np.int32) if seqs else np.zeros(0, np.int32)
        return steps, off

    def sequences(self) -> bytes:
        total = int(self.seq_lengths.sum())
        u = rng_u64(self.seq_seed, 7, total)
        return np.frombuffer(b"ACGT", dtype=np.uint8)[(u & np.uint64(3)).astype(np.int64)].tobytes()

    def to_gfa(self) -> bytes:
        """GFA v1 text: H, S, L, P, W lines (tab separated)."""
        out = [self.header.encode() + b"\n"]
        seq = self.sequences()
        pos = 0
        for i, ln in enumerate(self.seq_lengths.tolist()):
            out.append(b"S\t%d\t%s\n" % (i + 1, seq[pos:pos + ln]))
            pos += ln
        for a, b in self.links.tolist():
            out.append(b"L\t%d\t+\t%d\t+\t0M\n" % (a, b))
        for name, p in zip(self.path_names, self.paths):
            steps = ",".join(f"{abs(v)}{'-' if v < 0 else '+'}" for v in p.tolist())
            out.append(f"P\t{name}\t{steps}\t*\n".encode())
        for (sample, hap, seqid, start, end), w in zip(self.walk_meta, self.walks):
            steps = "".join(f"{'<' if v < 0 else '>'}{abs(v)}" for v in w.tolist())
            s = "*" if start < 0 else str(start)
            e = "*" if end < 0 else str(end)
            out.append(f"W\t{sample}\t{hap}\t{seqid}\t{s}\t{e}\t{steps}\n".encode())
        return b"".join(out)


def _expand_runs(start: np.ndarray, length: np.ndarray, rev: np.ndarray) -> np.ndarray:
    """Concatenate runs of consecutive IDs start..start+len-1; reversed runs
    are walked backwards with negated IDs."""
    total = int(length.sum())
    roff = np.zeros(len(length), dtype=np.int64)
    np.cumsum(length[:-1], out=roff[1:])
    idx = np.arange(total, dtype=np.int64) - np.repeat(roff, length)
    s = np.repeat(start, length)
    r = np.repeat(rev, length)
    ln = np.repeat(length, length)
    ids = np.where(r, s + (ln - 1 - idx), s + idx)
    return np.where(r, -ids, ids).astype(np.int32)


def cfg1(seed: int = 1, n_backbone: int = 20000, bubble_every: int = 10, n_paths: int = 16,
         rev_num: int = 2, rev_den: int = 100, seq_mean: int = 30) -> Graph:
    """Backbone of n_backbone segments, a 2-allele bubble after every
    bubble_every backbone segments; each path walks the whole backbone and
    picks an allele with p=0.5; rev_num/rev_den of the bubbles are walked
    with '-' orientation."""
    nblk = n_backbone // bubble_every
    blk = bubble_every + 2
    nseg = nblk * blk
    base = np.arange(nblk, dtype=np.int64) * blk + 1
    lens = _geometric(rng_u64(seed, 1, nseg), seq_mean)
    links = []
    bb_from = (base[:, None] + np.arange(bubble_every - 1)[None, :]).ravel()
    links.append(np.stack([bb_from, bb_from + 1], 1))
    last = base + bubble_every - 1
    a1, a2 = last + 1, last + 2
    links.append(np.stack([last, a1], 1))
    links.append(np.stack([last, a2], 1))
    nxt = base[1:]
    links.append(np.stack([a1[:-1], nxt], 1))
    links.append(np.stack([a2[:-1], nxt], 1))
    g = Graph(seq_lengths=lens, seq_seed=seed, links=np.concatenate(links).astype(np.int64))
    for p in range(n_paths):
        u = rng_u64(seed, 100 + p, 2 * nblk)
        choice = (u[:nblk] & np.uint64(1)).astype(np.int64)
        rev = _bernoulli(u[nblk:] >> np.uint64(1), rev_num, rev_den)
        starts = np.empty(2 * nblk, np.int64)
        lengths = np.empty(2 * nblk, np.int64)
        revs = np.zeros(2 * nblk, bool)
        starts[0::2], lengths[0::2] = base, bubble_every
        starts[1::2], lengths[1::2], revs[1::2] = last + 1 + choice, 1, rev
        g.paths.append(_expand_runs(starts, lengths, revs))
        g.path_names.append(f"hap{p}")
    return g


def cfg2_stream(seed: int = 2, n_segments: int = 8_000_000, n_paths: int = 90,
                bubble_every: int = 6, detour_pct: int = 5, rev_pct: int = 1,
                zipf_s: float = 1.2):
    """Chromosome-scale traversal stream (no text): returns (steps int32,
    offsets uint64, num_segments).  Block layout: bubble_every backbone
    segments, then k in {2,3,4} alleles; in detour blocks allele 0 is a chain
    of 10-200 segments.  Each path takes every block, the allele by
    Zipf(zipf_s), and walks the allele reversed with rev_pct% probability."""
    # size the block count so segments ~= n_segments
    est_per_block = bubble_every + 3 + detour_pct / 100.0 * 104
    nblk = max(1, int(n_segments / est_per_block))
    u = rng_u64(seed, 1, 3 * nblk)
    k = 2 + (u[:nblk] % np.uint64(3)).astype(np.int64)
    detour = _bernoulli(u[nblk:2 * nblk], detour_pct, 100)
    dlen = 10 + (u[2 * nblk:] % np.uint64(191)).astype(np.int64)
    allele0_len = np.where(detour, dlen, 1)
    seg_per_blk = bubble_every + (k - 1) + allele0_len
    base = np.zeros(nblk, np.int64)
    np.cumsum(seg_per_blk[:-1], out=base[1:])
    base += 1
    nseg = int(seg_per_blk.sum())
    thr = {kk: _zipf_thresholds(kk, zipf_s) for kk in (2, 3, 4)}

    def one_path(p):
        r = rng_u64(seed, 1000 + p, 2 * nblk)
        hi = r[:nblk] >> np.uint64(32)
        choice = np.zeros(nblk, np.int64)
        for kk, t in thr.items():
            m = k == kk
            choice[m] = np.searchsorted(t, hi[m], side="right")
        rev = _bernoulli(r[nblk:], rev_pct, 100)
        a_start = np.where(choice == 0, base + bubble_every,
                           base + bubble_every + allele0_len + choice - 1)
        a_len = np.where(choice == 0, allele0_len, 1)
        starts = np.empty(2 * nblk, np.int64)
        lengths = np.empty(2 * nblk, np.int64)
        revs = np.zeros(2 * nblk, bool)
        starts[0::2], lengths[0::2] = base, bubble_every
        starts[1::2], lengths[1::2], revs[1::2] = a_start, a_len, rev
        return _expand_runs(starts, lengths, revs)

    paths = _parallel_map(one_path, range(n_paths))
    lens = np.array([len(x) for x in paths], dtype=np.uint64)
    off = np.zeros(n_paths + 1, np.uint64)
    np.cumsum(lens, out=off[1:])
    return np.concatenate(paths), off, nseg


def _parallel_map(fn, items):
    """Order-preserving map over a thread pool (numpy releases the GIL in
    the array kernels used by the generators)."""
    import os
    from concurrent.futures import ThreadPoolExecutor
    items = list(items)
    workers = max(1, min(len(items), os.cpu_count() or 1, 16))
    if workers == 1:
        return [fn(x) for x in items]
    with ThreadPoolExecutor(workers) as ex:
        return list(ex.map(fn, items))


def cfg3_stream(seed: int = 3, n_backbone: int = 1_666_667, n_walks: int = 2000,
                median: float = 5e4, sigma: float = 2.0, lo: int = 100, hi: int = 20_000_000,
                rev_num: int = 2, rev_den: int = 100, max_total: int | None = None):
    """Walk stream over a cfg1-shaped bubble graph (~2M segments): each walk
    starts at a random block and walks forward (wrapping at the end) for a
    lognormal number of steps.  Returns (steps int32, offsets uint64,
    num_segments, walk_meta)."""
    bubble_every = 10
    nblk = n_backbone // bubble_every
    blk = bubble_every + 2
    base = np.arange(nblk, dtype=np.int64) * blk + 1
    u = rng_u64(seed, 1, 2 * n_walks)
    # lognormal via inverse-normal on a 2**32 grid (floating point, once)
    q = ((u[:n_walks] >> np.uint64(32)).astype(np.float64) + 0.5) / float(1 << 32)
    z = np.array([_inv_norm(x) for x in q.tolist()])
    steps_n = np.clip(np.round(median * np.exp(sigma * z)), lo, hi).astype(np.int64)
    if max_total is not None and steps_n.sum() > max_total:
        steps_n = np.maximum(lo, (steps_n * (max_total / steps_n.sum())).astype(np.int64))
    start_blk = (u[n_walks:] % np.uint64(nblk)).astype(np.int64)
    walks, meta = [], []
    per_blk = bubble_every + 1
    for w in range(n_walks):
        n = int(steps_n[w])
        nb = n // per_blk + 2
        bidx = (start_blk[w] + np.arange(nb)) % nblk
        r = rng_u64(seed, 10_000 + w, 2 * nb)
        choice = (r[:nb] & np.uint64(1)).astype(np.int64)
        rev = _bernoulli(r[nb:] >> np.uint64(1), rev_num, rev_den)
        starts = np.empty(2 * nb, np.int64)
        lengths = np.empty(2 * nb, np.int64)
        revs = np.zeros(2 * nb, bool)
        starts[0::2], lengths[0::2] = base[bidx], bubble_every
        starts[1::2], lengths[1::2], revs[1::2] = base[bidx] + bubble_every + choice, 1, rev
        walks.append(_expand_runs(starts, lengths, revs)[:n])
        start = int(start_blk[w]) * 300
        meta.append((f"sample{w // 2}", w % 2 + 1, f"chr{w % 24 + 1}", start, start + n * 30))
    lens = np.array([len(x) for x in walks], dtype=np.uint64)
    off = np.zeros(n_walks + 1, np.uint64)
    np.cumsum(lens, out=off[1:])
    return np.concatenate(walks), off, nblk * blk, meta


def cfg4_stream(seed: int = 4, n_components: int = 24, n_haps: int = 180, line_steps: int = 833_327,
                rev_num: int = 2, rev_den: int = 100):
    """Whole-genome-shaped walk stream: component c holds blocks of 10
    backbone segments followed by a 2-allele bubble; haplotype h walks every
    component from its first block to its last, taking allele (bit of a
    per-(c, h) random stream) reversed with rev_num/rev_den probability.
    W-line (c, h) is traversal h * n_components + c.  line_steps is rounded
    down to whole blocks (11 steps).  Returns (steps int32, offsets uint64,
    num_segments, walk_meta)."""
    bubble_every = 10
    per_blk = bubble_every + 1
    blk = bubble_every + 2
    nblk = max(1, line_steps // per_blk)
    L = nblk * per_blk
    seg_per_comp = nblk * blk
    n_lines = n_components * n_haps
    steps = np.empty(n_lines * L, np.int32)
    cols = np.arange(bubble_every, dtype=np.int64)

    def fill(line):
        h, c = divmod(line, n_components)
        base = 1 + c * seg_per_comp + np.arange(nblk, dtype=np.int64) * blk
        u = rng_u64(seed, 100_000 + line, nblk)
        choice = (u & np.uint64(1)).astype(np.int64)
        rev = _bernoulli(u >> np.uint64(1), rev_num, rev_den)
        out = steps[line * L:(line + 1) * L].reshape(nblk, per_blk)
        out[:, :bubble_every] = base[:, None] + cols[None, :]
        allele = base + bubble_every + choice
        out[:, bubble_every] = np.where(rev, -allele, allele)
        return None

    _parallel_map(fill, range(n_lines))
    off = np.arange(n_lines + 1, dtype=np.uint64) * np.uint64(L)
    meta = []
    for line in range(n_lines):
        h, c = divmod(line, n_components)
        meta.append((f"HG{h // 2:03d}", h % 2 + 1, f"chr{c + 1}", 0, L * 30))
    return steps, off, n_components * seg_per_comp, meta


def serve_paths(seed: int = 5, n_backbone: int = 600_000, n_paths: int = 64, median: float = 2e5,
                sigma: float = 0.5, lo: int = 1000, rev_num: int = 2, rev_den: int = 100):
    """Serving graph: the config-1 bubble graph on a longer backbone, whose
    P-lines are windows of lognormal length (median `median` steps) of a
    config-1 traversal starting at a random block, so that extract requests
    have the serving config's lengths.  Returns (steps int32, offsets
    uint64, names, num_segments, links (L, 2))."""
    bubble_every = 10
    nblk = n_backbone // bubble_every
    blk = bubble_every + 2
    base = np.arange(nblk, dtype=np.int64) * blk + 1
    per_blk = bubble_every + 1
    hi = (nblk - 3) * per_blk  # a window of nb = n // per_blk + 2 blocks fits the backbone
    u = rng_u64(seed, 1, 2 * n_paths)
    q = ((u[:n_paths] >> np.uint64(32)).astype(np.float64) + 0.5) / float(1 << 32)
    z = np.array([_inv_norm(x) for x in q.tolist()])
    steps_n = np.clip(np.round(median * np.exp(sigma * z)), lo, hi).astype(np.int64)
    paths = []
    for p in range(n_paths):
        n = int(steps_n[p])
        nb = n // per_blk + 2
        first = int(u[n_paths + p] % np.uint64(max(1, nblk - nb)))
        bidx = first + np.arange(nb)
        r = rng_u64(seed, 100 + p, 2 * nb)
        choice = (r[:nb] & np.uint64(1)).astype(np.int64)
        rev = _bernoulli(r[nb:] >> np.uint64(1), rev_num, rev_den)
        starts = np.empty(2 * nb, np.int64)
        lengths = np.empty(2 * nb, np.int64)
        revs = np.zeros(2 * nb, bool)
        starts[0::2], lengths[0::2] = base[bidx], bubble_every
        starts[1::2], lengths[1::2], revs[1::2] = base[bidx] + bubble_every + choice, 1, rev
        paths.append(_expand_runs(starts, lengths, revs)[:n])
    lens = np.array([len(x) for x in paths], dtype=np.uint64)
    off = np.zeros(n_paths + 1, np.uint64)
    np.cumsum(lens, out=off[1:])
    last = base + bubble_every - 1
    links = [np.stack([(base[:, None] + np.arange(bubble_every - 1)[None, :]).ravel(),
                       (base[:, None] + np.arange(1, bubble_every)[None, :]).ravel()], 1),
             np.stack([last, last + 1], 1), np.stack([last, last + 2], 1),
             np.stack([last[:-1] + 1, base[1:]], 1), np.stack([last[:-1] + 2, base[1:]], 1)]
    return (np.concatenate(paths).astype(np.int32), off, [f"hap{p}" for p in range(n_paths)], nblk * blk,
            np.concatenate(links).astype(np.int64))


def _inv_norm(p: float) -> float:
    """Acklam's rational approximation of the standard normal quantile."""
    a = [-3.969683028665376e+01, 2.209460984245205e+02, -2.759285104469687e+02,
         1.383577518672690e+02, -3.066479806614716e+01, 2.506628277459239e+00]
    b = [-5.447609879822406e+01, 1.615858368580409e+02, -1.556989798598866e+02,
         6.680131188771972e+01, -1.328068155288572e+01]
    c = [-7.784894002430293e-03, -3.223964580411365e-01, -2.400758277161838e+00,
         -2.549732539343734e+00, 4.374664141464968e+00, 2.938163982698783e+00]
    d = [7.784695709041462e-03, 3.224671290700398e-01, 2.445134137142996e+00,
         3.754408661907416e+00]
    pl = 0.02425
    if p < pl:
        q = math.sqrt(-2 * math.log(p))
        return (((((c[0] * q + c[1]) * q + c[2]) * q + c[3]) * q + c[4]) * q + c[5]) / \
            ((((d[0] * q + d[1]) * q + d[2]) * q + d[3]) * q + 1)
    if p > 1 - pl:
        q = math.sqrt(-2 * math.log(1 - p))
        return -(((((c[0] * q + c[1]) * q + c[2]) * q + c[3]) * q + c[4]) * q + c[5]) / \
            ((((d[0] * q + d[1]) * q + d[2]) * q + d[3]) * q + 1)
    q = p - 0.5
    r = q * q
    return (((((a[0] * r + a[1]) * r + a[2]) * r + a[3]) * r + a[4]) * r + a[5]) * q / \
        (((((b[0] * r + b[1]) * r + b[2]) * r + b[3]) * r + b[4]) * r + 1)


def pw_text_bytes(steps: np.ndarray, off: np.ndarray, names=None) -> int:
    """Exact byte count of the P-lines 'P\\t<name>\\t<id><o>,...\\t*\\n' for the
    given traversals (names default to p<i>)."""
    a = np.abs(steps.astype(np.int64))
    digits = np.ones(a.shape, np.int64)
    for t in (10, 100, 1000, 10**4, 10**5, 10**6, 10**7, 10**8, 10**9):
        digits += a >= t
    n = len(off) - 1
    total = int(digits.sum()) + 2 * len(steps)  # digit + orientation + comma
    lens = np.diff(off.astype(np.int64))
    total -= int((lens > 0).sum())              # no comma after the last step
    if names is None:
        names = [f"p{i}" for i in range(n)]
    total += sum(len(nm) for nm in names) + n * (2 + 1 + 1 + 1 + 1)  # P\t name \t ... \t * \n
    return total
