"""Pure-Python restatement of the reference pangenome growth
(src/workflows/growth_workflow.cpp).

TEST INFRASTRUCTURE ONLY: the checker of the growth tests; the product
package never imports it.

  * groups (:134-240, :296-357): every P/W line its own group, or keys from
    PanSN path names sample#hap#seq (coordinates ":start-end" cleared from
    the last field) and walk columns, first-seen order;
  * coverage (:364-437): a node counts once per group visiting it (ids
    1 .. num_nodes; others ignored);
  * hist[c] = nodes with coverage c; growth[k] = sum over c of hist[c] *
    (1 - prod_{i<c} (N-k-i)/(N-i)), 1 when c >= N or N - c < k
    (:106-118, :439-500), in double precision, c ascending.
"""
from __future__ import annotations

from typing import List, Sequence, Tuple

import numpy as np


def _strip_coords(s: str) -> str:
    colon = s.rfind(":")
    if colon <= 0:
        return s
    dash = s.find("-", colon + 1)
    if dash < 0 or dash == colon + 1 or dash + 1 == len(s):
        return s
    if s[colon + 1:dash].isdigit() and s[dash + 1:].isdigit() and s[colon + 1:dash].isascii() \
            and s[dash + 1:].isascii():
        return s[:colon]
    return s


def _pansn(name: str):
    a = name.find("#")
    if a < 0:
        return _strip_coords(name), None, None
    sample = name[:a]
    b = name.find("#", a + 1)

    def two(hap):
        return (sample, _strip_coords(hap), None) if hap else (sample, None, None)
    if b < 0:
        return two(name[a + 1:])
    if b == a + 1:
        return sample, None, None
    seq = name[b + 1:]
    if not seq or seq[0] == "#":
        return two(name[a + 1:b])
    return sample, name[a + 1:b], _strip_coords(seq)


def path_key(name: str, mode: str) -> str:
    sample, hap, seq = _pansn(name)
    if mode == "sample":
        return sample
    if mode == "sample-hap":
        return sample + "#" + (hap if hap is not None else "")
    if hap is not None:
        return sample + "#" + hap + ("#" + seq if seq is not None else "")
    return sample + "#*#" + seq if seq is not None else sample


def walk_key(sample: str, hap: int, seq: str, mode: str) -> str:
    if mode == "sample":
        return sample
    if mode == "sample-hap":
        return "%s#%d" % (sample, hap)
    return "%s#%d#%s" % (sample, hap, seq)


def groups(path_names: Sequence[str], walks: Sequence[Tuple[str, int, str]], mode: str) -> List[int]:
    n = len(path_names) + len(walks)
    if mode == "path":
        return list(range(n))
    keys = [path_key(p, mode) for p in path_names] + [walk_key(s, h, q, mode) for s, h, q in walks]
    seen = {}
    return [seen.setdefault(k, len(seen)) for k in keys]


def coverage_hist(traversals: Sequence[np.ndarray], gid: Sequence[int], num_nodes: int) -> np.ndarray:
    ng = (max(gid) + 1) if len(gid) else 0
    cov = np.zeros(num_nodes + 1, np.int64)
    members = {}
    for t, g in enumerate(gid):
        members.setdefault(g, []).append(t)
    for g in range(ng):
        seen = np.zeros(num_nodes + 1, bool)
        for t in members.get(g, []):
            a = np.abs(np.asarray(traversals[t], np.int64))
            a = a[(a >= 1) & (a <= num_nodes)]
            seen[a] = True
        cov += seen
    hist = np.zeros(ng + 1, np.int64)
    np.add.at(hist, cov[1:][cov[1:] <= ng], 1)
    return hist


def growth_curve(hist: Sequence[int], N: int) -> List[float]:
    out = [0.0] * (N + 1)
    for k in range(1, N + 1):
        s = 0.0
        for c in range(1, N + 1):
            if hist[c] == 0:
                continue
            if c >= N or N - c < k:
                frac = 1.0
            else:
                ratio = 1.0
                for i in range(c):
                    ratio *= float(N - k - i) / float(N - i)
                frac = 1.0 - ratio
            s += float(hist[c]) * frac
        out[k] = s
    return out


def growth_text(num_nodes: int, hist, growth, mode: str) -> str:
    N = len(hist) - 1 if len(hist) else 0
    out = ["# gfaz growth (count=node, coverage>=1, quorum>=0)\n# group-by=%s\n" % mode,
           "# num_haplotypes=%d num_nodes=%d\nk\tgrowth\n" % (N, num_nodes)]
    out += ["%d\t%.4f\n" % (k, growth[k]) for k in range(1, N + 1)]
    return "".join(out)
