"""Balanced l1-row strips for splitting one coupling problem over ranks.

Row l1 of the upper triangle holds lmax - l1 + 1 pairs, each a family of
2 l1 + 1 terms, so its cost is (lmax - l1 + 1)(2 l1 + 1).  Rows are dealt
greedily (heaviest first, to the lightest rank), which keeps the per-rank work
within a fraction of a percent at the benchmark sizes.  Each rank writes the
disjoint rows l1 (and mirrored columns) of its strip; no collective is needed
beyond gathering the results.
"""
import heapq


def row_cost(l1, lmax):
    return (lmax - l1 + 1) * (2 * l1 + 1)


def row_shards(lmin, lmax, world):
    heap = [(0, r) for r in range(world)]
    shards = [[] for _ in range(world)]
    for l1 in sorted(range(lmin, lmax + 1), key=lambda l: -row_cost(l, lmax)):
        c, r = heapq.heappop(heap)
        shards[r].append(l1)
        heapq.heappush(heap, (c + row_cost(l1, lmax), r))
    return [sorted(s) for s in shards]
