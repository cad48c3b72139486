"""The pair enumeration of the conflict and contact tube sweeps, where probe
and target entries are one list (a cell's survivors, or its rods): every
unordered pair of a cell's entries must be tested exactly once, whatever the
cell's size, for both item forms the sweeps read:

- cell items: (probe chunk of <= 32 entries, segment of <= 128 targets) in
  tiles of 32; a tile before the chunk is skipped, the chunk's own tile is
  tested cyclically (a probe at place x of n tests the next (n - 1) // 2
  entries, and the opposite one when n is even and x < n / 2), a tile after
  the chunk is tested whole;
- packed items: the small cells (<= 32 entries) of a run, probe lane p being
  target slot p, each probe tested cyclically within its own cell's range.

This restates the rule of k_tube_conf / k_tube_ct (nf_generate.cu,
nf_contacts.cu) on the host; the GPU parity tests check the sweeps' results
against the oracle.
"""
import itertools

import pytest


def cyclic_half(n, x):
    """Targets (places in the range) a probe at place x of n tests."""
    nd = (n - 1) // 2 + (1 if n % 2 == 0 and x < n // 2 else 0) if n else 0
    return [(x + 1 + u) % n for u in range(nd)]


def cell_item_pairs(n, chunk=32, seg=128, tile=32):
    """Pairs (probe entry, target entry) the cell items of an n-entry cell test."""
    out = []
    for a in range(0, n, chunk):
        np_ = min(chunk, n - a)
        for s in range(0, n, seg):
            nt = min(seg, n - s)
            for b in range(0, nt, tile):
                t0, m = s + b, min(tile, nt - b)
                if t0 < a:
                    continue  # a tile before the chunk
                if t0 == a:  # the chunk's own tile
                    assert m == np_
                    for x in range(np_):
                        out += [(a + x, t0 + y) for y in cyclic_half(m, x)]
                else:  # after the chunk
                    out += [(a + x, t0 + y) for x in range(np_) for y in range(m)]
    return out


@pytest.mark.parametrize("n", list(range(0, 70)) + [95, 96, 97, 127, 128, 129, 160, 255, 256, 257, 300])
def test_cell_items_test_every_pair_once(n):
    pairs = cell_item_pairs(n)
    assert all(p != q for p, q in pairs)
    unordered = [frozenset(pq) for pq in pairs]
    assert len(unordered) == len(set(unordered)) == n * (n - 1) // 2


def test_packed_items_test_every_pair_once():
    # runs of small cells packed into one warp item: each lane's probe tests
    # its own cell's range cyclically
    for sizes in ([1], [2], [3, 5], [4, 4, 4, 4], [7, 1, 9, 15], [32], [16, 16], [31, 1]):
        assert sum(sizes) <= 32
        lo, pairs = 0, []
        for n in sizes:
            for x in range(n):
                pairs += [(lo + x, lo + y) for y in cyclic_half(n, x)]
            lo += n
        seen = [frozenset(pq) for pq in pairs]
        assert len(seen) == len(set(seen)) == sum(n * (n - 1) // 2 for n in sizes)
        # no pair crosses cells
        bounds = list(itertools.accumulate([0] + sizes))
        cell = {e: c for c in range(len(sizes)) for e in range(bounds[c], bounds[c + 1])}
        assert all(cell[p] == cell[q] for p, q in pairs)


def test_cyclic_half_balances_the_lanes():
    # every probe of a range tests (n - 1) // 2 or n // 2 targets: the warp's
    # marking loop is as long as half the range, not the whole range
    for n in range(1, 33):
        lens = [len(cyclic_half(n, x)) for x in range(n)]
        assert max(lens) - min(lens) <= 1 and max(lens) <= n // 2
