"""The work lists of the in-place ghost-cell fill and fold (k_gc_fill,
k_gc_fold in pfft_gb300/csrc/gcell.cu), restated in Python and checked on the
CPU for every shape class the kernels meet: halos narrower and wider than
the block, halos on some axes only, tuples of 1 to 3 reals.

For each case the restatement walks the same index arithmetic as the
kernels (warp-level work units, lanes, part A / part B) and checks that
  * every access stays inside the box,
  * the fill writes each ghost scalar exactly once, from its periodic image,
    and never reads a scalar it (or another thread) writes,
  * the fold writes exactly the block cells with more than one periodic
    image, summing all images in (k0, k1, k2) order, and no thread reads a
    scalar another thread writes,
so the single launch of each is race-free whatever the scheduling.
"""
import itertools

import pytest


def fill_work(n, ng, tu):
    e2 = ng[2] - n[2]
    per = e2 * tu
    rows_a = n[0] * n[1] if per > 0 else 0
    rows_b = (ng[0] - n[0]) * ng[1] + n[0] * (ng[1] - n[1])
    rpw = 32 // per if 0 < per <= 16 else 1
    return rows_a, rows_b, max(per, 1), rpw


def fold_work(n, ng, tu):
    m = [min(ng[i] - n[i], n[i]) for i in range(3)]
    per = m[2] * tu
    rows_a = (n[0] - m[0]) * (n[1] - m[1]) if per > 0 else 0
    rows_b = m[0] * n[1] + (n[0] - m[0]) * m[1]
    rpw = 32 // per if 0 < per <= 16 else 1
    return rows_a, rows_b, max(per, 1), rpw


def lanes(per, rpw):
    for lane in range(32):
        yield (lane // per if rpw > 1 else 0), (lane % per if rpw > 1 else lane), lane


def run_fill(n, gb, ng, tu):
    """(write, read) scalar pairs of k_gc_fill."""
    rows_a, rows_b, per, rpw = fill_work(n, ng, tu)
    rb = ng[2] * tu
    e0, e1 = ng[0] - n[0], ng[1] - n[1]
    groups_a = (rows_a + rpw - 1) // rpw
    out = []
    for q in range(groups_a + rows_b):
        for lr, lc0, lane in lanes(per, rpw):
            if q < groups_a:
                row = q * rpw + lr
                if lr >= rpw or row >= rows_a:
                    continue
                j0, j1 = divmod(row, n[1])
                base = ((j0 + gb[0]) * ng[1] + j1 + gb[1]) * rb
                for lc in range(lc0, per, 32):
                    c, h = divmod(lc, tu)
                    k2 = c if c < gb[2] else c + n[2]
                    out.append((base + k2 * tu + h, base + ((k2 - gb[2]) % n[2] + gb[2]) * tu + h))
            else:
                r = q - groups_a
                planes = e0 * ng[1]
                if r < planes:
                    p, k1 = divmod(r, ng[1])
                    k0 = p if p < gb[0] else p + n[0]
                else:
                    p, c = divmod(r - planes, e1)
                    k0 = gb[0] + p
                    k1 = c if c < gb[1] else c + n[1]
                src = (((k0 - gb[0]) % n[0] + gb[0]) * ng[1] + (k1 - gb[1]) % n[1] + gb[1]) * rb
                dst = (k0 * ng[1] + k1) * rb
                for t in range(lane, rb, 32):
                    k2, h = divmod(t, tu)
                    out.append((dst + t, src + ((k2 - gb[2]) % n[2] + gb[2]) * tu + h))
    return out


def run_fold(n, gb, ng, tu):
    """{written scalar: [read scalars in order]} of k_gc_fold."""
    rows_a, rows_b, per, rpw = fold_work(n, ng, tu)
    m = [min(ng[i] - n[i], n[i]) for i in range(3)]
    rb = ng[2] * tu
    groups_a = (rows_a + rpw - 1) // rpw
    out = {}
    for q in range(groups_a + rows_b):
        for lr, lc0, lane in lanes(per, rpw):
            if q < groups_a:
                row = q * rpw + lr
                if lr >= rpw or row >= rows_a:
                    continue
                a0, a1 = divmod(row, n[1] - m[1])
                rowp = ((m[0] + a0) * ng[1] + m[1] + a1) * rb
                for lc in range(lc0, per, 32):
                    s2, h = divmod(lc, tu)
                    at = rowp + ((s2 - gb[2]) % n[2] + gb[2]) * tu + h
                    assert at not in out
                    out[at] = [rowp + k2 * tu + h for k2 in range(s2, ng[2], n[2])]
            else:
                r = q - groups_a
                if r < m[0] * n[1]:
                    s0, j1 = divmod(r, n[1])
                    s1 = (j1 + gb[1]) % n[1]
                else:
                    p, s1 = divmod(r - m[0] * n[1], m[1])
                    s0 = m[0] + p
                at0 = (((s0 - gb[0]) % n[0] + gb[0]) * ng[1] + (s1 - gb[1]) % n[1] + gb[1]) * rb
                for t in range(lane, n[2] * tu, 32):
                    j2, h = divmod(t, tu)
                    s2 = (j2 + gb[2]) % n[2]
                    at = at0 + (j2 + gb[2]) * tu + h
                    assert at not in out
                    out[at] = [((k0 * ng[1] + k1) * ng[2] + k2) * tu + h for k0 in range(s0, ng[0], n[0])
                               for k1 in range(s1, ng[1], n[1]) for k2 in range(s2, ng[2], n[2])]
    return out


CASES = [((4, 5, 6), (1, 2, 1), (2, 0, 1), 1), ((8, 8, 8), (2, 2, 2), (2, 2, 2), 2),
         ((3, 4, 5), (0, 0, 0), (0, 0, 0), 1), ((2, 3, 4), (5, 1, 9), (3, 7, 2), 3),
         ((6, 5, 4), (0, 3, 0), (0, 0, 0), 2), ((5, 6, 7), (0, 0, 2), (0, 0, 0), 1),
         ((4, 4, 40), (1, 1, 0), (0, 1, 20), 1), ((7, 3, 2), (9, 0, 0), (0, 0, 0), 1),
         ((3, 3, 3), (0, 0, 20), (0, 0, 17), 2)]


@pytest.mark.parametrize("n,gb,ga,tu", CASES)
def test_fill_and_fold_work_lists(n, gb, ga, tu):
    ng = [n[i] + gb[i] + ga[i] for i in range(3)]
    total = ng[0] * ng[1] * ng[2] * tu
    interior = lambda k: all(gb[i] <= k[i] < gb[i] + n[i] for i in range(3))  # noqa: E731
    cell = lambda k: ((k[0] * ng[1] + k[1]) * ng[2] + k[2]) * tu  # noqa: E731

    fill = run_fill(n, gb, ng, tu)
    writes = [w for w, _ in fill]
    reads = {r for _, r in fill}
    assert all(0 <= w < total for w in writes) and all(0 <= r < total for r in reads)
    assert len(set(writes)) == len(writes)
    ghosts = {cell(k) + h for k in itertools.product(*(range(g) for g in ng)) if not interior(k) for h in range(tu)}
    assert set(writes) == ghosts
    assert not reads & set(writes)
    for w, r in fill:  # each ghost scalar from its periodic image
        (cw, hw), (cr, hr) = divmod(w, tu), divmod(r, tu)
        assert hw == hr
        kw = (cw // (ng[1] * ng[2]), cw // ng[2] % ng[1], cw % ng[2])
        kr = (cr // (ng[1] * ng[2]), cr // ng[2] % ng[1], cr % ng[2])
        assert all((kw[i] - gb[i]) % n[i] == kr[i] - gb[i] for i in range(3))

    fold = run_fold(n, gb, ng, tu)
    want = {}
    for j in itertools.product(*(range(v) for v in n)):
        s = [(j[i] + gb[i]) % n[i] for i in range(3)]
        ims = [cell((k0, k1, k2)) for k0 in range(s[0], ng[0], n[0]) for k1 in range(s[1], ng[1], n[1])
               for k2 in range(s[2], ng[2], n[2])]
        if len(ims) > 1:
            for h in range(tu):
                want[cell(tuple(j[i] + gb[i] for i in range(3))) + h] = [c + h for c in ims]
    assert set(fold) == set(want)
    for at, rd in fold.items():
        assert rd == want[at]
        assert all(0 <= x < total for x in rd)
    owner = {}
    for at, rd in fold.items():
        for x in rd:
            owner.setdefault(x, set()).add(at)
    for at in fold:  # a written scalar is read by its own thread only
        assert owner.get(at, {at}) == {at}
