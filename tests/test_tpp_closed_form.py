"""The closed-form two-pointer partition used by the GPU kd-tree build
(csrc/kdtree.cuh) against the reference's sequential swap loop
(src/fast3tree.c:751-774), on random flag patterns and edge cases."""
import numpy as np
import pytest


def sequential(big):
    """The reference loop, on flags: returns (permutation, num_left)."""
    p = list(range(len(big)))
    n = len(p)
    j = n - 1
    i = 0
    while i < j:
        if big[p[i]]:
            p[i], p[j] = p[j], p[i]
            j -= 1
            continue
        i += 1
    if i == j and not big[p[i]]:
        i += 1
    return p, i


def closed_form(big):
    big = np.asarray(big, bool)
    n = len(big)
    m = int((~big).sum())
    rank = np.concatenate([[0], np.cumsum(big)])
    q = int(rank[m])
    fb = np.zeros(n, int)
    bs = np.zeros(n, int)
    for l in range(n):
        br = rank[l]
        sr = l - br
        if big[l] and l < m:
            fb[br] = l
        if not big[l] and l >= m:
            bs[m - 1 - sr] = l
    out = [None] * n
    pos_last = bs[q - 1] if q > 0 else n
    for l in range(n):
        br = rank[l]
        sr = l - br
        if not big[l] and l < m:
            d = l
        elif big[l] and l < m:
            d = n - 1 if br == 0 else bs[br - 1] - 1
        elif not big[l]:
            d = fb[m - 1 - sr]
        else:
            if l > pos_last:
                d = l - 1
            elif pos_last - m >= 2:
                d = pos_last - 1 if l == m else l - 1
            else:
                d = l
        assert out[d] is None
        out[d] = l
    return out, m


@pytest.mark.parametrize("seed", range(40))
def test_random(seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 90))
    big = rng.random(n) < rng.random()
    big[rng.integers(0, n)] = False  # the reference always has one small element
    a = sequential(list(big))
    b = closed_form(big)
    assert a[1] == b[1]
    assert a[0] == b[0]


@pytest.mark.parametrize("pattern", ["0", "01", "10", "0011", "0101", "1100", "000111",
                                     "0111111", "1110000", "0" * 30, "01" * 20, "1" * 10 + "0"])
def test_edges(pattern):
    big = [c == "1" for c in pattern]
    assert sequential(big) == closed_form(big)
