"""The min / max windows of the differentiable chain's tiles by doubling (csrc/soft.cu:
k_soft_pass_x, k_soft_ext_yz, k_soft_adj_x, k_soft_ext_adj_yz), restated with the kernels'
index arithmetic and checked against the sequential fold and first-extreme scan that the
untiled kernels (k_soft_pass, k_soft_minmax_adj) run.

A tile stages L = n_out + 2R values of a line from position p0 = c0 - R on (clamped to the
line); after the doubling steps with spans q = 1, 2, ... < q_end (q_end the largest power of
two <= 2R + 1), entry k (k <= L - 2q) holds the extreme of the 2q staged values from k on and
the staged position of the first of them; output t is the extreme of entries t and
t + 2R + 1 - q_end, the later one winning only when strictly better.  The values must equal
the sequential fold's and the positions, clamped to the line, the sequential scan's first
extreme (the window visited from c - R to c + R, replaced only by a strictly better value).
"""
import numpy as np
import pytest


def span(R):
    return 1 << ((2 * R + 1).bit_length() - 1)


def doubling(line, c0, R, n_out, is_max):
    n = len(line)
    L = n_out + 2 * R
    pos = np.clip(c0 - R + np.arange(L), 0, n - 1)
    v = line[pos].copy()
    at = np.arange(L)
    q_end = span(R)
    q = 1
    while q < q_end:
        lim = L - 2 * q + 1            # entries whose span of 2q stays inside the tile
        a, b = v[:lim], v[q:q + lim]
        better = b > a if is_max else b < a
        v = np.concatenate([np.where(better, b, a), v[lim:]])
        at = np.concatenate([np.where(better, at[q:q + lim], at[:lim]), at[lim:]])
        q *= 2
    t = np.arange(n_out)
    j = t + 2 * R + 1 - q_end
    assert j.max() <= L - 1
    a, b = v[t], v[j]
    better = b > a if is_max else b < a
    val = np.where(better, b, a)
    arg = np.clip(c0 - R + np.where(better, at[j], at[t]), 0, n - 1)
    return val, arg


def sequential(line, c, R, is_max):
    n = len(line)
    arg = min(max(c - R, 0), n - 1)
    best = line[arg]
    for j in range(-R + 1, R + 1):
        p = min(max(c + j, 0), n - 1)
        if (line[p] > best) if is_max else (line[p] < best):
            best, arg = line[p], p
    return best, arg


# (reach, tile outputs): the y / z kernels take reaches up to 32 with 64 outputs per tile, the
# x kernels reaches up to 64 with 256
CASES = [(R, 64) for R in (0, 1, 2, 3, 5, 8, 15, 16, 20, 31, 32)] + [(R, 256) for R in (0, 4, 20, 33, 47, 63, 64)]


@pytest.mark.parametrize("R,n_out", CASES)
@pytest.mark.parametrize("is_max", [False, True])
def test_doubling_equals_the_sequential_window(R, n_out, is_max):
    rng = np.random.default_rng(1000 * R + n_out + is_max)
    for n in (1, 3, 40, n_out + 7, 3 * n_out):
        line = rng.integers(0, 4, n).astype(np.float32)     # few values: ties everywhere
        for c0 in range(0, n, n_out):
            val, arg = doubling(line, c0, R, n_out, is_max)
            for t in range(min(n_out, n - c0)):
                best, first = sequential(line, c0 + t, R, is_max)
                assert val[t] == best, (n, c0 + t, val[t], best)
                assert arg[t] == first, (n, c0 + t, arg[t], first)
