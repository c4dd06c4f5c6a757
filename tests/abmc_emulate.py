"""CPU emulation of the device ABMC ordering (senk_gb300/csrc/colour.cu), step
for step, for the tests: blocks of bs consecutive rows, the sorted distinct
neighbour blocks of each block, the symmetric adjacency, each colour by the
kernels' rounds (a candidate joins when no smaller neighbour is a candidate;
the neighbours of those that joined leave), then the reference's ordering
(colours in order, blocks ascending). It must equal the reference's
GetABMCPermutation(..., "simple") and the device result. Test code only."""
import numpy as np

def adjacency(cind, rptr, N, bs):
    nb = N // bs
    rows = np.repeat(np.arange(N), np.diff(rptr))
    src = rows // bs
    dst = np.asarray(cind) // bs
    keep = src != dst
    pairs = np.unique(np.stack([np.concatenate([src[keep], dst[keep]]), np.concatenate([dst[keep], src[keep]])]),
                      axis=1)
    order = np.lexsort((pairs[1], pairs[0]))
    a, c = pairs[0][order], pairs[1][order]
    aoff = np.zeros(nb + 1, np.int64)
    np.add.at(aoff, a + 1, 1)
    return np.cumsum(aoff), c


def abmc(cind, rptr, N, bs):
    nb = N // bs
    aoff, acol = adjacency(cind, rptr, N, bs)
    src = np.repeat(np.arange(nb), np.diff(aoff))
    colour = np.zeros(nb, np.int64)
    c = 0
    rounds = 0
    while (colour == 0).any():
        c += 1
        cand = colour == 0
        while True:
            rounds += 1
            # select: candidates without a smaller candidate neighbour
            smaller = cand[acol] & (acol < src)
            lost = np.zeros(nb, bool)
            np.logical_or.at(lost, src, smaller)
            chosen = cand & ~lost
            colour[chosen] = c
            # prune: chosen blocks and their neighbours leave
            hit = np.zeros(nb, bool)
            np.logical_or.at(hit, src, colour[acol] == c)
            cand = cand & (colour == 0) & ~hit
            if not cand.any():
                break
    nc = c
    size_color = [0]
    LP = np.empty(N, np.int32)
    pos = 0
    for k in range(1, nc + 1):
        blocks = np.nonzero(colour == k)[0]
        for b in blocks:
            LP[pos * bs:(pos + 1) * bs] = np.arange(b * bs, (b + 1) * bs)
            pos += 1
        size_color.append(pos)
    RP = np.empty(N, np.int32)
    RP[LP] = np.arange(N, dtype=np.int32)
    return nc, np.array(size_color, np.int32), LP, RP, rounds


def check_ordering(cind, rptr, N, bs, nc, size_color, LP, RP):
    """Colours are independent sets of blocks; LP, RP inverse permutations that
    keep blocks whole; size_color covers all blocks."""
    assert size_color[0] == 0 and size_color[-1] == N // bs and np.all(np.diff(size_color) >= 0)
    assert len(size_color) == nc + 1
    assert np.array_equal(np.sort(LP), np.arange(N)) and np.array_equal(RP[LP], np.arange(N))
    newblock = RP // bs
    assert np.array_equal(newblock.reshape(-1, bs).min(1), newblock.reshape(-1, bs).max(1))
    colour_of_new = np.searchsorted(size_color, np.arange(N // bs), side="right") - 1
    col = colour_of_new[newblock]  # colour of each old row
    rows = np.repeat(np.arange(N), np.diff(rptr))
    cind = np.asarray(cind)
    other = (rows // bs) != (cind // bs)
    assert not np.any(col[rows[other]] == col[cind[other]]), "adjacent blocks share a colour"
