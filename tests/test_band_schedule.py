"""The band schedule of hgpu_update_host (Solver<real>::hostStep, csrc/host/solver.cu),
restated and checked on the CPU for every slow-axis size 5-1099 (2D) and 5-79 (3D).

The slowest axis (y in 2D, z in 3D) is cut into K bands of `per` eigenbasis tiles
(T_A planes each; the last band takes the remainder).  Upload order: band K-1, then
0, 1, ..., K-2.  On the preparation stream, in order: prep(K-1), prep(0), the slow
axis's ghost fill, mark(0) (band K-1 shares that mark), then prep(j), mark(j) for
j = 1..K-2.  prep(j) makes the band's planes ready (landed, E += 0, ghost fill of the
other axes).  work(j), the band's eigenbasis (tile t reads planes t*T_A - 1 ..
t*T_A + T_A - 1), runs on one of two streams after mark(j) (band K-1: after
mark(K-2)), so it may only read planes that were ready at that mark; bands' works run
in any order relative to each other.  Checked: the bands partition the axis, every
plane a work reads is ready at the mark it waits for, the slow fill's planes (2, 3,
S-4, S-3 read; 0, 1, S-2, S-1 written) are all in the first two bands uploaded, and
the other axes' line ranges stay inside their line counts."""
import pytest


def plan(dim, S_A):
    T_A = 8 if dim == 2 else 2                      # roeBasisSlowTile: BasisTile<2>::Y, <3>::Z
    tiles = (S_A + T_A - 1) // T_A
    per = max(16 if dim == 2 else 8, (4 + T_A - 1) // T_A + 1)
    K = max(1, tiles // per)
    t0 = [j * per for j in range(K)]
    t1 = [tiles if j == K - 1 else (j + 1) * per for j in range(K)]
    p0 = [t * T_A for t in t0]
    p1 = [min(t * T_A, S_A) for t in t1]
    return T_A, K, t0, t1, p0, p1


def check_schedule(dim, S):
    A = dim - 1
    S_A = S[A]
    T_A, K, t0, t1, p0, p1 = plan(dim, S_A)
    covered = [p for j in range(K) for p in range(p0[j], p1[j])]
    assert covered == list(range(S_A))
    ready = set()
    marks = {}

    def prep(j):
        ready.update(range(p0[j], p1[j]))
        for a in range(A):                          # lines of axis a through the band
            per_plane = 1 if dim == 2 else S[1 if a == 0 else 0]
            lines = S[1] if dim == 2 else S[1 if a == 0 else 0] * S[2]
            assert 0 <= p0[j] * per_plane < p1[j] * per_plane <= lines

    def work(j):
        need = K - 2 if (j == K - 1 and K > 2) else j
        seen = marks[need]
        for t in range(t0[j], t1[j]):
            for p in range(t * T_A - 1, t * T_A + T_A):
                if 0 <= p < S_A:
                    assert p in seen, (dim, S, j, t, p)

    prep(K - 1)
    if K > 1:
        prep(0)
    for p in (2, 3, S_A - 4, S_A - 3, 0, 1, S_A - 2, S_A - 1):
        assert p in ready, (dim, S, K, p)
    marks[0] = marks[K - 1] = frozenset(ready)
    for j in range(1, K - 1):
        prep(j)
        marks[j] = frozenset(ready)
    for j in range(K):                              # any order: each waits for its own mark
        work(j)
    return K


@pytest.mark.parametrize("dim", [2, 3])
def test_band_schedule_reads_only_ready_planes(dim):
    seen = set()
    for s in range(5, 1100 if dim == 2 else 80):
        S = (7, s) if dim == 2 else (6, 9, s)
        seen.add(check_schedule(dim, S))
    assert max(seen) > 2                            # several bands were exercised


def test_benchmark_sizes():
    assert check_schedule(2, (2048, 2048)) == 16
    assert check_schedule(3, (256, 256, 256)) == 16
