"""The kernels reorganise some sequential steps of the reference for the
GPU; these tests restate both forms in Python and check that they give the
same answer on random inputs (no GPU needed):

* the swap targets of a reshuffle round (quickstep.cpp:471-478), drawn by
  csrc/sor_fwd.cuh over one contiguous run of (island, step) entries per lane
  instead of island by island;
* the canonical pair order (i < k in geom order), walked by each lane of
  csrc/world_step.cuh phase_collide 32 pairs at a time instead of unranked
  pair by pair;
* the heightfield collider's plane grouping (heightfield.cpp:1387-1440) and
  plane sort (sortPlanes, :910-932), which csrc/heightfield.cuh does with a
  window of the triangles sorted by plane offset and a stable merge sort.
"""
import math
import random

import numpy as np

M32 = 0xFFFFFFFF


def _lcg_next(s):
    return (1664525 * s + 1013904223) & M32


def _lcg_jump(s, k):
    a, c, A, C = 1664525, 1013904223, 1, 0
    while k:
        if k & 1:
            A, C = (a * A) & M32, (a * C + c) & M32
        c, a = (a * c + c) & M32, (a * a) & M32
        k >>= 1
    return (A * s + C) & M32


def _rand_int_from(r, n):
    # dRandInt's xor-fold of the LCG value, then the modulus (misc.cpp:65-117)
    if n <= 0x10:
        r ^= r >> 16; r ^= r >> 8; r ^= r >> 4
        if n <= 2:
            r ^= r >> 2; r ^= r >> 1
        elif n <= 4:
            r ^= r >> 2
    elif n <= 0x100:
        r ^= r >> 16; r ^= r >> 8
    elif n <= 0x10000:
        r ^= r >> 16
    return r % n


def _draws_by_island(seed, ms, n_shuffles, rnd):
    """Island by island: draw q of island i is the seed advanced by the draws
    of the islands before it, the rounds of island i before this one, and q."""
    rstart = np.concatenate([[0], np.cumsum(ms)])
    out, prefix = {}, 0
    for i, m in enumerate(ms):
        s = _lcg_jump(seed, prefix + rnd * max(m - 1, 0) + 1)
        for q in range(1, m):
            out[rstart[i] + q] = _rand_int_from(s, q + 1)
            s = _lcg_next(s)
        prefix += n_shuffles * (m - 1) if m > 0 else 0
    return out


def _draws_by_lane_runs(seed, ms, n_shuffles, rnd):
    """The kernel's form: the round's (island, q) entries cut into one
    contiguous run per lane; a jump-ahead to each run's first entry, then one
    LCG step per entry."""
    nisl = len(ms)
    rstart = np.concatenate([[0], np.cumsum(ms)])
    iex, ist, T, base = [0] * nisl, [0] * nisl, 0, 0
    for i, m in enumerate(ms):
        e = m - 1 if m > 1 else 0
        iex[i], ist[i] = T, _lcg_jump(seed, (base + rnd * e) & M32)
        T, base = T + e, base + n_shuffles * e
    per = (T + 31) >> 5
    out = {}
    for lane in range(32):
        e0, e1 = lane * per, min(T, lane * per + per)
        if e0 >= e1:
            continue
        lo, hi = 0, nisl - 1
        while lo < hi:
            mid = (lo + hi + 1) >> 1
            lo, hi = (mid, hi) if iex[mid] <= e0 else (lo, mid - 1)
        i = lo
        r0, m, q = rstart[i], rstart[i + 1] - rstart[i], e0 - iex[i] + 1
        sd, e = _lcg_jump(ist[i], q), e0
        while True:
            out[r0 + q] = _rand_int_from(sd, q + 1)
            e += 1
            if e >= e1:
                break
            q += 1
            if q < m:
                sd = _lcg_next(sd)
                continue
            while True:
                i += 1
                r0, m = rstart[i], rstart[i + 1] - rstart[i]
                if m > 1:
                    break
            q, sd = 1, _lcg_next(ist[i])
    return out


def test_reshuffle_draws_per_lane_run_equal_per_island():
    rng = random.Random(1)
    for _ in range(400):
        n = rng.randint(1, 64)
        ms = [rng.choice([1, 1, 2, 3, rng.randint(1, 40), rng.randint(1, 300)]) for _ in range(n)]
        seed, n_shuffles = rng.getrandbits(32), rng.randint(1, 7)
        for rnd in range(n_shuffles):
            assert _draws_by_island(seed, ms, n_shuffles, rnd) == _draws_by_lane_runs(seed, ms, n_shuffles, rnd)


def _unrank(p, ng):
    tn = 2.0 * ng - 1.0
    i = int(math.floor((tn - math.sqrt(max(tn * tn - 8.0 * p, 0.0))) * 0.5))
    i = max(0, min(i, ng - 2))
    while i > 0 and i * (2 * ng - i - 1) // 2 > p:
        i -= 1
    while (i + 1) * (2 * ng - (i + 1) - 1) // 2 <= p:
        i += 1
    return i, p - i * (2 * ng - i - 1) // 2 + i + 1


def test_pair_walk_follows_canonical_order():
    for ng in range(2, 80):
        npairs = ng * (ng - 1) // 2
        canonical = [(i, k) for i in range(ng) for k in range(i + 1, ng)]
        for lane in range(min(32, npairs)):
            pi, pk = _unrank(lane, ng)
            for p in range(lane, npairs, 32):
                assert (pi, pk) == canonical[p] == _unrank(p, ng)
                pk += 32
                while pk >= ng and pi < ng - 2:
                    over = pk - ng
                    pi += 1
                    pk = pi + 1 + over


EPS = np.float32(1.1920928955078125e-07)


def _group_sequential(tp):
    """heightfield.cpp's grouping: triangle k, untaken, leads a plane and
    takes every later untaken triangle whose plane matches within dEpsilon in
    all four components."""
    n = len(tp)
    taken = [False] * n
    groups = []
    for k in range(n):
        if taken[k]:
            continue
        g = [k]
        for m in range(k + 1, n):
            if not taken[m] and all(abs(tp[k][c] - tp[m][c]) < EPS for c in (1, 3, 0, 2)):
                g.append(m)
                taken[m] = True
        taken[k] = True
        groups.append(g)
    return groups


def _group_windowed(tp):
    """The kernel's form: the candidates of leader k lie within dEpsilon of its
    offset, a window of the triangles sorted by offset; the matches are put
    back in triangle order."""
    n = len(tp)
    order = sorted(range(n), key=lambda k: tp[k][3])
    rank = [0] * n
    for i, k in enumerate(order):
        rank[k] = i
    taken = [False] * n
    groups = []
    for k in range(n):
        if taken[k]:
            continue
        b, found = tp[k], []

        def take(m):
            if m > k and not taken[m] and all(abs(b[c] - tp[m][c]) < EPS for c in (1, 0, 2)):
                found.append(m)
        j = rank[k] - 1
        while j >= 0 and b[3] - tp[order[j]][3] < EPS:
            take(order[j])
            j -= 1
        j = rank[k] + 1
        while j < n and tp[order[j]][3] - b[3] < EPS:
            take(order[j])
            j += 1
        found.sort()
        for m in found:
            taken[m] = True
        taken[k] = True
        groups.append([k] + found)
    return groups


def _sort_insertion(keys):
    order = list(range(len(keys)))
    for i in range(1, len(order)):
        cur, j = order[i], i
        while j > 0 and keys[order[j - 1]] - keys[cur] > EPS:
            order[j] = order[j - 1]
            j -= 1
        order[j] = cur
    return order


def _sort_merge(keys):
    src = list(range(len(keys)))
    n, width = len(src), 1
    while width < n:
        dst = []
        for lo in range(0, n, 2 * width):
            a, b = src[lo:lo + width], src[lo + width:lo + 2 * width]
            i = j = 0
            while i < len(a) and j < len(b):
                if keys[a[i]] - keys[b[j]] > EPS:
                    dst.append(b[j]); j += 1
                else:
                    dst.append(a[i]); i += 1
            dst += a[i:] + b[j:]
        src, width = dst, width * 2
    return src


def test_plane_grouping_and_sort_match_the_sequential_forms():
    rng = np.random.default_rng(7)
    for trial in range(300):
        n = int(rng.integers(1, 163))
        # planes of a few distinct definitions, some repeated exactly, some
        # moved by a few FP32 units (within and beyond dEpsilon)
        base = rng.normal(size=(int(rng.integers(1, 12)), 4)).astype(np.float32)
        tp = base[rng.integers(0, len(base), n)].copy()
        jitter = rng.random(n) < 0.3
        tp[jitter] += (rng.integers(-3, 4, size=(int(jitter.sum()), 4)) * EPS * 0.4).astype(np.float32)
        tp = [tuple(np.float32(x) for x in row) for row in tp]
        assert _group_sequential(tp) == _group_windowed(tp), trial
        # heights that are equal or further apart than dEpsilon
        keys = [np.float32(x) for x in rng.integers(0, 20, size=int(rng.integers(1, 90))) * 0.25]
        assert _sort_insertion(keys) == _sort_merge(keys), trial
