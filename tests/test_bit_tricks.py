"""Integer tricks of the row-pair, packed and cluster-resident sweep kernels, restated in Python and checked against
the plain definitions they replace.  No GPU: the formulas are the kernels', evaluated on the host.

- sweep_rows.cu: neighbour values below 128 packed four per word and the byte-lane unlike count (unlike_packed);
  the stamp-table first-appearance mask (first_appearance_stamped) against the reference's distinct-value list
  (src/app_potts_neighonly.cpp:80-88); the position of the n-th set bit (nth_set_bit) against __fns.
- packed.cu: the threshold level of a Boltzmann draw as two bit planes (hi, lo) against the three tests
  [y < t2], [y < t4], [y < t6].
- sweep_resident.cu: the x-pairs of a band (one site of each colour per pair, both sites' draws in one Philox
  block) against the per-colour site order."""

import random

import pytest

M32 = 0xFFFFFFFF


def pack_neighbors(nb):
    """PackedNb: four values per word, lanes in neighbour order, empty lanes 0"""
    nw = (len(nb) + 3) // 4
    return [sum((nb[4 * k + q] if 4 * k + q < len(nb) else 0) << (8 * q) for q in range(4)) for k in range(nw)]


def unlike_packed(words, nn, v):
    """the byte-lane count: (b ^ v) + 0x7F sets bit 7 exactly where the lane is non-zero"""
    vv = (v * 0x01010101) & M32
    acc = 0
    for w in words:
        acc = (acc + ((((w ^ vv) + 0x7F7F7F7F) & M32 & 0x80808080) >> 7)) & M32
    return (((acc * 0x01010101) & M32) >> 24) - (4 * len(words) - nn)


@pytest.mark.parametrize("nn", [4, 6, 8, 26])
def test_unlike_packed_equals_plain_count(nn):
    rng = random.Random(nn)
    for _ in range(3000):
        q = rng.choice([2, 5, 20, 100, 127])
        nb = [rng.randint(1, q) for _ in range(nn)]
        words = pack_neighbors(nb)
        for v in {rng.randint(1, q), nb[0], 1, q}:
            assert unlike_packed(words, nn, v) == sum(1 for n in nb if n != v)


def first_appearance(own, nb):
    """the reference's distinct list: neighbour j is listed when its value differs from own and from every
    earlier neighbour"""
    return sum(1 << j for j in range(len(nb)) if nb[j] != own and nb[j] not in nb[:j])


def first_appearance_stamped(own, nb, table, stamp):
    """one byte per value: own's entry stamped first, then each neighbour's in order"""
    table[own] = stamp
    first = 0
    for j, v in enumerate(nb):
        if table[v] != stamp:
            first |= 1 << j
        table[v] = stamp
    return first


def test_stamp_table_first_appearance_over_successive_sites():
    """one table per thread, cleared once per CTA; the thread's two sites use stamps 1 and 2"""
    rng = random.Random(7)
    for _ in range(2000):
        q = rng.choice([2, 3, 10, 40, 127])
        nn = rng.choice([8, 26])
        table = [0] * 128
        for stamp in (1, 2):
            own = rng.randint(1, q)
            nb = [rng.randint(1, q) for _ in range(nn)]
            assert first_appearance_stamped(own, nb, table, stamp) == first_appearance(own, nb)


def nth_set_bit(m, n):
    """popc search over halves, bytes, nibbles and pairs"""
    pos = 0
    for width in (16, 8, 4, 2):
        c = bin(m & ((1 << width) - 1)).count("1")
        if n >= c:
            n -= c
            m >>= width
            pos += width
    if n >= (m & 1):
        pos += 1
    return pos


def fns(m, n):
    """__fns(m, 0, n + 1): position of the (n+1)-th set bit from bit 0"""
    seen = -1
    for b in range(32):
        if (m >> b) & 1:
            seen += 1
            if seen == n:
                return b
    raise AssertionError


def test_nth_set_bit_equals_fns():
    rng = random.Random(3)
    masks = [rng.getrandbits(26) for _ in range(3000)] + [1, 1 << 25, (1 << 26) - 1, 0xFFFFFFFF, 0x80000001]
    for m in masks:
        for n in range(bin(m).count("1")):
            assert nth_set_bit(m, n) == fns(m, n)


def test_threshold_level_planes():
    """hi = [y < t4]; lo = [y < t6] where hi is set, [y < t2] where it is not (t2 >= t4 >= t6)"""
    rng = random.Random(11)
    edges = [0, 1, 2, (1 << 31) - 1, 1 << 31]
    for _ in range(20000):
        t = sorted([rng.choice(edges + [rng.getrandbits(31)]) for _ in range(3)], reverse=True)
        t2, t4, t6 = t
        y = rng.choice([rng.getrandbits(31), t2, t4, t6, max(t6 - 1, 0), min(t2 + 1, (1 << 31) - 1)])
        y &= 0x7FFFFFFF
        hi = int(y < t4)
        lo = int(y < (t6 if hi else t2))
        assert (hi | lo, hi, hi & lo) == (int(y < t2), int(y < t4), int(y < t6))


def resident_pairs(nx, ny, cl, threads):
    """the band sites each thread owns: pair pr = tid + threads*q of band row ly = pr // (nx/2); colour c site
    x = 2m + ((y + c) & 1); both sites' block is that of the pair's even site"""
    out = []
    r = ny // cl
    for rank in range(cl):
        r0 = rank * r
        npairs = r * nx // 2
        for tid in range(threads):
            for q in range((npairs + threads - 1) // threads):
                pr = tid + threads * q
                if pr >= npairs:
                    continue
                ly, m = divmod(pr, nx // 2)
                y = r0 + ly
                s_even = y * nx + 2 * m
                for c in (0, 1):
                    x = 2 * m + ((y + c) & 1)
                    out.append((c, y, x, s_even))
    return out


@pytest.mark.parametrize("nx,ny,cl", [(128, 128, 16), (128, 128, 8), (32, 32, 16), (96, 64, 16), (16, 16, 16)])
def test_resident_pairs_cover_each_colour_once(nx, ny, cl):
    pairs = resident_pairs(nx, ny, cl, min(512, (nx * ny // cl // 2 + 31) // 32 * 32))
    for c in (0, 1):
        sites = sorted((y, x) for cc, y, x, _ in pairs if cc == c)
        want = sorted((y, x) for y in range(ny) for x in range(nx) if (x + y) % 2 == c)
        assert sites == want
    for c, y, x, s_even in pairs:
        s = y * nx + x
        # Ising: one block per four sites (s >> 2); Potts-family apps: one block per x-pair (s >> 1)
        assert s >> 2 == s_even >> 2 and s >> 1 == s_even >> 1
        assert s & 1 == x & 1
