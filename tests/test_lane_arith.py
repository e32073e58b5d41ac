"""The byte-lane arithmetic of the warp-tile Ising sweep (spparks_gb300/csrc/warp_tile.cuh), restated in Python
and checked against the per-site rule of AppIsing::site_event_rejection (src/app_ising.cpp:104-136) under the
Ising draw contract: every combination of site value, neighbour values, proposal bit and threshold level, four
sites per 32-bit word; and the __byte_perm selectors that gather a colour phase's four sites of an 8-site segment
into one word and put them back.  No GPU: the formulas are the kernel's, evaluated on the host."""

import itertools
import random

M32 = 0xFFFFFFFF


def byte_perm(x, y, s):
    """CUDA __byte_perm(x, y, s) for selector nibbles 0-7: byte n of the result is byte (s >> 4n) & 7 of y:x."""
    v = (y << 32) | x
    return sum(((v >> (8 * ((s >> (4 * n)) & 7))) & 0xFF) << (8 * n) for n in range(4))


def word(bs):
    return sum(b << (8 * i) for i, b in enumerate(bs))


def lane_rule(v, nsum, code):
    """warp_lanes: new values of four lanes, all of the phase's colour"""
    x = (v * 15 - 0x0F0F0F0F) & M32
    s = ((nsum ^ x) + ((code - 3 * v) & M32)) & M32
    am = ((s & 0x20202020) * 6) & M32
    return (((s & am) | ((v << 6) & ~am & M32)) >> 6) & M32


def code_byte(p1, lvl):
    """0x9D + lvl - 0x40 p with p = [word < 2^31] (proposal of value 1)"""
    return 0x9D + lvl - 0x40 * p1


def reference_rule(v, nbs, p1, y, t2, t4):
    """AppIsing::site_event_rejection with u0 < 0.5 <=> p1 and the Boltzmann test y < thr[dE]"""
    news = 1 if p1 else 2
    e0 = sum(1 for n in nbs if n != v)
    if news == v:
        return v
    e1 = sum(1 for n in nbs if n != news)
    if e1 <= e0:
        return news
    thr = {2: t2, 4: t4}[e1 - e0]
    return news if y < thr else v


def test_lane_rule_matches_the_per_site_rule():
    # thr[4] <= thr[2] <= 2^31; y values around both thresholds
    rng = random.Random(7)
    cases = []
    for t2, t4 in ((0, 0), (2**31, 2**31), (1000, 10), (2**31, 5), (7, 7)):
        for y in sorted({0, t4 - 1, t4, t2 - 1, t2, 2**31 - 1}):
            if 0 <= y < 2**31:
                cases.append((t2, t4, y))
    for v, p1, (t2, t4, y), nbs in itertools.product((1, 2), (0, 1), cases, itertools.product((1, 2), repeat=4)):
        lvl = int(y < t4) + int(y < t2)
        want = reference_rule(v, nbs, p1, y, t2, t4)
        # the same site in each of the four byte lanes, the other lanes random
        for lane in range(4):
            vs = [rng.choice((1, 2)) for _ in range(4)]
            sums = [rng.randint(4, 8) for _ in range(4)]
            codes = [code_byte(rng.randint(0, 1), rng.randint(0, 2)) for _ in range(4)]
            vs[lane], sums[lane], codes[lane] = v, sum(nbs), code_byte(p1, lvl)
            got = lane_rule(word(vs), word(sums), word(codes))
            assert (got >> (8 * lane)) & 0xFF == want, (v, nbs, p1, y, t2, t4, lane)


def phase_sel(act):
    """phase_sel of warp_tile.cuh"""
    odd = act == 0x7531
    return {"act": act, "other": act ^ 0x1111, "side": 0x4321 if odd else 0x2107, "off": 8 if odd else -4,
            "lo": 0x1504 if odd else 0x5140, "hi": 0x3726 if odd else 0x7362}


def test_phase_gather_selectors():
    """warp_segment: the active x parity's four sites, their x-neighbours (the other four sites and one edge site)
    and their up/down neighbours (same parity of the rows above and below), and the merge back into x order"""
    rng = random.Random(11)
    for _ in range(500):
        row = [rng.randint(1, 200) for _ in range(16)]  # sites x0-4 .. x0+11 of the segment's row
        up = [rng.randint(1, 200) for _ in range(8)]
        dn = [rng.randint(1, 200) for _ in range(8)]
        vx, vy = word(row[4:8]), word(row[8:12])
        for par in (0, 1):
            p = phase_sel(0x6420 if par == 0 else 0x7531)
            edge = word(row[0:4]) if p["off"] == -4 else word(row[12:16])
            act = [row[4 + par + 2 * i] for i in range(4)]
            other = [row[4 + (1 - par) + 2 * i] for i in range(4)]
            left = [row[4 + par + 2 * i - 1] for i in range(4)]
            right = [row[4 + par + 2 * i + 1] for i in range(4)]
            a, b = byte_perm(vx, vy, p["act"]), byte_perm(vx, vy, p["other"])
            assert a == word(act) and b == word(other)
            side = byte_perm(b, edge, p["side"])
            assert sorted([b, side]) == sorted([word(left), word(right)])
            assert byte_perm(word(up[:4]), word(up[4:]), p["act"]) == word([up[par + 2 * i] for i in range(4)])
            assert byte_perm(word(dn[:4]), word(dn[4:]), p["act"]) == word([dn[par + 2 * i] for i in range(4)])
            new = [rng.randint(1, 200) for _ in range(4)]
            merged = row[4:12]
            for i in range(4):
                merged[par + 2 * i] = new[i]
            an = word(new)
            assert (byte_perm(an, b, p["lo"]), byte_perm(an, b, p["hi"])) == (word(merged[:4]), word(merged[4:]))


def test_colour1_code_words():
    """warp_draws: the codes of sites x0..x0+3 and x0+4..x0+7 split into the colour-1 word (the row's x parity)
    and the colour-2 word with one selector and its complement (selector ^ 0x1111)"""
    lo, hi = word([1, 2, 3, 4]), word([5, 6, 7, 8])
    for row_odd in (0, 1):
        sel1 = 0x6420 + 0x1111 * row_odd
        c1, c2 = byte_perm(lo, hi, sel1), byte_perm(lo, hi, sel1 ^ 0x1111)
        assert c1 == word([1 + row_odd + 2 * i for i in range(4)])
        assert c2 == word([2 - row_odd + 2 * i for i in range(4)])
