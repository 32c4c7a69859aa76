"""The Fp Montgomery squaring's row structure, emulated word by word.

The device squaring (gb_field.cuh, mont_sqr_fp_device) is CIOS whose step i
adds a_i times (a_i at word i, then the words of 2 * sum_{j>i} a_j 2^(32 j)):
an even-word carry chain starting at word (i + 1) & ~1, an odd-word row of
plain products, the Montgomery rows and the fold, exactly as the product
does.  This restatement runs those rows on 32-bit words and checks the
result against a^2 R^-1 mod p, and that no carry leaves the 13-word
accumulator (the bound the device code relies on).  The device code itself
is checked bit-exact by every GPU MSM test: each mixed addition squares
twice.
"""
import random

P = 0x1A0111EA397FE69A4B1BA7B6434BACD764774B84F38512BF6730D2A0F6B0F6241EABFFFEB153FFFFB9FEFFFFFFFFAAAB
M32 = 0xFFFFFFFF
R = 1 << 384
INV = (-pow(P, -1, 1 << 32)) % (1 << 32)
PW = [(P >> (32 * i)) & M32 for i in range(12)]


def _chain(acc, j0, xs, y):
    """acc[j0 ..] += sum_k xs[k] * y at words j0 + 2k, j0 + 2k + 1; the
    carry ends in acc[12] and must not leave it."""
    carry, w = 0, j0
    for x in xs:
        t = x * y
        s = acc[w] + (t & M32) + carry
        acc[w], carry = s & M32, s >> 32
        s = acc[w + 1] + (t >> 32) + carry
        acc[w + 1], carry = s & M32, s >> 32
        w += 2
    assert w == 12
    s = acc[12] + carry
    assert s >> 32 == 0
    acc[12] = s


def mont_sqr_rows(a):
    aw = [(a >> (32 * i)) & M32 for i in range(12)]
    d = [((aw[j] << 1) | (aw[j - 1] >> 31 if j else 0)) & M32 for j in range(12)]
    even = [0] * 13
    for i in range(12):
        def y(j):
            if j < i:
                return 0
            if j == i:
                return aw[i]
            if j == i + 1:
                return (aw[i + 1] << 1) & M32
            return d[j]
        j0 = (i + 1) & ~1
        _chain(even, j0, [y(j) for j in range(j0, 12, 2)], aw[i])
        odd = [0] * 13
        for k in range(6):
            t = y(2 * k + 1) * aw[i]
            odd[2 * k], odd[2 * k + 1] = t & M32, t >> 32
        m = (even[0] * INV) & M32
        _chain(even, 0, PW[0::2], m)
        _chain(odd, 0, PW[1::2], m)
        assert even[0] == 0
        carry, nxt = 0, [0] * 13
        for w in range(12):
            s = even[w + 1] + odd[w] + carry
            nxt[w], carry = s & M32, s >> 32
        s = odd[12] + carry
        assert s >> 32 == 0
        nxt[12] = s
        even = nxt
    v = sum(w << (32 * i) for i, w in enumerate(even))
    assert v < 2 * P
    return v - P if v >= P else v


def test_fp_sqr_rows_match_definition():
    rng = random.Random(381)
    cases = [0, 1, 2, P - 1, P - 2, P >> 1, (P >> 1) + 1, (1 << 380) % P, R % P, (R * R) % P]
    cases += [rng.randrange(P) for _ in range(400)]
    rinv = pow(R, -1, P)
    for a in cases:
        assert mont_sqr_rows(a) == a * a * rinv % P, hex(a)
