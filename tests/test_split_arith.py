"""CPU checks of the arithmetic the split-BF16 kernels rely on, restated in
numpy float32 (IEEE round-to-nearest-even, as the GPU's FP32 adds):

- the FP32 three-part split (fx_split_f in csrc/lcp_kernels_tc.cu): every
  part is an integer multiple of its quantum (2^-8, 2^-17, 2^-26) of at most
  256 quanta, hence exact in BF16, and the parts carry p + e to within
  2^-27 + 2^-34;
- the FP64 table split (fx_split) gives the same parts;
- the integer split of an FP64 value's bits (fx_split_bits, the split-BF16
  table build): parts of at most 256 quanta, exact in BF16, carrying
  v / 2^k to within 2^-27, and equal to the exact rounding of v / 2^k to
  2^-26 split into nearest digits;
- the brick dealing of the persistent kernels (round_brick) visits every
  brick exactly once for any brick count and grid size.
"""
import numpy as np

F = np.float32


def _round_add(x, c):
    """(x + c) - c in FP32: x rounded to a multiple of ulp(c)."""
    return (F(x) + F(c)) - F(c)


def split_f(p, e):
    p = np.asarray(p, dtype=np.float32)
    e = np.asarray(e, dtype=np.float32)
    h = _round_add(p, 49152.0)          # 1.5 * 2^15 -> multiples of 2^-8
    r1 = (p - h) + e
    m = _round_add(r1, 96.0)            # 1.5 * 2^6 -> multiples of 2^-17
    r2 = r1 - m
    lo = _round_add(r2, 0.1875)         # 1.5 * 2^-3 -> multiples of 2^-26
    return h, m, lo


def split_d(u):
    h = np.rint(u * 256.0) / 256.0
    r1 = u - h
    m = np.rint(r1 * 131072.0) / 131072.0
    lo = np.rint((r1 - m) * 67108864.0) / 67108864.0
    return h, m, lo


def _is_bf16_exact(x):
    x = np.asarray(x, dtype=np.float32)
    bits = x.view(np.uint32)
    return np.all((bits & 0xFFFF) == 0)


def test_fp32_split_parts_exact_and_residual():
    rng = np.random.default_rng(5)
    n = 200000
    # magnitudes from 1 down to 2^-40, both signs, and the edges
    p = (rng.uniform(-1, 1, n) * 2.0 ** -rng.integers(0, 40, n)).astype(np.float32)
    p[:6] = [1.0, -1.0, 0.0, 2.0 ** -9, -(2.0 ** -9), 0.99999994]
    e = (p.astype(np.float64) * rng.uniform(-2.0 ** -23, 2.0 ** -23, n)).astype(np.float32)
    h, m, lo = split_f(p, e)
    for part, q in ((h, 2.0 ** -8), (m, 2.0 ** -17), (lo, 2.0 ** -26)):
        k = part.astype(np.float64) / q
        assert np.all(k == np.rint(k))
        assert np.all(np.abs(k) <= 256)
        assert _is_bf16_exact(part)
    total = h.astype(np.float64) + m + lo
    target = p.astype(np.float64) + e.astype(np.float64)
    assert np.max(np.abs(total - target)) <= 2.0 ** -27 + 2.0 ** -34


def test_fp64_split_matches_and_is_exact():
    rng = np.random.default_rng(6)
    u = rng.uniform(-1, 1, 100000) * 2.0 ** -rng.integers(0, 30, 100000)
    h, m, lo = split_d(u)
    for part in (h, m, lo):
        assert _is_bf16_exact(part.astype(np.float32))
        assert np.all(part.astype(np.float32).astype(np.float64) == part)
    assert np.max(np.abs(h + m + lo - u)) <= 2.0 ** -27
    # the FP32 split of the FP32 value plus its FP64 remainder gives the same parts
    uf = u.astype(np.float32)
    hf, mf, lf = split_f(uf, (u - uf.astype(np.float64)).astype(np.float32))
    same = (hf == h) & (mf == m) & (lf == lo)
    assert same.mean() > 0.999  # ties of the last part may round apart


def split_bits(v, k):
    """fx_split_bits restated on the IEEE bits of float64 v (numpy int64)."""
    v = np.asarray(v, dtype=np.float64)
    b = v.view(np.uint64)
    e = ((b >> np.uint64(52)) & np.uint64(0x7ff)).astype(np.int64)
    m = ((b & np.uint64((1 << 52) - 1)) | np.uint64(1 << 52)).astype(object)
    sh = 1049 + k - e
    a = np.zeros(v.shape, dtype=object)
    for i in range(v.size):
        if e.flat[i] == 0:
            continue
        s_ = int(sh.flat[i])
        if s_ <= 0:
            a.flat[i] = 1 << 26
        elif s_ < 64:
            mm = int(m.flat[i])
            half = 1 << (s_ - 1)
            rem = mm & ((half << 1) - 1)
            q = mm >> s_
            if rem > half or (rem == half and (q & 1)):
                q += 1
            a.flat[i] = q
    a = a.astype(np.int64)
    q1 = (a + (1 << 17)) >> 18
    r = a - (q1 << 18)
    q2 = (r + 256) >> 9
    q3 = r - (q2 << 9)
    sgn = np.where((b >> np.uint64(63)) != 0, -1.0, 1.0)
    return sgn * q1 * 2.0 ** -8, sgn * q2 * 2.0 ** -17, sgn * q3 * 2.0 ** -26, sgn * a


def test_integer_bits_split():
    rng = np.random.default_rng(8)
    n = 20000
    for k in (-3, 0, 2, 7):
        v = rng.uniform(-1, 1, n) * 2.0 ** -rng.integers(0, 45, n) * 2.0 ** k
        v[:5] = [2.0 ** k, -(2.0 ** k), 0.0, 2.0 ** (k - 27), 3 * 2.0 ** (k - 28)]
        h, m, lo, q = split_bits(v, k)
        x = v / 2.0 ** k
        for part, qu in ((h, 2.0 ** -8), (m, 2.0 ** -17), (lo, 2.0 ** -26)):
            kk = part / qu
            assert np.all(kk == np.rint(kk)) and np.all(np.abs(kk) <= 256)
            assert _is_bf16_exact(part.astype(np.float32))
            assert np.all(part.astype(np.float32).astype(np.float64) == part)
        assert np.max(np.abs(h + m + lo - x)) <= 2.0 ** -27
        # q is x * 2^26 rounded to nearest, ties to even (exact in float64 here)
        assert np.array_equal(np.abs(q).astype(np.float64), np.abs(np.rint(x * 2.0 ** 26)))


def round_brick(j, b, g, ntotal):
    k = j * g + ((g - 1 - b) if (j & 1) else b)
    return k if k < ntotal else -1


def test_round_brick_covers_every_brick_once():
    for g in (1, 2, 7, 152):
        for ntotal in (0, 1, g - 1, g, g + 1, 3 * g + 5, 45 * g + 73):
            if ntotal < 0:
                continue
            seen = []
            for b in range(g):
                j = 0
                while j * g < ntotal:
                    k = round_brick(j, b, g, ntotal)
                    if k >= 0:
                        seen.append(k)
                    j += 1
            assert sorted(seen) == list(range(ntotal)), (g, ntotal)
