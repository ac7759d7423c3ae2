"""The tensor kernels' FP16 digit planes (wannier90_gb300/csrc/oz.cuh pack_digits7 for the
M update's 7-bit digits, csrc/k_oz_exp.cu slice_run8_h for the exp's 8-bit digits),
restated bit for bit in NumPy: a byte permute of two values' words, a mask, 0x6400 in
the upper bits of each half and one packed FP16 subtraction.  Every digit must be the
serial centred recoding's (digits7 / digits7x8 in oz.cuh), lie in [-128, 128] and be
exact in FP16, and the digits must sum back to the scaled integer N -- over random N of
full width and the extremes."""
import numpy as np

M64 = (1 << 64) - 1


def _byte_perm(x, y, sel):
    b = [(x >> (8 * i)) & 255 for i in range(4)] + [(y >> (8 * i)) & 255 for i in range(4)]
    r = 0
    for n in range(4):
        nib = (sel >> (4 * n)) & 15
        v = b[nib & 7]
        if nib & 8:
            v = 255 if v & 128 else 0
        r |= v << (8 * n)
    return r


def _f16(bits):
    return float(np.array([bits & 0xFFFF], dtype=np.uint16).view(np.float16)[0])


def _sub_f16x2(x, c):
    """sub.rn.f16x2 of two packed pairs; the test requires the difference to be exact."""
    out = []
    for sh in (0, 16):
        d = _f16(x >> sh) - _f16(c >> sh)
        assert float(np.float16(d)) == d
        out.append(d)
    return out


def _sar(v, s):
    v = v - (1 << 64) if v >= (1 << 63) else v
    return v >> s


def _serial(n, bits, ndig):
    x = [0] * ndig
    for t in range(ndig - 1, 0, -1):
        lo = n & ((1 << bits) - 1)
        d = lo - ((lo & (1 << (bits - 1))) << 1)
        x[t] = d
        n = (n - d) >> bits
    x[0] = n
    return x


def _planes7(na, nb):
    """pack_digits7's two values: 7 planes of (digit of a, digit of b)."""
    ma, mb = (na + 0x20408102040) & M64, (nb + 0x20408102040) & M64
    la, lb, ha, hb = ma & 0xFFFFFFFF, mb & 0xFFFFFFFF, ma >> 32, mb >> 32
    fsr = lambda lo, hi: ((hi << 32 | lo) >> 28) & 0xFFFFFFFF          # __funnelshift_r(lo, hi, 28)
    q = [_byte_perm(la, lb, 0x5410), _byte_perm(la >> 14, lb >> 14, 0x5410), _byte_perm(fsr(la, ha), fsr(lb, hb), 0x5410)]
    w = [None] * 7
    for j in range(3):
        w[6 - 2 * j] = _sub_f16x2((q[j] & 0x007F007F) | 0x64006400, 0x64406440)
        w[5 - 2 * j] = _sub_f16x2(((q[j] >> 7) & 0x007F007F) | 0x64006400, 0x64406440)
    ta, tb = _sar(ma, 42) + 128, _sar(mb, 42) + 128
    assert 0 <= ta <= 256 and 0 <= tb <= 256
    w[0] = _sub_f16x2(ta | (tb << 16) | 0x64006400, 0x64806480)
    return w


def _planes8(na, nb):
    """slice_run8_h's two values: 7 planes of (digit of a, digit of b)."""
    ma, mb = (na + 0x808080808080) & M64, (nb + 0x808080808080) & M64
    la, lb, ha, hb = ma & 0xFFFFFFFF, mb & 0xFFFFFFFF, ma >> 32, mb >> 32
    w = [None] * 7
    for t in range(6):
        bt = t & 3
        sel = bt | (bt << 4) | ((4 + bt) << 8) | ((4 + bt) << 12)
        p = _byte_perm(la if t < 4 else ha, lb if t < 4 else hb, sel)
        w[6 - t] = _sub_f16x2((p & 0x00FF00FF) | 0x64006400, 0x64806480)
    ta, tb = _sar(ma, 48) + 128, _sar(mb, 48) + 128
    assert 0 <= ta <= 256 and 0 <= tb <= 256
    w[0] = _sub_f16x2(ta | (tb << 16) | 0x64006400, 0x64806480)
    return w


def _values(rng, top, n):
    ext = [0, 1, -1, top, -top, top - 1, 1 - top, 63, -64, 64, 127, -128, 128]
    v = [int(x) for x in rng.integers(-top, top + 1, n, dtype=np.int64)]
    return ext + v


def _check(planes, bits, top, n=20000):
    rng = np.random.default_rng(bits)
    vals = _values(rng, top, n)
    for a, b in zip(vals[0::2], vals[1::2]):
        w = planes(a, b)
        for k, v in enumerate((a, b)):
            d = [int(w[t][k]) for t in range(7)]
            assert d == _serial(v, bits, 7), (v, d)
            assert all(abs(x) <= 128 for x in d)
            assert sum(x << (bits * (6 - t)) for t, x in enumerate(d)) == v


def test_seven_bit_planes_match_the_serial_recoding():
    _check(_planes7, 7, 1 << 49)


def test_eight_bit_planes_match_the_serial_recoding():
    _check(_planes8, 8, 1 << 55)
