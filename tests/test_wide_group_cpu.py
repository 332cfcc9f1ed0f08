"""The algebra of the tensor-core engine's wide first group, checked on the
CPU with the Python oracle's own stage formulas (no GPU).

The forward transform's first six stages act on the top six element bits as
one 64 x 64 matrix per column.  The engine builds it from the first two
three-stage groups' matrices: A (stages 0-2, top three bits) and B_kh
(stages 3-5, the next three bits, one matrix per value kh of the top three
bits after A), G6[(kh, kl)][(ih, il)] = B_kh[kl][il] * A[kh][ih]
(hmpc_gb300/csrc/tensor_ntt.cuh, tc_combine6_kernel).  Here every matrix
comes from applying the reference's butterflies (the oracle's restatement of
number_theoretic_transform.hpp:144-197) to unit vectors, and the product is
compared with the six-stage map entry by entry; the p-scaled variant the
encryption uses is the same map times p.
"""
import pytest

from oracle import pyoracle

PRIMES = [12289, 0x8822D80623320001]  # 3 * 2^12 + 1 (one limb); the reference's p (two limbs)


def stages(m, n, values, first, last):
    """forward stages [first, last) of the transform of one polynomial"""
    bits = n.bit_length() - 1
    t = pyoracle.twiddles(m, n)
    a = list(values)
    for s in range(first, last):
        length = 1 << s
        step = n // length // 2
        for tid in range(n // 2):
            ps = tid // step
            tgt = ps * step * 2 + tid % step
            u, v = a[tgt], m.mul(a[tgt + step], t[length + ps])
            a[tgt], a[tgt + step] = m.add(u, v), m.sub(u, v)
    assert bits >= last
    return a


def column(m, n, index, first, last):
    unit = [0] * n
    unit[index] = m.one
    return stages(m, n, unit, first, last)


@pytest.mark.parametrize("q", PRIMES)
@pytest.mark.parametrize("log_n", [8, 10])
def test_six_stages_factor_into_the_first_two_groups(q, log_n):
    m = pyoracle.Mod(q)
    n = 1 << log_n
    lo = log_n - 6

    def element(high, low, c):
        return (((high << 3) | low) << lo) | c

    for c in (0, (1 << lo) - 1):
        g6 = {i: column(m, n, element(i >> 3, i & 7, c), 0, 6) for i in range(64)}
        a = {ih: column(m, n, element(ih, 0, c), 0, 3) for ih in range(8)}
        for kh in range(8):
            b = {il: column(m, n, element(kh, il, c), 3, 6) for il in range(8)}
            for kl in range(8):
                for i in range(64):
                    ih, il = i >> 3, i & 7
                    a_entry = a[ih][element(kh, 0, c)]
                    b_entry = b[il][element(kh, kl, c)]
                    assert g6[i][element(kh, kl, c)] == m.mul(b_entry, a_entry)
        # the map touches only the 64 elements of this column
        for i in range(64):
            others = [x for e, x in enumerate(g6[i]) if (e & ((1 << lo) - 1)) != c]
            assert not any(others)


def test_p_scaled_map_is_the_map_of_p_times_the_input():
    """the encryption's p * w draws: constants G6 * p give the six-stage map
    of p * w (linearity), so the samples stay single digits"""
    m = pyoracle.Mod(PRIMES[0])
    p = 97
    n = 1 << 8
    x = [m.mont(v % m.q) for v in range(-20, n - 20)]
    direct = stages(m, n, [m.mul(v, m.mont(p)) for v in x], 0, 6)
    scaled = [m.mul(v, m.mont(p)) for v in stages(m, n, x, 0, 6)]
    assert direct == scaled
