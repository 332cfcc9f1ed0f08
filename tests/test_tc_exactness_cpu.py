"""The arithmetic arguments the tensor-core transform's exactness rests on,
checked on the CPU with exact integers at the extremes of their ranges.

These restate three pieces of hmpc_gb300/csrc/tensor_ntt.cuh step by step:

* DigitCarryByte (two float operations per digit, groups fed by digits):
  T = s + x must stay in [2^23, 2^24), where the low byte of T's bits is the
  biased digit.  Column sums reach |s| <= 128 * 32512 when every constant
  column's sum of |digit| is at the engine's bound 32512;
* DigitCarry (four operations per digit, groups fed by limbs): every
  intermediate an integer in [0, 2^24), with column sums of up to
  K * 255 * 128 (K = 8 elements x 4L bytes);
* tc_reduce: the quotient estimate from the value's signed top word in f32
  (times 2^(32(L-1)) / q rounded to f32) leaves a remainder in [-q, 2q), so
  one correction each way
  gives the reduced representative, for |value / q| < 2^15 and q at both
  admission edges (top limb 32, floor(q/2) = 0x7F..7F).

A float step is exact when its result is an integer of magnitude below 2^24;
each step below asserts that range and then uses exact integer arithmetic.
"""
import numpy as np
import pytest

EDGE_Q = [
    0x20000E0001, 0xFEFEFEFEFEE40001,
    0x200000000000000000002C0001, 0xFEFEFEFEFEFEFEFEFEFEFEFEFE860001,
    0x20000000000000000000000000000000000000000000000000006A0001,
    0xFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFDAC0001,
    0xCFF479B9B12CCF05AF55BCA0D7AE005D53E20D920B577D2785F3A1F156740001,
]
TWO23, TWO24 = 1 << 23, 1 << 24


def byte_carry(sums):
    """DigitCarryByte over column sums, then two carry digits: the biased
    digit bytes and the final carry state"""
    x = 12583040  # carry 0: 128 + C2, C2 = 2^23 + 2^22
    out = []
    for s in list(sums) + [0, 0]:
        t = s + x  # FADD: exact while an integer below 2^24
        assert TWO23 <= t < TWO24, t
        nxt = t // 256 + 12533888  # FFMA round-down: floor, with the result in [2^23, 2^24)
        assert TWO23 <= nxt < TWO24
        out.append(t & 255)  # low byte of the float bits of T (mantissa T - 2^23)
        x = nxt
    return out, x - 12583040  # carry()


def four_op_carry(sums):
    """DigitCarry over column sums: biased digit bytes and the carry out"""
    x = 8421504  # carry 0: 128 + C, C = 2^23 + 2^15
    out = []
    for s in sums:
        tc = s + x
        assert 0 <= tc < TWO24, tc
        x = tc // 256 + TWO23  # FFMA round-down
        assert TWO23 <= x < TWO24
        z = x - 8421376  # next carry + 128
        d = tc - 256 * z  # FFMA: 2^23 + digit + 128
        assert TWO23 <= d < TWO23 + 256
        out.append(d - TWO23)
    return out, x - TWO23 - 32896


def value_of(digits, carry):
    return sum((d - 128) << (8 * k) for k, d in enumerate(digits)) + (carry << (8 * len(digits)))


def extreme_sequences(limit, count, rng):
    seqs = [[limit] * count, [-limit] * count, [limit, -limit] * (count // 2), [0] * count]
    seqs += [[int(v) for v in rng.integers(-limit, limit + 1, size=count)] for _ in range(200)]
    seqs += [[int(v) for v in rng.choice([-limit, limit, 0, 1, -1], size=count)] for _ in range(200)]
    return seqs


@pytest.mark.parametrize("dc", [8, 16, 32])
def test_two_operation_carry_at_the_column_bound(dc):
    limit = 128 * 32512  # |digit| <= 128 times the largest column sum of |digit|
    rng = np.random.default_rng(dc)
    for sums in extreme_sequences(limit, dc, rng):
        digits, carry = byte_carry(sums)
        assert carry == 0  # two carry digits hold what is left
        assert value_of(digits, 0) == sum(s << (8 * k) for k, s in enumerate(sums))


def test_two_operation_carry_needs_the_bound():
    """just past the bound the first T leaves [2^23, 2^24)"""
    with pytest.raises(AssertionError):
        byte_carry([128 * 32512 + 16640] * 32)


@pytest.mark.parametrize("limbs", [2, 4, 8])
def test_four_operation_carry_of_limb_input(limbs):
    dc = 4 * limbs
    k = 8 * dc  # K slots: 8 elements x 4L bytes
    hi, lo = k * 255 * 127, -k * 255 * 128
    rng = np.random.default_rng(limbs)
    seqs = [[hi] * dc, [lo] * dc, [hi, lo] * (dc // 2)]
    seqs += [[int(v) for v in rng.integers(lo, hi + 1, size=dc)] for _ in range(300)]
    for sums in seqs:
        digits, carry = four_op_carry(sums)
        assert value_of(digits, carry) == sum(s << (8 * j) for j, s in enumerate(sums))


def quotient_estimate(value, q, limbs):
    """tc_reduce's t from the top word of the value (the carry out and limb
    L-1), in f32 exactly as the device rounds"""
    top_d = (q >> (32 * (limbs - 1))) + ((q >> (32 * (limbs - 2))) & 0xFFFFFFFF) / 4294967296.0
    inv_q_top = np.float32(1.0 / top_d)
    u = value % (1 << (32 * limbs))  # limbs as stored (two's complement wrap)
    top = value >> (32 * limbs)  # signed carry above the limbs
    x_top = (u >> (32 * (limbs - 1))) & 0xFFFFFFFF
    # the signed top word as one 64-bit integer, converted once to f32
    word = top * (1 << 32) + x_top
    est = np.float32(np.float32(np.int64(word)) * inv_q_top)
    return int(np.floor(np.float64(est)))


def quotient_estimate_two_roundings(value, q, limbs):
    """the estimate with the top limb converted to f32 on its own before the
    signed carry is added (the form the engine must not use)"""
    top_d = (q >> (32 * (limbs - 1))) + ((q >> (32 * (limbs - 2))) & 0xFFFFFFFF) / 4294967296.0
    inv_q_top = np.float32(1.0 / top_d)
    u = value % (1 << (32 * limbs))
    top = value >> (32 * limbs)
    x_top = (u >> (32 * (limbs - 1))) & 0xFFFFFFFF
    est = np.float32(np.float64(top) * 4294967296.0 + np.float64(np.float32(x_top)))
    return int(np.floor(np.float64(np.float32(est * inv_q_top))))


@pytest.mark.parametrize("q", EDGE_Q)
def test_one_correction_each_way_after_the_estimate(q):
    limbs = (q.bit_length() + 31) // 32
    rng = np.random.default_rng(q % 1000)
    ks = [0, 1, -1, 2, -2, (1 << 15) - 1, -(1 << 15) + 1, 4095, -4096]
    ks += [int(v) for v in rng.integers(-(1 << 15) + 1, 1 << 15, size=64)]
    rs = [0, 1, q - 1, q // 2, (q + 1) // 2, q - 2]
    rs += [int.from_bytes(rng.bytes(40), "little") % q for _ in range(16)]
    for k in ks:
        for r in rs:
            value = k * q + r
            t = quotient_estimate(value, q, limbs)
            rem = value - t * q
            assert -q <= rem < 2 * q, (k, r, t)


def test_top_limb_alone_in_f32_would_need_more_corrections():
    """a negative value at the smallest admitted top limb: rounding the top
    limb to f32 before the carry cancels it puts the estimate two quotients off"""
    q = EDGE_Q[4]  # top limb 32, 8 limbs
    t = quotient_estimate_two_roundings(-2 * q, q, 8)
    assert not (-q <= -2 * q - t * q < 2 * q)
    t = quotient_estimate(-2 * q, q, 8)
    assert -q <= -2 * q - t * q < 2 * q
