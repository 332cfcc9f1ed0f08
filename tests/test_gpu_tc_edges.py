"""Worst cases of the tensor-core transform engine, bit-exact against the CPU
oracle.

The engine is exact by construction under three conditions, and these tests
drive each to its edge:

* every fp16 MMA column sum is an integer below 2^24 in magnitude (8-bit
  digits: inputs of all q-1 and of all-0xFF bytes put every limb-fed digit at
  its maximum);
* the two-operation carry of digit-fed groups needs each constant column's
  sum of |digit| to be at most 32512 -- the engine measures it when it builds
  a modulus's constants and refuses the modulus above it (driven here by
  lowering the bound on a fresh context);
* the last group's float quotient estimate with one correction each way
  needs q's top limb >= 32 and floor(q/2) <= 0x7F7F...7F: moduli exactly at
  both admission edges run bit-exact, moduli just outside are refused.

hmpc's own transform (hmpc/expr/number_theoretic_transform.hpp:144-197,
262-549) ends every product with REDC's conditional subtract
(hmpc/core/num/modulo.hpp:63-65), so its outputs are the reduced
representatives these tests compare against (tests/ints/poly_mod.cpp:92-103
checks the same property on the reference).
"""
import numpy as np
import pytest

from hmpc_gb300 import _lib, lhe
from hmpc_gb300.comp import Queue, Tensor

gpu = pytest.mark.gpu

KEY = [0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344, 0xA4093822, 0x299F31D0, 0x082EFA98, 0xEC4E6C89]
P_64 = 0x8822D80623320001  # tests/expr/crypto/lhe/enc.cpp:16

# NTT-friendly primes (q = 1 mod 2^17) at the engine's admission edges, per
# limb count: the top limb exactly 32 (lowest accepted), the largest prime
# with floor(q/2) <= 0x7F7F...7F (highest accepted); and just outside both
EDGE = {
    2: {"low": 0x20000E0001, "high": 0xFEFEFEFEFEE40001,
        "below": 0x1F002C0001, "above": 0xFEFEFEFEFF9A0001},
    4: {"low": 0x200000000000000000002C0001, "high": 0xFEFEFEFEFEFEFEFEFEFEFEFEFE860001,
        "below": 0x1F0000000000000000000E0001, "above": 0xFEFEFEFEFEFEFEFEFEFEFEFEFF000001},
    8: {"low": 0x20000000000000000000000000000000000000000000000000006A0001,
        "high": 0xFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFDAC0001,
        "below": 0x1F00000000000000000000000000000000000000000000000000920001,
        "above": 0xFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFEFF580001},
}
ACCEPTED = [(limbs, side) for limbs in (2, 4, 8) for side in ("low", "high")]
COLUMN_BOUND = 32512


@pytest.fixture(scope="module")
def queue():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    q = Queue(key=KEY)
    yield q
    q.close()


def worst_values(value, count, seed):
    """stored representatives that maximise the digits: q-1, the all-0xFF
    value below q's top bit, zero, and random residues, interleaved"""
    rng = np.random.default_rng(seed)
    top = (1 << (value.bit_length() - 1)) - 1
    pool = [value - 1, top, 0, value - 2, (value - 1) // 2, (value + 1) // 2]
    out = []
    for i in range(count):
        k = i % 8
        out.append(pool[k] if k < len(pool) else int.from_bytes(rng.bytes(40), "little") % value)
    return out


def stored(oracle, mod, values):
    return oracle.planar(values, mod.limbs)


def tensor_plan(gm, n, batch, splits=1):
    for inverse in (False, True):
        gm.set_plan(n, batch, inverse, radix_bits=0, local_bits=splits)
        assert gm.plan(n, batch, inverse)["radix_bits"] == 0


def test_edge_moduli_have_the_expected_limbs(oracle):
    for limbs, edge in EDGE.items():
        for side, value in edge.items():
            m = oracle.Modulus(value)
            assert m.limbs == limbs, (limbs, side)
            assert value % (1 << 17) == 1
            top = value >> (32 * (limbs - 1))
            half = value // 2
            bound = int("7F" * (4 * limbs), 16)
            accepted = top >= 32 and half <= bound
            assert accepted == (side in ("low", "high")), (limbs, side)


@gpu
@pytest.mark.parametrize("limbs", [2, 4, 8])
@pytest.mark.parametrize("side", ["below", "above"])
def test_moduli_outside_the_edges_are_refused(queue, limbs, side):
    gm = queue.modulus(EDGE[limbs][side])
    with pytest.raises(_lib.HmpcError) as err:
        gm.set_plan(1 << 10, 2, False, radix_bits=0)
    assert err.value.code == 2


@gpu
@pytest.mark.parametrize("limbs,side", ACCEPTED)
@pytest.mark.parametrize("n,batch", [(16, 9), (64, 3), (1 << 10, 130), (1 << 13, 2)])
@pytest.mark.parametrize("splits", [1, 2])
def test_worst_digits_forward_and_inverse(queue, oracle, limbs, side, n, batch, splits, cpu_threads):
    value = EDGE[limbs][side]
    om, gm = oracle.Modulus(value), queue.modulus(value)
    tensor_plan(gm, n, batch, splits)
    x = stored(oracle, om, worst_values(value, n * batch, n + batch + limbs))
    y = queue.ntt(Tensor.from_numpy(gm, x, (batch,), n))
    assert np.array_equal(y.numpy(), oracle.ntt(om, n, batch, src=x, threads=cpu_threads))
    assert np.array_equal(queue.intt(y).numpy(), x)
    # the inverse fed directly with the worst digits (its first group reads limbs)
    z = queue.intt(Tensor.from_numpy(gm, x, (batch,), n))
    assert np.array_equal(z.numpy(), oracle.ntt(om, n, batch, src=x, inverse=True, threads=cpu_threads))
    assert _lib.call("hmpc_context_synchronize", queue.handle) == 0


@gpu
@pytest.mark.parametrize("limbs,side", ACCEPTED)
def test_all_q_minus_one_at_full_depth(queue, oracle, limbs, side, cpu_threads):
    """five groups (N = 2^15): every group fed by the largest digits the one
    before it can carry out"""
    value = EDGE[limbs][side]
    om, gm = oracle.Modulus(value), queue.modulus(value)
    n, batch = 1 << 15, 2
    tensor_plan(gm, n, batch)
    x = stored(oracle, om, [value - 1] * (n * batch))
    y = queue.ntt(Tensor.from_numpy(gm, x, (batch,), n))
    assert np.array_equal(y.numpy(), oracle.ntt(om, n, batch, src=x, threads=cpu_threads))
    z = queue.intt(Tensor.from_numpy(gm, x, (batch,), n))
    assert np.array_equal(z.numpy(), oracle.ntt(om, n, batch, src=x, inverse=True, threads=cpu_threads))


@gpu
@pytest.mark.parametrize("limbs,side", ACCEPTED)
@pytest.mark.parametrize("vx2", [1, 64])
def test_fused_cbd_at_the_edges(queue, oracle, limbs, side, vx2, cpu_threads):
    value = EDGE[limbs][side]
    om, gm = oracle.Modulus(value), queue.modulus(value)
    n, batch = 1 << 12, 3
    tensor_plan(gm, n, batch)
    nonce = [0xFFFFFFFE, 0xFFFFFFFF, 9]
    queue.nonce = nonce
    y = queue.ntt_centered_binomial(gm, n, (batch,), vx2)
    ref = oracle.ntt(om, n, batch, sampler="cbd", variance_x2=vx2, key=KEY, nonce=nonce, threads=cpu_threads)
    assert np.array_equal(y.numpy(), ref)


@gpu
@pytest.mark.parametrize("limbs,side", [(4, "low"), (4, "high"), (8, "low"), (8, "high")])
def test_stacked_encryption_at_the_edges(queue, oracle, limbs, side, cpu_threads):
    """the small-integer first group (p * e + lift(m), |x| < 2^70) and the
    stacked groups with plaintexts at the centring edges of the lift
    (v > floor(p/2) becomes v - p)"""
    value = EDGE[limbs][side]
    n, batch = 1 << 12, 3
    om_q, om_p = oracle.Modulus(value), oracle.Modulus(P_64)
    gq, gp = queue.modulus(value), queue.modulus(P_64)
    queue.nonce = [3, 1, 4]
    s, key = lhe.keygen(queue, gq, gp, n)
    _, a_ref, b_ref, nonce = oracle.lhe_keygen(om_q, om_p, n, KEY, [3, 1, 4], threads=cpu_threads)
    assert np.array_equal(key.a.numpy(), a_ref)
    gq.set_plan(n, batch, False, radix_bits=0)
    canonical = [P_64 - 1, (P_64 - 1) // 2, (P_64 + 1) // 2, 0, 1]
    vals = [canonical[i % len(canonical)] for i in range(n * batch)]
    msgs_ref = oracle.from_uint(om_p, oracle.planar(vals, om_p.limbs))
    # half the plaintexts as raw representatives p - 1 (the loader's largest)
    msgs_ref[:, : n] = oracle.planar([P_64 - 1] * n, om_p.limbs)
    msgs = Tensor.from_numpy(gp, msgs_ref, (batch,), n)
    queue.nonce = nonce
    ct = lhe.enc(queue, key, msgs, gq)
    c0, c1, _ = oracle.lhe_enc(om_q, om_p, n, batch, a_ref, b_ref, msgs_ref, False, KEY, nonce,
                               threads=cpu_threads)
    assert np.array_equal(ct.c0.numpy(), c0)
    assert np.array_equal(ct.c1.numpy(), c1)


@gpu
@pytest.mark.parametrize("limbs,side", ACCEPTED)
def test_column_bound_of_edge_moduli(queue, limbs, side):
    """the largest constant column sum of |digit| stays within the carry's
    range for every group shape of both directions"""
    gm = queue.modulus(EDGE[limbs][side])
    for log_n in (4, 5, 6, 10, 15):
        for inverse in (False, True):
            for splits in (1, 2):
                top = gm.tc_column_max(1 << log_n, inverse, splits)
                assert 0 < top <= COLUMN_BOUND, (log_n, inverse, splits, top)


@gpu
def test_constants_over_the_column_bound_are_refused(oracle, cpu_threads):
    """A context whose bound is one below a modulus's largest column sum
    refuses that modulus's transform (HMPC_ERROR_UNSUPPORTED, the context stays
    usable, the tuner keeps the CUDA-core tiles); at the bound it is accepted
    and bit-exact."""
    value = EDGE[8]["high"]
    n, batch = 1 << 10, 4
    om = oracle.Modulus(value)
    x = stored(oracle, om, worst_values(value, n * batch, 5))
    ref = oracle.ntt(om, n, batch, src=x, threads=cpu_threads)
    probe = Queue(key=KEY)
    top = probe.modulus(value).tc_column_max(n)
    probe.close()
    assert 0 < top <= COLUMN_BOUND

    refusing = Queue(key=KEY)
    with pytest.raises(_lib.HmpcError):
        refusing.set_tc_column_bound(COLUMN_BOUND + 1)
    refusing.set_tc_column_bound(top - 1)
    gm = refusing.modulus(value)
    gm.set_plan(n, batch, False, radix_bits=0)
    dx = Tensor.from_numpy(gm, x, (batch,), n)
    with pytest.raises(_lib.HmpcError) as err:
        refusing.ntt(dx)
    assert err.value.code == 2
    assert gm.tc_column_max(n) == top
    gm.tune(n, batch)
    assert gm.plan(n, batch)["radix_bits"] != 0
    assert np.array_equal(refusing.ntt(dx).numpy(), ref)
    refusing.close()

    accepting = Queue(key=KEY)
    accepting.set_tc_column_bound(top)
    gm = accepting.modulus(value)
    gm.set_plan(n, batch, False, radix_bits=0)
    before = accepting.launches
    y = accepting.ntt(Tensor.from_numpy(gm, x, (batch,), n))
    assert accepting.launches - before == 4  # four tensor-core groups for 2^10
    assert np.array_equal(y.numpy(), ref)
    accepting.close()
