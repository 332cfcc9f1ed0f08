"""Pin the CPU oracle against the reference's own known-answer vectors
(tests/golden/reference_kats.json, extracted from hmpc's Catch2 tests) and
against the independent big-integer restatement (oracle/pyoracle.py)."""
import random

import numpy as np
import pytest

from oracle import pyoracle as py


def test_chacha_quarter_round(oracle, kats):
    qr = kats["chacha20"]["quarter_round"]
    assert oracle.quarter_round(*qr["input"]) == qr["output"]
    assert list(py.quarter_round(*qr["input"])) == qr["output"]


def test_chacha_blocks(oracle, kats):
    blocks = kats["chacha20"]["blocks"]
    assert len(blocks) == 6
    for b in blocks:
        assert oracle.chacha20_block(b["key"], b["counter"], b["nonce"]) == b["words"], b["lines"]
        assert py.chacha20_block(b["key"], b["counter"], b["nonce"]) == b["words"], b["lines"]


def test_generator_refills_after_sixteen_words(oracle):
    key = list(range(8))
    nonce = [7, 8, 9]
    g = oracle.Generator(key, nonce, 5)
    words = [g.next() for _ in range(40)]
    expect = (oracle.chacha20_block(key, 5, nonce) + oracle.chacha20_block(key, 6, nonce)
              + oracle.chacha20_block(key, 7, nonce))[:40]
    assert words == expect
    pg = py.Generator(key, nonce, 5)
    assert [pg.next() for _ in range(40)] == expect


def test_montgomery_constants(oracle, kats):
    k = kats["mod"]
    m = oracle.Modulus(k["p"])
    assert m.one == k["R_mod_p"]["value"]
    assert m.from_uint(512) == k["montgomery_512"]["value"]
    assert m.to_uint(m.from_uint(512)) == 512
    # powers of 512 (tests/ints/mod.cpp:37-42)
    x = m.from_uint(512)
    acc = m.one
    for e in range(1, 6):
        acc = m.mul(acc, x)
        assert m.to_uint(acc) == 512 ** e
    assert m.to_uint(m.from_uint(k["p"])) == 0
    assert m.to_uint(m.from_uint(k["p"] + 1)) == 1


def test_montgomery_conversions(oracle, kats):
    k = kats["mod"]
    m = oracle.Modulus(k["p"])
    for c in k["conversions"]:
        if c["input_negative"]:
            v = m.from_uint(c["input"] % k["p"])
            got = m.to_uint(m.sub(0, v))
        else:
            got = m.to_uint(m.from_uint(c["input"]))
        assert got == c["canonical"], c["line"]
    assert m.to_uint(m.from_int(-1)) == k["p"] - 1


def test_cross_modulus_cast(oracle):
    # tests/ints/mod.cpp:57-79 with q = 99
    p = oracle.Modulus(0x2FAEADBE7A0195C011AC195AD10269830E8001)
    q = oracle.Modulus(99)
    for i in range(50):
        assert p.to_uint(p.cast_from(q, q.from_uint(i))) == i
        assert q.to_uint(q.cast_from(p, p.from_uint(i))) == i
        if i:
            assert p.to_uint(p.cast_from(q, q.from_int(-i))) == p.value - i
            assert q.to_uint(q.cast_from(p, p.from_int(-i))) == 99 - i


def test_root_of_unity_pins(oracle, kats):
    k = kats["poly_mod_ntt"]
    m = oracle.Modulus(k["q"])
    root = m.root_of_unity(2 * k["N"])
    assert m.to_uint(root) == k["root"]["value"]
    table_inv = m.twiddles(k["N"], inverse=True)
    # T_inv[bitrev(1)] = T_inv[N/2] is the inverse root
    inv = oracle.from_limbs(table_inv[k["N"] // 2])
    assert m.to_uint(inv) == k["inverse_root"]["value"]
    pm = py.Mod(k["q"])
    assert pm.canon(py.root_of_unity(pm, 2 * k["N"])) == k["root"]["value"]


def test_root_of_unity_property(oracle, kats):
    k = kats["root_of_unity"]
    m = oracle.Modulus(k["p"])
    root = m.to_uint(m.root_of_unity(k["degree"]))
    assert pow(root, k["degree"], k["p"]) == 1
    for i in range(1, k["degree"]):
        assert pow(root, i, k["p"]) != 1


@pytest.mark.slow
def test_ntt_known_answers_and_round_trip(oracle, kats, cpu_threads):
    k = kats["poly_mod_ntt"]
    n = k["N"]
    m = oracle.Modulus(k["q"])
    batch = 2
    x = oracle.from_uint(m, oracle.planar(list(range(n)) * batch, m.limbs))
    y = oracle.ntt(m, n, batch, src=x, threads=cpu_threads)
    yc = oracle.to_uint(m, y)
    for j in range(batch):
        for rec in k["ntt_outputs"]:
            got = oracle.from_limbs(yc[:, j * n + rec["index"]])
            assert got == rec["canonical"], rec["line"]
    z = oracle.ntt(m, n, batch, src=y, inverse=True, threads=cpu_threads)
    assert np.array_equal(z, x)
    zero = np.zeros_like(x)
    assert not oracle.ntt(m, n, batch, src=zero, threads=cpu_threads).any()


MODULI = [
    0x18F25CD9A75CCBD9C146D4ABAEC00001,  # examples/ntt.cpp:22 (L=4)
    0x2FAEADBE7A0195C011AC195AD10269830E8001,  # examples/bgv.cpp:25 (L=5)
    0x8822D80623320001,  # tests/expr/crypto/lhe/enc.cpp:16 (L=2)
    0x8605423C957246B58997DEC24F688AB3DD46CB31C5700001,  # 192-bit (L=6)
    0xCFF479B9B12CCF05AF55BCA0D7AE005D53E20D920B577D2785F3A1F156740001,  # 256-bit (L=8)
]


@pytest.mark.parametrize("q", MODULI)
def test_ntt_matches_pyoracle_and_direct_dft(oracle, q):
    n, batch = 64, 2
    m = oracle.Modulus(q)
    pm = py.Mod(q)
    rng = random.Random(q)
    vals = [pm.mont(rng.randrange(q)) for _ in range(n * batch)]
    y = oracle.ntt(m, n, batch, src=oracle.planar(vals, m.limbs))
    ref = py.ntt(pm, n, batch, vals)
    assert oracle.unplanar(y) == ref
    root = pm.canon(py.root_of_unity(pm, 2 * n))
    dft = py.negacyclic_dft(pm, [pm.canon(v) for v in vals[:n]], root)
    assert [pm.canon(v) for v in ref[:n]] == dft
    z = oracle.ntt(m, n, batch, src=y, inverse=True)
    assert oracle.unplanar(z) == vals
    assert py.ntt(pm, n, batch, ref, inverse=True) == vals


@pytest.mark.parametrize("q", MODULI)
@pytest.mark.parametrize("sampler,vx2", [("cbd", 1), ("cbd", 20), ("uniform", 0)])
def test_sampler_fused_ntt_matches_pyoracle(oracle, q, sampler, vx2):
    n, batch = 32, 3
    key = [0x01234567 * (i + 1) & 0xFFFFFFFF for i in range(8)]
    nonce = [5, 0xFFFFFFFF, 2]
    m = oracle.Modulus(q)
    pm = py.Mod(q)
    y = oracle.ntt(m, n, batch, sampler=sampler, variance_x2=vx2, key=key, nonce=nonce)
    ref = py.ntt(pm, n, batch, sampler=sampler, variance_x2=vx2, key=key, nonce=nonce)
    assert oracle.unplanar(y) == ref


@pytest.mark.parametrize("q", MODULI)
def test_elementwise_samplers_match_pyoracle(oracle, q):
    key = [9, 8, 7, 6, 5, 4, 3, 2]
    nonce = [1, 2, 3]
    m = oracle.Modulus(q)
    pm = py.Mod(q)
    u = oracle.unplanar(oracle.sample_uniform(m, 40, key, nonce))
    assert u == [py.uniform(pm, py.Generator(key, nonce, e)) for e in range(40)]
    for vx2 in (1, 20):
        c = oracle.unplanar(oracle.sample_cbd(m, 40, key, nonce, vx2))
        vals = [py.cbd(py.Generator(key, nonce, e), vx2) for e in range(40)]
        assert c == [pm.mont(v % q) for v in vals]
        assert all(abs(v) <= vx2 for v in vals)


def test_cbd_distribution(oracle):
    g = oracle.Generator([1] * 8, [0] * 3, 0)
    half = [g.cbd(1) for _ in range(20000)]
    assert set(half) <= {-1, 0, 1}
    assert abs(half.count(0) / len(half) - 0.5) < 0.02
    ten = [g.cbd(20) for _ in range(20000)]
    assert min(ten) >= -20 and max(ten) <= 20
    assert abs(np.var(ten) - 10.0) < 0.6


def test_uniform_bit_width_and_range(oracle):
    # tests/random/uniform.cpp: drowned draws carry bit_width(Q-1)+80 bits
    q = MODULI[4]
    m = oracle.Modulus(q)
    pm = py.Mod(q)
    g = py.Generator([3] * 8, [0] * 3, 0)
    v, n = g.words(pm.bits + 80)
    assert n == (256 + 80 + 31) // 32
    vals = oracle.unplanar(oracle.sample_uniform(m, 64, [3] * 8, [0] * 3))
    assert all(0 <= x < q for x in vals)


def test_fma_and_binary_ops(oracle):
    q = 0x95D13129B10A9D6E4BFC74319391CCE9  # examples/fma.cpp:15
    m = oracle.Modulus(q)
    pm = py.Mod(q)
    rng = random.Random(1)
    a, b, c = ([pm.mont(rng.randrange(q)) for _ in range(100)] for _ in range(3))
    d = oracle.unplanar(oracle.fma(m, oracle.planar(a, 4), oracle.planar(b, 4), oracle.planar(c, 4)))
    assert d == [pm.add(pm.mul(x, y), z) for x, y, z in zip(a, b, c)]
    for op, f in ((oracle.OP_ADD, pm.add), (oracle.OP_SUB, pm.sub), (oracle.OP_MUL, pm.mul)):
        r = oracle.unplanar(oracle.binary(m, op, oracle.planar(a, 4), oracle.planar(b[:10], 4)))
        assert r == [f(x, b[i % 10]) for i, x in enumerate(a)]


def test_nonce_add_carries(oracle):
    assert oracle.nonce_add([0xFFFFFFFF, 0xFFFFFFFF, 0], 1) == [0, 0, 1]
    assert py.nonce_add([0xFFFFFFFF, 0xFFFFFFFF, 0], 1) == [0, 0, 1]
    assert oracle.nonce_add([5, 0, 0], (1 << 33) + 2) == [7, 2, 0]


def test_lhe_round_trip_small(oracle):
    # the shape of tests/expr/crypto/lhe/enc.cpp at a small degree
    p = oracle.Modulus(0x8822D80623320001)
    q = oracle.Modulus(0x591F5B834C0D961F67343BCC8902BDEDA2771F54306FF151162FF8D2B40F4194DC0001)
    n, batch = 256, 8
    a = np.array([[(i >> (32 * j)) & 0xFFFFFFFF for i in range(n)] for j in range(q.limbs)], dtype=np.uint32)
    s = oracle.planar([q.one] * n, q.limbs)
    x = oracle.planar(list(range(n * batch)), p.limbs)
    key = [11] * 8
    c0, c1, nonce = oracle.lhe_enc(q, p, n, batch, a, a, x, True, key, [0, 0, 0])
    assert nonce == [3 * n * batch, 0, 0]
    y = oracle.lhe_dec(q, p, n, batch, s, c0, c1, True)
    assert np.array_equal(y, x)


def test_lhe_keygen_enc_dec_small(oracle):
    p = oracle.Modulus(0x8822D80623320001)
    q = oracle.Modulus(MODULI[4])
    n, batch = 128, 3
    key = [0xDEADBEEF] * 8
    s, a, b, nonce = oracle.lhe_keygen(q, p, n, key, [0, 0, 0])
    assert nonce == [3 * n, 0, 0]
    msgs = oracle.sample_uniform(p, n * batch, key, nonce)
    c0, c1, _ = oracle.lhe_enc(q, p, n, batch, a, b, msgs, False, key, oracle.nonce_add(nonce, n * batch))
    y = oracle.lhe_dec(q, p, n, batch, s, c0, c1, False)
    assert np.array_equal(y, msgs)


def _words_le(byts):
    padded = list(byts) + [0] * (-len(byts) % 4)
    return [padded[i] | padded[i + 1] << 8 | padded[i + 2] << 16 | padded[i + 3] << 24 for i in range(0, len(padded), 4)]


def test_cipher_rfc8439_vector(oracle, kats):
    """RFC 8439 section 2.4.2 (tests/crypto/cipher.cpp): the keystream starts at
    block counter 1, so a zero block is put in front of the message."""
    c = kats["cipher"]
    msg = _words_le(c["plaintext"])
    planar = np.array([[0] * 16 + msg], dtype=np.uint32)
    out = oracle.cipher_enc(c["key"], c["nonce"], planar)
    got = b"".join(int(w).to_bytes(4, "little") for w in out[16:])[: len(c["ciphertext"])]
    assert list(got) == c["ciphertext"]
    back = oracle.cipher_dec(c["key"], c["nonce"], out, 1)
    assert np.array_equal(back, planar)


@pytest.mark.parametrize("limbs", [1, 3, 4, 5, 8, 16])
def test_cipher_batches_equal_plain_keystream(oracle, limbs):
    """the reference's lcm(16, L)-word batches are the plain keystream"""
    key, nonce = [42] + [0] * 7, [1, 0, 0]
    elements = 37
    rng = np.random.default_rng(limbs)
    planar = rng.integers(0, 2**32, size=(limbs, elements), dtype=np.uint64).astype(np.uint32)
    out = oracle.cipher_enc(key, nonce, planar)
    words = elements * limbs
    stream = []
    for blk in range((words + 15) // 16):
        stream += py.chacha20_block(key, blk, nonce)
    flat = planar.T.reshape(-1)
    assert np.array_equal(out, flat ^ np.array(stream[:words], dtype=np.uint32))
