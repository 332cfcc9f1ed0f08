"""Parity of the CUDA path (through the C ABI) with the CPU oracle: bit-exact
for every output, on the same seeds and inputs."""
import random

import numpy as np
import pytest

from hmpc_gb300 import _lib
from hmpc_gb300.comp import Queue, Tensor

pytestmark = pytest.mark.gpu

KEY = [0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344, 0xA4093822, 0x299F31D0, 0x082EFA98, 0xEC4E6C89]

Q_NTT = 0x18F25CD9A75CCBD9C146D4ABAEC00001  # examples/ntt.cpp:22, L=4
Q_BGV_EXAMPLE = 0x2FAEADBE7A0195C011AC195AD10269830E8001  # examples/bgv.cpp:25, L=5
Q_FMA = 0x95D13129B10A9D6E4BFC74319391CCE9  # examples/fma.cpp:15, L=4
Q_192 = 0x8605423C957246B58997DEC24F688AB3DD46CB31C5700001  # L=6
Q_256 = 0xCFF479B9B12CCF05AF55BCA0D7AE005D53E20D920B577D2785F3A1F156740001  # L=8
Q_279 = 0x591F5B834C0D961F67343BCC8902BDEDA2771F54306FF151162FF8D2B40F4194DC0001  # enc.cpp test, L=9
P_64 = 0x8822D80623320001  # tests/expr/crypto/lhe/enc.cpp:16, L=2


@pytest.fixture(scope="module")
def queue():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    q = Queue(key=KEY)
    yield q
    q.close()


def random_residues(oracle, mod, count, seed):
    """uniform canonical values in [0, Q) -> Montgomery form (oracle)"""
    rng = np.random.default_rng(seed)
    words = rng.integers(0, 2**32, size=(mod.limbs, count), dtype=np.uint64).astype(np.uint32)
    words[mod.limbs - 1] &= np.uint32((1 << (mod.bits % 32 or 32)) - 1)
    vals = [v % mod.value for v in oracle.unplanar(words)]
    return oracle.from_uint(mod, oracle.planar(vals, mod.limbs))


def upload(queue, q, arr, shape, n=1):
    return Tensor.from_numpy(queue.modulus(q), arr, shape, n)


@pytest.mark.parametrize("q", [Q_FMA, Q_NTT, Q_256, P_64, Q_279])
@pytest.mark.parametrize("count", [4096, 1001, 4, 1])
def test_fma(queue, oracle, q, count):
    m = oracle.Modulus(q)
    a, b, c = (random_residues(oracle, m, count, s) for s in (1, 2, 3))
    da, db, dc = (upload(queue, q, x, (count,)) for x in (a, b, c))
    d = queue.fma(da, db, dc)
    assert np.array_equal(d.numpy(), oracle.fma(m, a, b, c))


@pytest.mark.parametrize("q", [Q_NTT, Q_192, Q_256, P_64])
@pytest.mark.parametrize("op", [0, 1, 2])
def test_binary_with_broadcast(queue, oracle, q, op):
    m = oracle.Modulus(q)
    n, batch = 64, 5
    a = random_residues(oracle, m, n * batch, 4)
    b = random_residues(oracle, m, n, 5)
    out = queue.binary(op, upload(queue, q, a, (batch,), n), upload(queue, q, b, (), n))
    assert np.array_equal(out.numpy(), oracle.binary(m, op, a, b))
    out = queue.binary(op, upload(queue, q, b, (), n), upload(queue, q, a, (batch,), n))
    assert np.array_equal(out.numpy(), oracle.binary(m, op, b, a, elements=n * batch))


@pytest.mark.parametrize("q,n,batch", [
    (Q_NTT, 4096, 1),
    (Q_NTT, 4, 3),
    (Q_NTT, 8, 1),
    (Q_BGV_EXAMPLE, 1 << 14, 2),
    (Q_192, 1 << 12, 3),
    (Q_192, 1 << 16, 1),
    (Q_256, 1 << 15, 2),
    (Q_256, 1 << 13, 5),
    (P_64, 1 << 15, 2),
    (Q_279, 1 << 11, 2),
])
def test_ntt_round_trip_matches_oracle(queue, oracle, q, n, batch, cpu_threads):
    m = oracle.Modulus(q)
    x = random_residues(oracle, m, n * batch, n + batch)
    dx = upload(queue, q, x, (batch,), n)
    y = queue.ntt(dx)
    ref = oracle.ntt(m, n, batch, src=x, threads=cpu_threads)
    assert np.array_equal(y.numpy(), ref)
    z = queue.intt(y)
    assert np.array_equal(z.numpy(), x)


def test_ntt_known_answers(queue, oracle, kats):
    """ψ, ψ^-1 and five outputs of x_i = i at N = 2^14 (tests/ints/poly_mod.cpp:78-96)."""
    k = kats["poly_mod_ntt"]
    n = k["N"]
    m = oracle.Modulus(k["q"])
    gm = queue.modulus(k["q"])
    assert m.to_uint(gm.root(n)) == k["root"]["value"]
    assert m.to_uint(gm.root(n, inverse=True)) == k["inverse_root"]["value"]
    assert np.array_equal(gm.twiddles(n), m.twiddles(n))
    assert np.array_equal(gm.twiddles(n, True), m.twiddles(n, True))
    x = oracle.from_uint(m, oracle.planar(list(range(n)) * 2, m.limbs))
    y = queue.ntt(upload(queue, k["q"], x, (2,), n))
    yc = oracle.to_uint(m, y.numpy())
    for j in range(2):
        for rec in k["ntt_outputs"]:
            assert oracle.from_limbs(yc[:, j * n + rec["index"]]) == rec["canonical"], rec["line"]
    z = queue.intt(y)
    assert np.array_equal(z.numpy(), x)


def test_ntt_in_place_and_zero(queue, oracle):
    m = oracle.Modulus(Q_256)
    n = 1 << 12
    x = random_residues(oracle, m, 3 * n, 9)
    dx = upload(queue, Q_256, x, (3,), n)
    queue.ntt(dx, out=dx)
    assert np.array_equal(dx.numpy(), oracle.ntt(m, n, 3, src=x))
    zero = upload(queue, Q_256, np.zeros_like(x), (3,), n)
    assert not queue.ntt(zero).numpy().any()


@pytest.mark.parametrize("q", [Q_NTT, Q_192, Q_256, P_64, Q_279])
@pytest.mark.parametrize("sampler,vx2", [("cbd", 1), ("cbd", 20), ("cbd", 64), ("cbd", 7), ("uniform", 0)])
def test_sampler_fused_ntt(queue, oracle, q, sampler, vx2, cpu_threads):
    m = oracle.Modulus(q)
    gm = queue.modulus(q)
    n, batch = 1 << 11, 3
    queue.nonce = [0xFFFFFFF0, 7, 1]
    if sampler == "cbd":
        y = queue.ntt_centered_binomial(gm, n, (batch,), vx2)
    else:
        y = queue.ntt_uniform(gm, n, (batch,))
    assert queue.nonce == oracle.nonce_add([0xFFFFFFF0, 7, 1], n * batch)
    ref = oracle.ntt(m, n, batch, sampler=sampler, variance_x2=vx2, key=KEY, nonce=[0xFFFFFFF0, 7, 1],
                     threads=cpu_threads)
    assert np.array_equal(y.numpy(), ref)


@pytest.mark.parametrize("q", [Q_NTT, Q_192, Q_256, P_64, Q_279, Q_FMA])
def test_elementwise_samplers(queue, oracle, q):
    m = oracle.Modulus(q)
    gm = queue.modulus(q)
    count = 5000
    queue.nonce = [3, 0, 0]
    u = queue.uniform(gm, (count,))
    assert np.array_equal(u.numpy(), oracle.sample_uniform(m, count, KEY, [3, 0, 0]))
    for vx2 in (1, 20):
        nonce = queue.nonce
        c = queue.centered_binomial(gm, (count,), vx2)
        assert np.array_equal(c.numpy(), oracle.sample_cbd(m, count, KEY, nonce, vx2))
    assert queue.nonce == [3 + 3 * count, 0, 0]


@pytest.mark.parametrize("dst,src", [(Q_256, P_64), (P_64, Q_256), (Q_279, P_64), (P_64, Q_279), (Q_NTT, Q_192),
                                     (Q_192, Q_NTT), (Q_FMA, Q_NTT), (Q_NTT, Q_FMA)])
def test_cast(queue, oracle, dst, src):
    md, ms = oracle.Modulus(dst), oracle.Modulus(src)
    x = random_residues(oracle, ms, 3000, 11)
    # include the values around src/2 and the extremes
    edge = [0, 1, ms.value - 1, ms.value // 2, ms.value // 2 + 1, ms.value // 2 - 1]
    e = oracle.from_uint(ms, oracle.planar(edge, ms.limbs))
    x = np.concatenate([x, e], axis=1)
    out = queue.cast(upload(queue, src, x, (x.shape[1],)), queue.modulus(dst))
    assert np.array_equal(out.numpy(), oracle.cast(md, ms, x))


def test_montgomery_conversions(queue, oracle):
    m = oracle.Modulus(Q_256)
    vals = [0, 1, 2, 512, Q_256 - 1] + [random.Random(5).randrange(Q_256) for _ in range(100)]
    canon = oracle.planar(vals, m.limbs)
    dm = queue.to_montgomery(upload(queue, Q_256, canon, (len(vals),)))
    assert np.array_equal(dm.numpy(), oracle.from_uint(m, canon))
    back = queue.from_montgomery(dm)
    assert np.array_equal(back.numpy(), canon)


def test_errors_are_reported(queue):
    gm = queue.modulus(Q_NTT)
    x = Tensor(gm, (1,), 6)
    with pytest.raises(_lib.HmpcError):
        queue.ntt(x)
    with pytest.raises(_lib.HmpcError):
        queue.modulus(Q_FMA).prepare(8)  # not NTT friendly for N = 8 (Q = 1 mod 8 fails)
    with pytest.raises(_lib.HmpcError):
        queue.centered_binomial(gm, (4,), 65)


@pytest.mark.parametrize("q,n,batch", [(Q_NTT, 4096, 1), (Q_256, 1 << 12, 2), (Q_192, 1 << 13, 1), (P_64, 16, 3)])
def test_plain_transform_matches_tiled_and_oracle(queue, oracle, q, n, batch):
    m = oracle.Modulus(q)
    x = random_residues(oracle, m, n * batch, 21)
    dx = upload(queue, q, x, (batch,), n)
    y = queue.ntt_plain(dx)
    assert np.array_equal(y.numpy(), oracle.ntt(m, n, batch, src=x))
    assert np.array_equal(queue.ntt_plain(y, inverse=True).numpy(), x)
    queue.nonce = [1, 2, 3]
    a = queue.ntt_plain_centered_binomial(queue.modulus(q), n, (batch,), 20)
    queue.nonce = [1, 2, 3]
    b = queue.ntt_centered_binomial(queue.modulus(q), n, (batch,), 20)
    assert np.array_equal(a.numpy(), b.numpy())


@pytest.mark.parametrize("radix_bits,local_bits,col_bits", [(2, 0, 4), (2, 8, 3), (3, 9, 5), (2, 11, 5), (3, 6, 3)])
@pytest.mark.parametrize("q,n,batch", [(Q_256, 1 << 15, 2), (Q_192, 1 << 12, 3), (P_64, 1 << 16, 1),
                                       (Q_NTT, 1 << 13, 2)])
def test_tile_shapes_give_identical_transforms(queue, oracle, q, n, batch, radix_bits, local_bits, col_bits,
                                               cpu_threads):
    m = oracle.Modulus(q)
    gm = queue.modulus(q)
    x = random_residues(oracle, m, n * batch, 33)
    for inverse in (False, True):
        gm.set_plan(n, batch, inverse, radix_bits, local_bits, col_bits)
    ref = oracle.ntt(m, n, batch, src=x, threads=cpu_threads)
    y = queue.ntt(upload(queue, q, x, (batch,), n))
    assert np.array_equal(y.numpy(), ref)
    assert np.array_equal(queue.intt(y).numpy(), x)
    queue.nonce = [9, 9, 9]
    c = queue.ntt_centered_binomial(gm, n, (batch,), 20)
    assert np.array_equal(c.numpy(), oracle.ntt(m, n, batch, sampler="cbd", variance_x2=20, key=KEY,
                                                nonce=[9, 9, 9], threads=cpu_threads))
    for inverse in (False, True):
        gm.set_plan(n, batch, inverse, 3, 0, 4)  # back to the default shape


def test_tuner_keeps_results_identical(queue, oracle):
    m = oracle.Modulus(Q_256)
    gm = queue.modulus(Q_256)
    n, batch = 1 << 12, 8
    x = random_residues(oracle, m, n * batch, 44)
    assert gm.tune(n, batch) > 0
    assert np.array_equal(queue.ntt(upload(queue, Q_256, x, (batch,), n)).numpy(), oracle.ntt(m, n, batch, src=x))
