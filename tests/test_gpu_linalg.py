"""Matrix-vector products and reductions on the GPU (through the C ABI)
against the CPU oracle, bit for bit, and against the reference's own vectors
(tests/expr/matrix_vector_product.cpp, tests/expr/reduce.cpp)."""
import random

import numpy as np
import pytest

from hmpc_gb300 import _lib
from hmpc_gb300.comp import Queue, Tensor

pytestmark = pytest.mark.gpu

KEY = [0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344, 0xA4093822, 0x299F31D0, 0x082EFA98, 0xEC4E6C89]

Q_32 = 0xFFFFFFFB  # L=1
P_64 = 0x8822D80623320001  # tests/expr/crypto/lhe/enc.cpp:16, L=2
Q_FMA = 0x95D13129B10A9D6E4BFC74319391CCE9  # examples/fma.cpp:15, L=4
Q_NTT = 0x18F25CD9A75CCBD9C146D4ABAEC00001  # examples/ntt.cpp:22, L=4, q = 1 mod 2^22
Q_192 = 0x8605423C957246B58997DEC24F688AB3DD46CB31C5700001  # L=6
Q_256 = 0xCFF479B9B12CCF05AF55BCA0D7AE005D53E20D920B577D2785F3A1F156740001  # L=8
Q_279 = 0x591F5B834C0D961F67343BCC8902BDEDA2771F54306FF151162FF8D2B40F4194DC0001  # L=9


@pytest.fixture(scope="module")
def queue():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    q = Queue(key=KEY)
    yield q
    q.close()


def residues(q, limbs, count, seed):
    """uniform words below Q (top limb masked under Q's top limb): valid
    Montgomery representatives, no conversion needed"""
    rng = np.random.default_rng(seed)
    words = rng.integers(0, 2**32, size=(limbs, count), dtype=np.uint64).astype(np.uint32)
    top = (q >> (32 * (limbs - 1))) & 0xFFFFFFFF
    words[limbs - 1] %= np.uint32(top)
    return words


def upload(queue, q, arr, shape, n=1):
    return Tensor.from_numpy(queue.modulus(q), arr, shape, n)


def centred(v, q):
    return v - q if v > q // 2 else v


@pytest.mark.parametrize("q", [Q_32, P_64, Q_FMA, Q_192, Q_256, Q_279])
@pytest.mark.parametrize("batch,rows,cols,coeffs,mb,xb", [
    (3, 2, 5, 64, 3, 3),     # NTT-form polynomials of degree 64
    (3, 2, 5, 64, 1, 3),     # one matrix for the whole batch
    (3, 2, 5, 64, 3, 1),     # one vector for the whole batch
    (2, 7, 3, 1000, 2, 2),   # coefficient count not a power of two
    (4, 33, 17, 1, 4, 4),    # plain residues
    (1, 1, 1, 1, 1, 1),
])
def test_matvec_matches_oracle(queue, oracle, q, batch, rows, cols, coeffs, mb, xb):
    om = oracle.Modulus(q)
    seed = (q ^ batch ^ (rows << 8) ^ (cols << 16) ^ (coeffs << 24) ^ (mb << 40) ^ (xb << 44)) & 0xFFFFFFFF
    mat = residues(q, om.limbs, mb * rows * cols * coeffs, seed)
    x = residues(q, om.limbs, xb * cols * coeffs, seed + 1)
    expect = oracle.matvec(om, batch, rows, cols, coeffs, mat, x)
    got = queue.matrix_vector_product(upload(queue, q, mat, (mb, rows, cols), coeffs),
                                      upload(queue, q, x, (xb, cols), coeffs))
    assert got.shape == (batch, rows) and got.n == coeffs
    assert np.array_equal(got.numpy(), expect)


def test_matvec_is_the_ring_product_in_ntt_form(queue, oracle):
    """INTT(sum_k NTT(m_k) * NTT(x_k)) = sum_k m_k * x_k in Z_q[X]/(X^n + 1)"""
    q, n, rows, cols = Q_NTT, 16, 2, 3
    om = oracle.Modulus(q)
    rng = random.Random(3)
    mv = [rng.randrange(q) for _ in range(rows * cols * n)]
    xv = [rng.randrange(q) for _ in range(cols * n)]
    m_t = upload(queue, q, oracle.from_uint(om, oracle.planar(mv, om.limbs)), (rows * cols,), n)
    x_t = upload(queue, q, oracle.from_uint(om, oracle.planar(xv, om.limbs)), (cols,), n)
    m_hat = queue.ntt(m_t)
    x_hat = queue.ntt(x_t)
    z_hat = queue.matrix_vector_product(Tensor(m_hat.modulus, (1, rows, cols), n, m_hat.data),
                                        Tensor(x_hat.modulus, (1, cols), n, x_hat.data))
    z = oracle.unplanar(oracle.to_uint(om, queue.intt(Tensor(z_hat.modulus, (rows,), n, z_hat.data)).numpy()))
    for i in range(rows):
        acc = [0] * n
        for k in range(cols):
            a = mv[(i * cols + k) * n:(i * cols + k + 1) * n]
            b = xv[k * n:(k + 1) * n]
            for s in range(n):
                for t in range(n):
                    e = s + t
                    acc[e % n] += a[s] * b[t] * (-1 if e >= n else 1)
        assert z[i * n:(i + 1) * n] == [v % q for v in acc]


def test_monomial_matvec_reference_vector(queue, oracle, kats):
    import torch

    k = kats["matrix_vector_product"]
    n, batch, rows, cols = k["n"], k["batch"], k["rows"], k["cols"]
    om = oracle.Modulus(Q_FMA)
    flat_x = [v for b in k["x"] for poly in b for v in poly]
    x = upload(queue, Q_FMA, oracle.from_uint(om, oracle.planar(flat_x, om.limbs)), (batch, cols), n)
    degrees = torch.tensor(k["degrees"], dtype=torch.int64, device=queue.device)
    z = queue.monomial_matrix_vector_product(degrees, x)
    got = [centred(v, Q_FMA) for v in oracle.unplanar(oracle.to_uint(om, z.numpy()))]
    assert got == [v for b in k["z"] for poly in b for v in poly], k["lines"]


@pytest.mark.parametrize("q", [Q_32, P_64, Q_256, Q_279])
@pytest.mark.parametrize("n,batch,rows,cols,db,xb", [
    (16, 2, 3, 4, 2, 2),
    (4096, 3, 2, 5, 1, 3),
    (4096, 3, 2, 5, 3, 1),
    (1, 2, 2, 2, 2, 2),
])
def test_monomial_matvec_matches_oracle(queue, oracle, q, n, batch, rows, cols, db, xb):
    import torch

    om = oracle.Modulus(q)
    rng = random.Random(q ^ n ^ db ^ (xb << 3))
    # nullopt, the wrap points 0, n - 1, n, 2n - 1, and degrees past 2n
    choices = [-1, 0, n - 1, n, 2 * n - 1, 2 * n, 5 * n + 3]
    degrees = [rng.choice(choices + [rng.randrange(8 * n)]) for _ in range(db * rows * cols)]
    x = residues(q, om.limbs, xb * cols * n, rng.randrange(2**32))
    expect = oracle.matvec_monomial(om, n, batch, rows, cols, np.array(degrees), x)
    d_t = torch.tensor(degrees, dtype=torch.int64, device=queue.device).reshape(db, rows, cols)
    got = queue.monomial_matrix_vector_product(d_t, upload(queue, q, x, (xb, cols), n))
    assert np.array_equal(got.numpy(), expect)


@pytest.mark.parametrize("q", [Q_32, P_64, Q_FMA, Q_256, Q_279])
@pytest.mark.parametrize("count", [0, 1, 255, 256, 257, 100_003, (1 << 20) + 3])
@pytest.mark.parametrize("op", ["add", "multiply"])
def test_reduce_matches_oracle(queue, oracle, q, count, op):
    om = oracle.Modulus(q)
    x = residues(q, om.limbs, count, (q + count) & 0xFFFFFFFF)
    got = queue.reduce(upload(queue, q, x, (count,)), op).numpy()[:, 0]
    assert np.array_equal(got, oracle.reduce_mod(om, op, x))


def test_sum_of_two_to_the_24_residues(queue, oracle):
    """the FMA configuration's size: 2^24 residues of the 128-bit modulus"""
    count = 1 << 24
    om = oracle.Modulus(Q_FMA)
    x = residues(Q_FMA, om.limbs, count, 24)
    t = upload(queue, Q_FMA, x, (count,))
    assert np.array_equal(queue.sum(t).numpy()[:, 0], oracle.reduce_mod(om, "add", x))
    assert np.array_equal(queue.product(t).numpy()[:, 0], oracle.reduce_mod(om, "multiply", x))


@pytest.mark.parametrize("bits", [1, 31, 32, 64, 127, 256, 288])
@pytest.mark.parametrize("count", [0, 1, 1000, 300_001])
def test_reduce_uint_matches_oracle(queue, oracle, bits, count):
    import torch

    limbs = (bits + 31) // 32
    rng = np.random.default_rng(bits * 7 + count)
    words = rng.integers(0, 2**32, size=(limbs, count), dtype=np.uint64).astype(np.uint32)
    if count > 2:
        words[:, 1] = 0           # a zero for and / min
        words[:, 2] = 0xFFFFFFFF  # all ones (above `bits` too: masked) for or / max
    data = torch.from_numpy(words.view(np.int32)).to(queue.device).contiguous()
    for op in _lib.REDUCE_OPS:
        got = queue.reduce_uint(data, bits, op).cpu().numpy().view(np.uint32)
        assert np.array_equal(got, oracle.reduce_uint(op, bits, words)), op


def test_reduce_reference_vector(queue, oracle, kats):
    import torch

    k = kats["reduce"]
    bits, limbs = k["bits"], (k["bits"] + 31) // 32
    x = torch.from_numpy(oracle.planar(k["x"], limbs).view(np.int32)).to(queue.device).contiguous()
    y = torch.from_numpy(oracle.planar(k["y"], limbs).view(np.int32)).to(queue.device).contiguous()
    for op in ("add", "multiply", "bit_or", "bit_and", "bit_xor", "min", "max"):
        got = oracle.from_limbs(queue.reduce_uint(x, bits, op).cpu().numpy().view(np.uint32))
        assert got == k["checks"][op]["value"], k["checks"][op]["line"]
    eq = queue.equal(x, y)
    assert queue.all(eq) == k["checks"]["all_x_eq_y"]["value"]
    assert queue.any(eq) == k["checks"]["any_x_eq_y"]["value"]
    assert queue.all(queue.equal(x, x)) == k["checks"]["all_x_eq_x"]["value"]


@pytest.mark.parametrize("limbs", [1, 4, 9])
def test_equal_matches_oracle(queue, oracle, limbs):
    import torch

    rng = np.random.default_rng(limbs)
    a = rng.integers(0, 4, size=(limbs, 5000), dtype=np.uint64).astype(np.uint32)
    b = rng.integers(0, 4, size=(limbs, 5000), dtype=np.uint64).astype(np.uint32)
    b[:, ::3] = a[:, ::3]
    to = lambda w: torch.from_numpy(w.view(np.int32)).to(queue.device).contiguous()  # noqa: E731
    got = queue.equal(to(a), to(b)).cpu().numpy().view(np.uint32)
    assert np.array_equal(got, oracle.equal(a, b))


def test_argument_errors_leave_the_context_usable(queue, oracle):
    import torch

    m = upload(queue, Q_FMA, residues(Q_FMA, 4, 2 * 3 * 4, 1), (2, 3), 4)
    x = upload(queue, Q_FMA, residues(Q_FMA, 4, 3 * 3 * 4, 2), (3, 3), 4)
    # matrix batch 2 against vector batch 3: neither broadcasts
    with pytest.raises(_lib.HmpcError) as e:
        queue.matrix_vector_product(Tensor(m.modulus, (2, 1, 3), 4, m.data), x)
    assert e.value.code == 1
    d = torch.zeros((1, 1, 3), dtype=torch.int64, device=queue.device)
    with pytest.raises(_lib.HmpcError) as e:
        _lib.call("hmpc_matvec_monomial", queue.handle, x.modulus.handle, 12, 3, 1, 3, d.data_ptr(), 1,
                  x.ptr(), 3, x.ptr())
    assert e.value.code == 1  # degree 12 is not a power of two
    data = torch.zeros((1, 4), dtype=torch.int32, device=queue.device)
    with pytest.raises(_lib.HmpcError) as e:
        _lib.call("hmpc_reduce_uint", queue.handle, 0, 289, 4, data.data_ptr(), data.data_ptr())
    assert e.value.code == 2
    with pytest.raises(_lib.HmpcError) as e:
        queue.reduce(x, "bit_or")
    assert e.value.code == 1
    # still usable
    om = oracle.Modulus(Q_FMA)
    assert np.array_equal(queue.sum(x).numpy()[:, 0], oracle.reduce_mod(om, "add", x.numpy()))
