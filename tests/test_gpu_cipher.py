"""ChaCha20 stream cipher over tensors on the GPU against the oracle, the RFC
8439 vector of the reference's tests, and the reference's round trip
(tests/expr/crypto/cipher.cpp)."""
import numpy as np
import pytest
import torch

from hmpc_gb300.comp import Queue, Tensor

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def queue():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    q = Queue(key=[0] * 8)
    yield q
    q.close()


def test_rfc8439_vector(queue, oracle, kats):
    c = kats["cipher"]
    byts = list(c["plaintext"]) + [0] * (-len(c["plaintext"]) % 4)
    msg = [byts[i] | byts[i + 1] << 8 | byts[i + 2] << 16 | byts[i + 3] << 24 for i in range(0, len(byts), 4)]
    mod = queue.modulus((1 << 31) + 11)  # any 1-limb modulus: the cipher only sees words
    x = Tensor.from_numpy(mod, np.array([[0] * 16 + msg], dtype=np.uint32), (16 + len(msg),))
    out = queue.cipher_enc(c["key"], c["nonce"], x).cpu().numpy().view(np.uint32)
    got = b"".join(int(w).to_bytes(4, "little") for w in out[16:])[: len(c["ciphertext"])]
    assert list(got) == c["ciphertext"]


@pytest.mark.parametrize("q,count", [((1 << 127) - 1, 4 * 2), (0xCFF479B9B12CCF05AF55BCA0D7AE005D53E20D920B577D2785F3A1F156740001, 1000),
                                     (0x8822D80623320001, 4097), (0x2FAEADBE7A0195C011AC195AD10269830E8001, 333)])
def test_matches_oracle_and_round_trips(queue, oracle, q, count):
    mod = queue.modulus(q)
    key, nonce = [42] + [0] * 7, [1, 0, 0]
    rng = np.random.default_rng(count)
    planar = rng.integers(0, 2**32, size=(mod.limbs, count), dtype=np.uint64).astype(np.uint32)
    x = Tensor.from_numpy(mod, planar, (count,))
    y = queue.cipher_enc(key, nonce, x)
    assert np.array_equal(y.cpu().numpy().view(np.uint32), oracle.cipher_enc(key, nonce, planar))
    back = queue.cipher_dec(key, nonce, y, mod, (count,))
    assert np.array_equal(back.numpy(), planar)
