"""Batched transforms of uneven degree against the oracle, per polynomial:
one persistent CUDA-core launch from a CUDA graph (default or autotuned tile
shape), or the tensor-core engine (one transform per degree over the
polynomials' own buffers, from one graph)."""
import numpy as np
import pytest

from hmpc_gb300.batch import NttBatch, uneven_degrees
from hmpc_gb300.comp import Queue, Tensor

pytestmark = pytest.mark.gpu

Q_192 = 0x8605423C957246B58997DEC24F688AB3DD46CB31C5700001
Q_256 = 0xCFF479B9B12CCF05AF55BCA0D7AE005D53E20D920B577D2785F3A1F156740001
P_64 = 0x8822D80623320001


@pytest.fixture(scope="module")
def queue():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    q = Queue(key=[5] * 8)
    yield q
    q.close()


@pytest.mark.parametrize("q", [Q_192, Q_256, P_64])
@pytest.mark.parametrize("mode", ["default", "autotune", "tensor"])
def test_uneven_batch_matches_oracle(queue, oracle, q, mode, cpu_threads):
    degrees = [1 << 12, 1 << 3, 1 << 16, 1 << 9, 1 << 13, 1 << 12, 1 << 15, 1 << 5, 1 << 14, 1 << 11]
    if mode == "tensor":
        degrees = [n if n >= 16 else 16 for n in degrees]  # the tensor-core engine takes degrees >= 16
    gm = queue.modulus(q)
    om = oracle.Modulus(q)
    xs = [queue.uniform(gm, (), n) for n in degrees]
    autotune = mode == "autotune"
    fwd = NttBatch(queue, gm, degrees, autotune=autotune, tensor_cores=mode == "tensor")
    if mode == "tensor":
        assert fwd.info()["engine"] == "tensor"
    ys = fwd.run(xs)
    assert fwd.status() == 0
    for x, y, n in zip(xs, ys, degrees):
        assert np.array_equal(y.numpy(), oracle.ntt(om, n, 1, src=x.numpy(), threads=cpu_threads)), n
    inv = NttBatch(queue, gm, degrees, inverse=True, autotune=autotune, tensor_cores=mode == "tensor")
    zs = inv.run(ys)
    assert inv.status() == 0
    for x, z in zip(xs, zs):
        assert np.array_equal(z.numpy(), x.numpy())
    # in place, and a second run with other buffers rebinds the pointers
    copies = [Tensor(gm, (), n, x.data.clone()) for x, n in zip(xs, degrees)]
    fwd.run(copies, copies)
    for c, y in zip(copies, ys):
        assert (c.data == y.data).all().item()
    fwd.close()
    inv.close()


def test_config_sized_batch_round_trip(queue, oracle, cpu_threads):
    """512 polynomials with degrees from {2^12..2^16} drawn from a seeded
    ChaCha20 stream, q 192-bit: forward then inverse is the identity, and a
    sample of polynomials matches the oracle."""
    degrees = uneven_degrees(512)
    gm = queue.modulus(Q_192)
    om = oracle.Modulus(Q_192)
    xs = [queue.uniform(gm, (), n) for n in degrees]
    fwd = NttBatch(queue, gm, degrees, autotune=True)
    inv = NttBatch(queue, gm, degrees, inverse=True, autotune=False)
    ys = fwd.run(xs)
    zs = inv.run(ys)
    assert fwd.status() == 0 and inv.status() == 0
    assert all((x.data == z.data).all().item() for x, z in zip(xs, zs))
    for i in (0, 1, 255, 511):
        assert np.array_equal(ys[i].numpy(), oracle.ntt(om, degrees[i], 1, src=xs[i].numpy(), threads=cpu_threads))
    info = fwd.info()
    assert info["radix"] in (1, 4, 8) and info["items"] > 0


def test_config_sized_batch_on_the_tensor_cores(queue, oracle, cpu_threads):
    """the batched configuration on the tensor-core engine: 512 polynomials
    of degrees 2^12..2^16, q 192-bit (6 limbs), forward bit-exact with the
    oracle on a sample and forward then inverse the identity; the degrees'
    transforms come from one graph launch"""
    degrees = uneven_degrees(512)
    gm = queue.modulus(Q_192)
    om = oracle.Modulus(Q_192)
    xs = [queue.uniform(gm, (), n) for n in degrees]
    fwd = NttBatch(queue, gm, degrees, tensor_cores=True)
    inv = NttBatch(queue, gm, degrees, inverse=True, tensor_cores=True)
    info = fwd.info()
    assert info["engine"] == "tensor"
    before = queue.launches
    ys = fwd.run(xs)
    assert queue.launches - before == info["items"]
    zs = inv.run(ys)
    assert fwd.status() == 0 and inv.status() == 0
    assert all((x.data == z.data).all().item() for x, z in zip(xs, zs))
    sample = [0, 1, 2, 3, 200, 255, 256, 510, 511]
    for i in sample:
        assert np.array_equal(ys[i].numpy(), oracle.ntt(om, degrees[i], 1, src=xs[i].numpy(), threads=cpu_threads))
    fwd.close()
    inv.close()


def test_tensor_core_batch_refuses_what_it_does_not_cover(queue):
    from hmpc_gb300 import _lib

    with pytest.raises(_lib.HmpcError):
        NttBatch(queue, queue.modulus(Q_192), [1 << 10, 8], tensor_cores=True)  # a degree below 16
    q9 = queue.modulus((1 << 287) + 0x5E0001)  # an odd 288-bit (9-limb) modulus
    with pytest.raises(_lib.HmpcError):
        NttBatch(queue, q9, [1 << 10], tensor_cores=True)
