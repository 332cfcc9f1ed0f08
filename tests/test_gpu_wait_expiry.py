"""Bounded device waits that run out: the kernel gives up, reports
HMPC_ERROR_TIMEOUT to the host and returns, and the context stays usable.

Each kernel that waits on other threads or on the tensor core bounds every
wait by a poll count.  A test hook shortens that count and makes one wait run
out -- a signal that is withheld (the batched transform) or a barrier nothing
arrives at (the tensor-core transform) -- so no kernel faults, traps or
spins without end.  After the hook is cleared, the same calls give results
bit-exact with the oracle again.
"""
import numpy as np
import pytest

from hmpc_gb300 import _lib
from hmpc_gb300.batch import NttBatch
from hmpc_gb300.comp import Queue, Tensor
from hmpc_gb300.moduli import MODULI

pytestmark = pytest.mark.gpu

KEY = [0x13579BDF, 0x2468ACE0, 0xFDB97531, 0x0ECA8642, 1, 2, 3, 4]
Q_256 = MODULI["q256"]


@pytest.fixture()
def queue():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    q = Queue(key=KEY)
    yield q
    q.close()


def test_batched_transform_wait_runs_out(queue, oracle, cpu_threads):
    qm = queue.modulus(MODULI["q192"])
    om = oracle.Modulus(MODULI["q192"])
    degrees = [1 << 15, 1 << 13, 1 << 15, 1 << 14]  # two passes each at 6 limbs
    xs = [queue.uniform(qm, (), n) for n in degrees]
    refs = [oracle.ntt(om, n, 1, src=x.numpy(), threads=cpu_threads) for n, x in zip(degrees, xs)]
    batch = NttBatch(queue, qm, degrees, autotune=False)
    items = batch.info()["items"]
    ys = batch.run(xs)
    assert batch.status() == 0
    assert all(np.array_equal(y.numpy(), r) for y, r in zip(ys, refs))

    # the last work item (second pass of a polynomial) waits for a signal
    # that never comes, at most 4096 polls
    _lib.call("hmpc_ntt_batch_set_test_wait", batch.handle, 4096, items)
    batch.run(xs, ys)
    with pytest.raises(_lib.HmpcError) as err:
        batch.status()
    assert err.value.code == 6  # HMPC_ERROR_TIMEOUT

    # an item that may not be withheld (the first, a first-pass item) is refused
    with pytest.raises(_lib.HmpcError):
        _lib.call("hmpc_ntt_batch_set_test_wait", batch.handle, 4096, 1)

    # cleared: the same batch runs to completion, bit-exact
    _lib.call("hmpc_ntt_batch_set_test_wait", batch.handle, 0, 0)
    ys = batch.run(xs)
    assert batch.status() == 0
    assert all(np.array_equal(y.numpy(), r) for y, r in zip(ys, refs))
    batch.close()
    # the context is usable for other work
    z = queue.intt(queue.ntt(xs[1]))
    assert (z.data == xs[1].data).all().item()


def test_tensor_core_wait_runs_out(queue, oracle, cpu_threads):
    gm = queue.modulus(Q_256)
    om = oracle.Modulus(Q_256)
    n, batch = 1 << 12, 4
    gm.set_plan(n, batch, False, radix_bits=0)
    x = queue.uniform(gm, (batch,), n)
    ref = oracle.ntt(om, n, batch, src=x.numpy(), threads=cpu_threads)
    y = queue.ntt(x)
    assert _lib.call("hmpc_context_synchronize", queue.handle) == 0
    assert np.array_equal(y.numpy(), ref)

    # the MMA thread of every group launch waits on a barrier nothing
    # arrives at: each launch gives up after 2048 polls and returns
    _lib.call("hmpc_context_set_test_wait", queue.handle, 2048, 1)
    before = queue.launches
    queue.ntt(x, out=y)
    assert queue.launches - before == 4  # four groups launched, each returned early
    with pytest.raises(_lib.HmpcError) as err:
        _lib.call("hmpc_context_synchronize", queue.handle)
    assert err.value.code == 6  # HMPC_ERROR_TIMEOUT
    # the error is reported once
    assert _lib.call("hmpc_context_synchronize", queue.handle) == 0

    # cleared: bit-exact again, and the sampling first group and the inverse too
    _lib.call("hmpc_context_set_test_wait", queue.handle, 0, 0)
    y = queue.ntt(x)
    assert _lib.call("hmpc_context_synchronize", queue.handle) == 0
    assert np.array_equal(y.numpy(), ref)
    gm.set_plan(n, batch, True, radix_bits=0)
    assert np.array_equal(queue.intt(y).numpy(), x.numpy())
    nonce = queue.nonce
    c = queue.ntt_centered_binomial(gm, n, (batch,), 20)
    assert np.array_equal(c.numpy(), oracle.ntt(om, n, batch, sampler="cbd", variance_x2=20, key=KEY, nonce=nonce,
                                                threads=cpu_threads))
