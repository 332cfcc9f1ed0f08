"""Named single workloads for profiling and quick timing on one GPU:

  python -m hmpc_gb300.workloads ntt-cbd --n 32768 --batch 160 --vx2 20 --reps 2
  python -m hmpc_gb300.workloads ntt --n 4096 --batch 1 --q ntt
  python -m hmpc_gb300.workloads fma --elements 16777216
  python -m hmpc_gb300.workloads bgv --batch 256
  python -m hmpc_gb300.workloads matvec --n 32768 --batch 16 --rows 4 --cols 4
  python -m hmpc_gb300.workloads sum --elements 16777216

Each runs the operation `--reps` times on cuda:0 and prints the mean time of
the repetitions after the first (CUDA events on the queue's stream).
"""
import argparse
import json

import torch

from . import lhe
from .comp import Queue, Tensor

MODULI = {
    "ntt": 0x18F25CD9A75CCBD9C146D4ABAEC00001,  # examples/ntt.cpp, 125-bit (4 limbs)
    "fma": 0x95D13129B10A9D6E4BFC74319391CCE9,  # examples/fma.cpp, 128-bit (4 limbs)
    "q128": 0xE78EC7A9E37BEFBFF59DF3057EBC0001,
    "q160": 0x92155E09E949EDD961C374C93DE4B90B9F220001,
    "q192": 0x8605423C957246B58997DEC24F688AB3DD46CB31C5700001,
    "q224": 0xE9E9C9C7700173EE913AE1871AE48451A42CE7E731BC0F8A00C20001,
    "q256": 0xCFF479B9B12CCF05AF55BCA0D7AE005D53E20D920B577D2785F3A1F156740001,
    "p64": 0x8822D80623320001,  # tests/expr/crypto/lhe/enc.cpp
}
KEY = [0x6A09E667, 0xBB67AE85, 0x3C6EF372, 0xA54FF53A, 0x510E527F, 0x9B05688C, 0x1F83D9AB, 0x5BE0CD19]


def chacha20_words(key, count, nonce=(0, 0, 0)):
    """`count` words of the ChaCha20 stream (RFC 8439 block function, counter
    from 0) on the host: seeds the workload shapes."""
    def rotl(v, c):
        return ((v << c) | (v >> (32 - c))) & 0xFFFFFFFF

    out = []
    counter = 0
    while len(out) < count:
        s = [0x61707865, 0x3320646E, 0x79622D32, 0x6B206574] + list(key) + [counter] + list(nonce)
        x = list(s)
        for _ in range(10):
            for a, b, c, d in ((0, 4, 8, 12), (1, 5, 9, 13), (2, 6, 10, 14), (3, 7, 11, 15),
                               (0, 5, 10, 15), (1, 6, 11, 12), (2, 7, 8, 13), (3, 4, 9, 14)):
                x[a] = (x[a] + x[b]) & 0xFFFFFFFF; x[d] = rotl(x[d] ^ x[a], 16)
                x[c] = (x[c] + x[d]) & 0xFFFFFFFF; x[b] = rotl(x[b] ^ x[c], 12)
                x[a] = (x[a] + x[b]) & 0xFFFFFFFF; x[d] = rotl(x[d] ^ x[a], 8)
                x[c] = (x[c] + x[d]) & 0xFFFFFFFF; x[b] = rotl(x[b] ^ x[c], 7)
        out.extend((x[i] + s[i]) & 0xFFFFFFFF for i in range(16))
        counter += 1
    return out[:count]


def timed(queue, fn, reps):
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    fn()
    queue.wait()
    start.record(queue.stream)
    for _ in range(max(0, reps - 1)):
        fn()
    stop.record(queue.stream)
    queue.wait()
    return start.elapsed_time(stop) / max(1, reps - 1)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("workload", choices=["ntt", "intt", "ntt-cbd", "ntt-uniform", "fma", "bgv", "plain-ntt", "matvec",
                                         "sum", "ntt-intt"])
    ap.add_argument("--rows", type=int, default=4)
    ap.add_argument("--cols", type=int, default=4)
    ap.add_argument("--n", type=int, default=1 << 15)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--q", default="q256")
    ap.add_argument("--vx2", type=int, default=20)
    ap.add_argument("--elements", type=int, default=1 << 24)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--tune", action="store_true", help="autotune the tile shape first")
    ap.add_argument("--radix-bits", type=int, default=None,
                    help="force a tile shape (with --local-bits, --col-bits); 0 = tensor-core engine")
    ap.add_argument("--local-bits", type=int, default=0)
    ap.add_argument("--col-bits", type=int, default=4)
    args = ap.parse_args(argv)
    queue = Queue(key=KEY)
    q = queue.modulus(MODULI[args.q])
    result = {"workload": args.workload, "q_limbs": q.limbs}
    if args.workload == "ntt-intt":
        # examples/ntt.cpp: one forward then one inverse transform
        q.prepare(args.n)
        if args.tune:
            q.tune(args.n, args.batch)
            q.tune(args.n, args.batch, inverse=True)
        elif args.radix_bits is not None:
            for inverse in (False, True):
                q.set_plan(args.n, args.batch, inverse, args.radix_bits, args.local_bits, args.col_bits)
        x = queue.uniform(q, (args.batch,), args.n)
        y, z = Tensor(q, (args.batch,), args.n), Tensor(q, (args.batch,), args.n)
        ms = timed(queue, lambda: (queue.ntt(x, out=y), queue.intt(y, out=z)), args.reps)
        result.update(n=args.n, batch=args.batch, ms=ms, tile=q.plan(args.n, args.batch),
                      tile_inverse=q.plan(args.n, args.batch, inverse=True))
    elif args.workload == "matvec":
        # batch x (rows x cols) matrices of NTT-form polynomials times cols-vectors
        m = queue.uniform(q, (args.batch, args.rows, args.cols), args.n)
        x = queue.uniform(q, (args.batch, args.cols), args.n)
        z = Tensor(q, (args.batch, args.rows), args.n)
        ms = timed(queue, lambda: queue.matrix_vector_product(m, x, out=z), args.reps)
        result.update(n=args.n, batch=args.batch, rows=args.rows, cols=args.cols, ms=ms)
    elif args.workload == "sum":
        q = queue.modulus(MODULI["fma"])
        result["q_limbs"] = q.limbs
        x = queue.uniform(q, (args.elements,))
        ms = timed(queue, lambda: queue.sum(x), args.reps)
        result.update(elements=args.elements, ms=ms, gbs=args.elements * 4 * q.limbs / (ms * 1e-3) / 1e9)
    elif args.workload in ("ntt", "intt", "ntt-cbd", "ntt-uniform", "plain-ntt"):
        q.prepare(args.n)
        if args.tune:
            result["tuned_ms"] = q.tune(args.n, args.batch, inverse=args.workload == "intt")
        elif args.radix_bits is not None:
            q.set_plan(args.n, args.batch, args.workload == "intt", args.radix_bits, args.local_bits, args.col_bits)
        result["tile"] = q.plan(args.n, args.batch, inverse=args.workload == "intt")
        x = queue.uniform(q, (args.batch,), args.n)
        out = Tensor(q, (args.batch,), args.n)
        if args.workload == "ntt":
            fn = lambda: queue.ntt(x, out=out)  # noqa: E731
        elif args.workload == "intt":
            fn = lambda: queue.intt(x, out=out)  # noqa: E731
        elif args.workload == "ntt-cbd":
            fn = lambda: queue.ntt_centered_binomial(q, args.n, (args.batch,), args.vx2, out=out)  # noqa: E731
        elif args.workload == "ntt-uniform":
            fn = lambda: queue.ntt_uniform(q, args.n, (args.batch,), out=out)  # noqa: E731
        else:
            fn = lambda: queue.ntt_plain(x, out=out)  # noqa: E731
        result.update(n=args.n, batch=args.batch, ms=timed(queue, fn, args.reps))
    elif args.workload == "fma":
        q = queue.modulus(MODULI["fma"])
        a, b, c = (queue.uniform(q, (args.elements,)) for _ in range(3))
        d = Tensor(q, (args.elements,))
        ms = timed(queue, lambda: queue.fma(a, b, c, out=d), args.reps)
        result.update(elements=args.elements, ms=ms, gbs=args.elements * 16 * q.limbs / (ms * 1e-3) / 1e9)
    elif args.workload == "bgv":
        p = queue.modulus(MODULI["p64"])
        q.prepare(args.n)
        p.prepare(args.n)
        if args.tune:
            result["tuned_ms"] = q.tune(args.n, args.batch)
            p.tune(args.n, args.batch, inverse=True)
        elif args.radix_bits is not None:
            q.set_plan(args.n, args.batch, False, args.radix_bits, args.local_bits, args.col_bits)
        result["tile"] = q.plan(args.n, args.batch)
        s, key = lhe.keygen(queue, q, p, args.n)
        msgs = queue.uniform(p, (args.batch,), args.n)
        ct = lhe.Ciphertext(Tensor(q, (args.batch,), args.n), Tensor(q, (args.batch,), args.n))
        ms = timed(queue, lambda: lhe.enc(queue, key, msgs, q, out=ct), args.reps)
        result.update(n=args.n, batch=args.batch, ms=ms, enc_per_s=args.batch / (ms * 1e-3))
    print(json.dumps(result))
    queue.close()


if __name__ == "__main__":
    main()
