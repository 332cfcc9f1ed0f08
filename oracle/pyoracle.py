"""Independent big-integer restatement of the same hot path, in pure Python.

TEST INFRASTRUCTURE ONLY.  It shares no code with the C oracle: arithmetic is
done on Python integers (x*R mod Q directly instead of word-by-word REDC), so
agreement between the two pins the C restatement.  Loops are pure Python, so
it is meant for small cases (N <= 2^10, a few polynomials).

References are to hmpc v0.5.2 (paths relative to the hmpc source tree).
"""

M32 = 0xFFFFFFFF


class Mod:
    """mod<Q> (ints/mod.hpp:73-379) on Python integers."""

    def __init__(self, q):
        self.q = int(q)
        self.bits = max(1, (self.q - 1).bit_length())
        self.limbs = (self.bits + 31) // 32
        self.R = 1 << (32 * self.limbs)
        self.Rinv = pow(self.R, -1, self.q)
        self.one = self.R % self.q

    def mont(self, v):
        return (int(v) * self.R) % self.q

    def canon(self, x):
        return (x * self.Rinv) % self.q

    def mul(self, a, b):
        return (a * b * self.Rinv) % self.q

    def add(self, a, b):
        return (a + b) % self.q

    def sub(self, a, b):
        return (a - b) % self.q

    def redc_wide(self, value, r):
        """montgomery_reduce with R' = 2^(32 r) (core/num/modulo.hpp:30-66)"""
        return (value * pow(1 << (32 * r), -1, self.q)) % self.q

    def cast_from(self, src, x):
        """centred lift (mod.hpp:259-307)"""
        v = src.canon(x)
        if v > src.q // 2:
            v -= src.q
        return self.mont(v % self.q)


def rotl(v, c):
    return ((v << c) | (v >> (32 - c))) & M32


def quarter_round(a, b, c, d):
    """crypto/chacha.hpp:13-30"""
    a = (a + b) & M32; d = rotl(d ^ a, 16)
    c = (c + d) & M32; b = rotl(b ^ c, 12)
    a = (a + b) & M32; d = rotl(d ^ a, 8)
    c = (c + d) & M32; b = rotl(b ^ c, 7)
    return a, b, c, d


def chacha20_block(key, counter, nonce):
    """crypto/chacha.hpp:91-166"""
    s = [0x61707865, 0x3320646E, 0x79622D32, 0x6B206574] + list(key) + [counter & M32] + list(nonce)
    x = list(s)
    for _ in range(10):
        for a, b, c, d in ((0, 4, 8, 12), (1, 5, 9, 13), (2, 6, 10, 14), (3, 7, 11, 15),
                           (0, 5, 10, 15), (1, 6, 11, 12), (2, 7, 8, 13), (3, 4, 9, 14)):
            x[a], x[b], x[c], x[d] = quarter_round(x[a], x[b], x[c], x[d])
    return [(x[i] + s[i]) & M32 for i in range(16)]


class Generator:
    """random/number_generator.hpp:42-104"""

    def __init__(self, key, nonce, counter):
        self.key, self.nonce = list(key), list(nonce)
        self.counter = counter & M32
        self.block = chacha20_block(self.key, self.counter, self.nonce)
        self.counter = (self.counter + 1) & M32
        self.index = 0

    def next(self):
        w = self.block[self.index]
        self.index += 1
        if self.index == 16:
            self.block = chacha20_block(self.key, self.counter, self.nonce)
            self.counter = (self.counter + 1) & M32
            self.index = 0
        return w

    def words(self, bits):
        n = (bits + 31) // 32
        ws = [self.next() for _ in range(n)]
        if bits % 32:
            ws[-1] &= (1 << (bits % 32)) - 1
        return sum(w << (32 * i) for i, w in enumerate(ws)), n


def cbd(gen, variance_x2):
    """random/binomial.hpp:29-86,110-122"""
    v, _ = gen.words(2 * variance_x2)
    return bin(v).count("1") - variance_x2


def uniform(m, gen, security=80):
    """random/uniform.hpp:62-66 -> mod.hpp:210-215"""
    v, n = gen.words(m.bits + security)
    return m.redc_wide(v, max(m.limbs, n))


def nonce_add(nonce, v):
    x = sum(int(w) << (32 * i) for i, w in enumerate(nonce)) + v
    return [(x >> (32 * i)) & M32 for i in range(3)]


def root_of_unity(m, degree):
    """ints/num/theory/root_of_unity.hpp:20-54 (Montgomery form)"""
    gen = Generator([0] * 8, [0] * 3, 0)
    e = (m.q - 1) // degree
    assert (m.q - 1) % degree == 0
    while True:
        x, _ = gen.words(m.bits)
        if x > m.q - 1:
            x -= m.q
        if x == 0:
            continue
        # x is used as a raw Montgomery representative
        g = m.mont(pow(m.canon(x), e, m.q))
        gc = m.canon(g)
        if pow(gc, degree // 2, m.q) != 1 and pow(gc, degree, m.q) == 1:
            return g


def bit_reverse(v, bits):
    return int(format(v, f"0{bits}b")[::-1], 2) if bits else 0


def twiddles(m, n, inverse=False):
    """number_theoretic_transform.hpp:35-88 (Montgomery form)"""
    bits = n.bit_length() - 1
    root = m.canon(root_of_unity(m, 2 * n))
    if inverse:
        root = pow(root, -1, m.q)
    ninv = pow(n, -1, m.q)
    t = [0] * n
    t[0] = m.mont(ninv if inverse else 1)
    for i in range(1, n):
        j = bit_reverse(i, bits)
        v = pow(root, i, m.q)
        if inverse and j == 1:
            v = v * ninv % m.q
        t[j] = m.mont(v)
    return t


def ntt(m, n, batch, inputs=None, inverse=False, sampler=None, variance_x2=0, key=(0,) * 8, nonce=(0, 0, 0)):
    """Stage-per-pass transform of `batch` polynomials (element e = i*n + k),
    values as Montgomery representatives; `inputs` is a flat list when no
    sampler is given (number_theoretic_transform.hpp:90-197,262-549)."""
    bits = n.bit_length() - 1
    t = twiddles(m, n, inverse)
    a = list(inputs) if inputs is not None else [0] * (n * batch)
    for s in range(bits):
        length = (n >> (s + 1)) if inverse else (1 << s)
        step = (1 << s) if inverse else (n // length // 2)
        for i in range(batch):
            base = i * n
            for tid in range(n // 2):
                ps = tid // step
                tgt = ps * step * 2 + tid % step
                psi = t[length + ps]
                if s == 0 and sampler is not None:
                    g = Generator(key, nonce, base + tgt)
                    if sampler == "cbd":
                        u = m.mont(cbd(g, variance_x2) % m.q)
                        v = m.mont(cbd(g, variance_x2) % m.q)
                    else:
                        u = uniform(m, g)
                        v = uniform(m, g)
                else:
                    u, v = a[base + tgt], a[base + tgt + step]
                if not inverse:
                    v = m.mul(v, psi)
                    a[base + tgt], a[base + tgt + step] = m.add(u, v), m.sub(u, v)
                elif s < bits - 1:
                    a[base + tgt], a[base + tgt + step] = m.add(u, v), m.mul(m.sub(u, v), psi)
                else:
                    a[base + tgt] = m.mul(m.add(u, v), t[0])
                    a[base + tgt + step] = m.mul(m.sub(u, v), t[1])
    return a


def negacyclic_dft(m, coeffs_canonical, root_canonical):
    """Direct O(N^2) evaluation: output position j holds
    sum_i x_i * psi^((2*bitrev(j)+1)*i) -- the value the in-place transform
    leaves there (independent check of the butterfly network)."""
    n = len(coeffs_canonical)
    bits = n.bit_length() - 1
    out = []
    for j in range(n):
        e = 2 * bit_reverse(j, bits) + 1
        w = pow(root_canonical, e, m.q)
        acc, p = 0, 1
        for x in coeffs_canonical:
            acc = (acc + x * p) % m.q
            p = p * w % m.q
        out.append(acc)
    return out
