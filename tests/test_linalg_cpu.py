"""Matrix-vector products and reductions: the CPU oracle pinned to the
reference's own tests (tests/expr/matrix_vector_product.cpp and
tests/expr/reduce.cpp, extracted into tests/golden/reference_kats.json) and
cross-checked against plain Python integers on random cases."""
import random

import numpy as np
import pytest

Q128 = 0x95D13129B10A9D6E4BFC74319391CCE9  # examples/fma.cpp:15


def centred(v, q):
    return v - q if v > q // 2 else v


def test_monomial_matvec_reference_vector(oracle, kats):
    """The bit-monomial matrix times integer polynomials of
    tests/expr/matrix_vector_product.cpp, computed mod a 128-bit Q: the
    products are small, so the centred residues are the reference's signed
    integers."""
    k = kats["matrix_vector_product"]
    n, batch, rows, cols = k["n"], k["batch"], k["rows"], k["cols"]
    m = oracle.Modulus(Q128)
    flat_x = [v for b in k["x"] for poly in b for v in poly]
    x = oracle.from_uint(m, oracle.planar(flat_x, m.limbs))
    z = oracle.matvec_monomial(m, n, batch, rows, cols, np.array(k["degrees"]), x)
    got = [centred(v, Q128) for v in oracle.unplanar(oracle.to_uint(m, z))]
    expect = [v for b in k["z"] for poly in b for v in poly]
    assert got == expect, k["lines"]


def test_reduce_reference_vector(oracle, kats):
    k = kats["reduce"]
    bits, limbs = k["bits"], (k["bits"] + 31) // 32
    x = oracle.planar(k["x"], limbs)
    y = oracle.planar(k["y"], limbs)
    checks = k["checks"]
    for op in ("add", "multiply", "bit_or", "bit_and", "bit_xor", "min", "max"):
        got = oracle.from_limbs(oracle.reduce_uint(op, bits, x))
        assert got == checks[op]["value"], checks[op]["line"]
    eq = oracle.equal(x, y)[None, :]
    assert bool(oracle.reduce_uint("bit_and", 1, eq)[0]) == checks["all_x_eq_y"]["value"]
    assert bool(oracle.reduce_uint("bit_or", 1, eq)[0]) == checks["any_x_eq_y"]["value"]
    assert bool(oracle.reduce_uint("bit_and", 1, oracle.equal(x, x)[None, :])[0]) == checks["all_x_eq_x"]["value"]


def _random_residues(m, count, rng):
    return [rng.randrange(m.value) for _ in range(count)]


@pytest.mark.parametrize("q", [0xFFFFFFFB, Q128, (1 << 255) - 19])
@pytest.mark.parametrize("m_batch,x_batch", [(3, 3), (1, 3), (3, 1)])
def test_matvec_matches_python_integers(oracle, q, m_batch, x_batch):
    rng = random.Random(q ^ (m_batch << 4) ^ x_batch)
    m = oracle.Modulus(q)
    batch, rows, cols, coeffs = 3, 2, 5, 4
    mv = _random_residues(m, m_batch * rows * cols * coeffs, rng)
    xv = _random_residues(m, x_batch * cols * coeffs, rng)
    mat = oracle.from_uint(m, oracle.planar(mv, m.limbs))
    x = oracle.from_uint(m, oracle.planar(xv, m.limbs))
    z = oracle.unplanar(oracle.to_uint(m, oracle.matvec(m, batch, rows, cols, coeffs, mat, x)))
    for b in range(batch):
        bm, bx = (b if m_batch > 1 else 0), (b if x_batch > 1 else 0)
        for i in range(rows):
            for c in range(coeffs):
                s = sum(mv[((bm * rows + i) * cols + kk) * coeffs + c] * xv[(bx * cols + kk) * coeffs + c]
                        for kk in range(cols)) % q
                assert z[(b * rows + i) * coeffs + c] == s


def _negacyclic_monomial(poly, d):
    """X^d * poly in Z[X]/(X^n + 1) by the definition (X^n = -1)."""
    n = len(poly)
    out = [0] * n
    for j, v in enumerate(poly):
        e = j + d
        sign = -1 if (e // n) % 2 else 1
        out[e % n] += sign * v
    return out


def test_monomial_matvec_matches_definition(oracle):
    rng = random.Random(5)
    m = oracle.Modulus(Q128)
    n, batch, rows, cols = 16, 2, 3, 4
    xv = _random_residues(m, batch * cols * n, rng)
    degrees = np.array([rng.choice([-1, rng.randrange(4 * n)]) for _ in range(batch * rows * cols)])
    x = oracle.from_uint(m, oracle.planar(xv, m.limbs))
    z = oracle.unplanar(oracle.to_uint(m, oracle.matvec_monomial(m, n, batch, rows, cols, degrees, x)))
    for b in range(batch):
        for i in range(rows):
            acc = [0] * n
            for kk in range(cols):
                d = int(degrees[(b * rows + i) * cols + kk])
                if d >= 0:
                    term = _negacyclic_monomial(xv[(b * cols + kk) * n:(b * cols + kk + 1) * n], d)
                    acc = [a + t for a, t in zip(acc, term)]
            assert z[(b * rows + i) * n:(b * rows + i + 1) * n] == [a % Q128 for a in acc]


@pytest.mark.parametrize("q", [0xFFFFFFFB, Q128])
def test_reduce_mod_matches_python_integers(oracle, q):
    rng = random.Random(q)
    m = oracle.Modulus(q)
    values = _random_residues(m, 1000, rng)
    x = oracle.from_uint(m, oracle.planar(values, m.limbs))
    total = oracle.from_limbs(oracle.to_uint(m, oracle.reduce_mod(m, "add", x)[:, None])[:, 0])
    assert total == sum(values) % q
    prod = 1
    for v in values:
        prod = prod * v % q
    got = oracle.from_limbs(oracle.to_uint(m, oracle.reduce_mod(m, "multiply", x)[:, None])[:, 0])
    assert got == prod
    with pytest.raises(ValueError):
        oracle.reduce_mod(m, "bit_or", x)


@pytest.mark.parametrize("bits", [1, 31, 32, 127, 256, 288])
def test_reduce_uint_identities_and_wraparound(oracle, bits):
    rng = random.Random(bits)
    limbs = (bits + 31) // 32
    mask = (1 << bits) - 1
    values = [rng.getrandbits(bits) for _ in range(50)]
    x = oracle.planar(values, limbs)
    expect = {"add": sum(values) & mask, "bit_or": 0, "bit_and": mask, "bit_xor": 0, "min": min(values),
              "max": max(values)}
    prod = 1
    for v in values:
        prod = prod * v & mask
        expect["bit_or"] |= v
        expect["bit_and"] &= v
        expect["bit_xor"] ^= v
    expect["multiply"] = prod
    for op, value in expect.items():
        assert oracle.from_limbs(oracle.reduce_uint(op, bits, x)) == value, op
    empty = np.zeros((limbs, 0), dtype=np.uint32)
    identity = {"add": 0, "multiply": 1, "bit_and": mask, "bit_or": 0, "bit_xor": 0, "min": mask, "max": 0}
    for op, value in identity.items():
        assert oracle.from_limbs(oracle.reduce_uint(op, bits, empty)) == value, op
