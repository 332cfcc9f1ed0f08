/*
 * hmpc_oracle.c -- CPU restatement of hmpc's data-parallel hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path and the timed CPU
 * baseline.  Nothing in the product links or calls this file.
 *
 * Each routine restates the reference algorithm it cites (hmpc v0.5.2, paths
 * relative to the hmpc source tree).  Loops that the reference runs as one
 * SYCL parallel_for per stage run here as one OpenMP parallel loop per stage
 * over the same index space.
 */
#include "hmpc_oracle.h"

#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_T_LIMBS (3 * ORC_MAX_LIMBS + 2)

/* ---------------------------------------------------------------- limbs -- */

static int big_cmp(const uint32_t* a, const uint32_t* b, int n)
{
    for (int i = n - 1; i >= 0; --i)
    {
        if (a[i] != b[i])
        {
            return a[i] > b[i] ? 1 : -1;
        }
    }
    return 0;
}

/* a -= b over n limbs, returns the borrow (core/subtract.hpp:61) */
static uint32_t big_sub(uint32_t* out, const uint32_t* a, const uint32_t* b, int n)
{
    uint32_t borrow = 0;
    for (int i = 0; i < n; ++i)
    {
        uint64_t d = (uint64_t)a[i] - b[i] - borrow;
        out[i] = (uint32_t)d;
        borrow = (uint32_t)(d >> 63);
    }
    return borrow;
}

/* out = a + b over n limbs, returns the carry (core/add.hpp:70,120) */
static uint32_t big_add(uint32_t* out, const uint32_t* a, const uint32_t* b, int n)
{
    uint64_t carry = 0;
    for (int i = 0; i < n; ++i)
    {
        uint64_t s = (uint64_t)a[i] + b[i] + carry;
        out[i] = (uint32_t)s;
        carry = s >> 32;
    }
    return (uint32_t)carry;
}

static int bit_width_words(const uint32_t* a, int n)
{
    for (int i = n - 1; i >= 0; --i)
    {
        if (a[i])
        {
            return 32 * i + (32 - __builtin_clz(a[i]));
        }
    }
    return 0;
}

/* schoolbook product, row by row with one carry per row
 * (core/num/multiply.hpp:19-101); out has na+nb limbs */
static void big_mul(uint32_t* out, const uint32_t* a, int na, const uint32_t* b, int nb)
{
    memset(out, 0, sizeof(uint32_t) * (size_t)(na + nb));
    for (int i = 0; i < nb; ++i)
    {
        uint64_t carry = 0;
        for (int j = 0; j < na; ++j)
        {
            uint64_t t = (uint64_t)a[j] * b[i] + out[i + j] + carry;
            out[i + j] = (uint32_t)t;
            carry = t >> 32;
        }
        out[i + na] = (uint32_t)carry;
    }
}

/* remainder of a (na limbs) modulo q (nq limbs) by shift-and-subtract; used
 * only for the precomputed constants, where the reference evaluates `%` at
 * compile time (ints/mod.hpp:114-117). */
static void big_mod(uint32_t* out, const uint32_t* a, int na, const uint32_t* q, int nq)
{
    uint32_t r[ORC_MAX_LIMBS + 1];
    uint32_t qq[ORC_MAX_LIMBS + 1];
    memset(r, 0, sizeof r);
    memset(qq, 0, sizeof qq);
    memcpy(qq, q, sizeof(uint32_t) * (size_t)nq);
    for (int bit = 32 * na - 1; bit >= 0; --bit)
    {
        /* r = 2r + bit */
        uint32_t top = 0;
        for (int i = 0; i <= nq; ++i)
        {
            uint32_t next = r[i] >> 31;
            r[i] = (r[i] << 1) | top;
            top = next;
        }
        r[0] |= (a[bit / 32] >> (bit % 32)) & 1u;
        if (big_cmp(r, qq, nq + 1) >= 0)
        {
            big_sub(r, r, qq, nq + 1);
        }
    }
    memcpy(out, r, sizeof(uint32_t) * (size_t)nq);
}

int orc_modulus_init(orc_modulus* m, const uint32_t* q, int q_limbs)
{
    memset(m, 0, sizeof *m);
    int width = bit_width_words(q, q_limbs);
    if (width == 0 || (q[0] & 1u) == 0)
    {
        return 1;
    }
    uint32_t qm1[ORC_MAX_LIMBS] = {0};
    uint32_t one_word[ORC_MAX_LIMBS] = {1};
    memcpy(qm1, q, sizeof(uint32_t) * (size_t)q_limbs);
    big_sub(qm1, qm1, one_word, q_limbs);
    m->bits = bit_width_words(qm1, q_limbs); /* mod.hpp:90 */
    if (m->bits == 0)
    {
        m->bits = 1;
    }
    m->limbs = (m->bits + 31) / 32; /* mod.hpp:93 */
    if (m->limbs > ORC_MAX_LIMBS)
    {
        return 2;
    }
    memcpy(m->q, q, sizeof(uint32_t) * (size_t)m->limbs);
    int L = m->limbs;
    for (int i = 0; i < L; ++i)
    {
        m->half[i] = (m->q[i] >> 1) | (i + 1 < L ? (m->q[i + 1] << 31) : 0u);
    }
    /* -Q^{-1} mod 2^32 by Newton iteration (mod.hpp:98-103) */
    uint32_t inv = 1;
    for (int i = 0; i < 6; ++i)
    {
        inv *= 2u - q[0] * inv;
    }
    m->ninv = (uint32_t)(0u - inv);
    /* R mod Q and R^2 mod Q (mod.hpp:105-117) */
    uint32_t R[2 * ORC_MAX_LIMBS + 1];
    memset(R, 0, sizeof R);
    R[L] = 1;
    big_mod(m->one, R, L + 1, m->q, L);
    memset(R, 0, sizeof R);
    R[2 * L] = 1;
    big_mod(m->r2, R, 2 * L + 1, m->q, L);
    return 0;
}

/* core/num/modulo.hpp:30-66: T holds r+p+1 limbs; for each of the r low
 * words add m*Q*B^i with m = T_i*N' and ripple the carry to the top; the
 * result is the upper part minus Q when it is >= Q. */
void orc_redc(const orc_modulus* m, uint32_t* out, const uint32_t* value, int value_limbs, int r)
{
    int p = m->limbs;
    int tl = r + p + 1;
    uint32_t T[ORC_T_LIMBS];
    memset(T, 0, sizeof(uint32_t) * (size_t)tl);
    memcpy(T, value, sizeof(uint32_t) * (size_t)(value_limbs < tl ? value_limbs : tl));
    for (int i = 0; i < r; ++i)
    {
        uint32_t mm = T[i] * m->ninv;
        uint64_t carry = 0;
        for (int j = 0; j < p; ++j)
        {
            uint64_t t = (uint64_t)mm * m->q[j] + T[i + j] + carry;
            T[i + j] = (uint32_t)t;
            carry = t >> 32;
        }
        for (int k = i + p; k < tl && carry; ++k)
        {
            uint64_t t = (uint64_t)T[k] + carry;
            T[k] = (uint32_t)t;
            carry = t >> 32;
        }
    }
    uint32_t* S = T + r; /* p + 1 limbs */
    uint32_t qx[ORC_MAX_LIMBS + 1];
    memcpy(qx, m->q, sizeof(uint32_t) * (size_t)p);
    qx[p] = 0;
    if (big_cmp(S, qx, p + 1) >= 0)
    {
        big_sub(S, S, qx, p + 1);
    }
    memcpy(out, S, sizeof(uint32_t) * (size_t)p);
}

/* mod.hpp:41-46 */
void orc_mul(const orc_modulus* m, uint32_t* out, const uint32_t* a, const uint32_t* b)
{
    uint32_t prod[2 * ORC_MAX_LIMBS];
    big_mul(prod, a, m->limbs, b, m->limbs);
    orc_redc(m, out, prod, 2 * m->limbs, m->limbs);
}

/* mod.hpp:17-34: (bit_size+1)-bit sum, subtract Q, keep the sum on underflow */
void orc_add(const orc_modulus* m, uint32_t* out, const uint32_t* a, const uint32_t* b)
{
    int L = m->limbs;
    uint32_t sum[ORC_MAX_LIMBS + 1];
    uint32_t diff[ORC_MAX_LIMBS + 1];
    uint32_t qx[ORC_MAX_LIMBS + 1];
    sum[L] = big_add(sum, a, b, L);
    memcpy(qx, m->q, sizeof(uint32_t) * (size_t)L);
    qx[L] = 0;
    uint32_t underflow = big_sub(diff, sum, qx, L + 1);
    memcpy(out, underflow ? sum : diff, sizeof(uint32_t) * (size_t)L);
}

/* mod.hpp:35-40: difference, then add Q masked by the borrow */
void orc_sub(const orc_modulus* m, uint32_t* out, const uint32_t* a, const uint32_t* b)
{
    int L = m->limbs;
    uint32_t diff[ORC_MAX_LIMBS];
    uint32_t masked[ORC_MAX_LIMBS];
    uint32_t underflow = big_sub(diff, a, b, L);
    for (int i = 0; i < L; ++i)
    {
        masked[i] = underflow ? m->q[i] : 0u;
    }
    big_add(out, diff, masked, L);
}

/* mod.hpp:327-341 */
void orc_neg(const orc_modulus* m, uint32_t* out, const uint32_t* a)
{
    int L = m->limbs;
    int nonzero = 0;
    for (int i = 0; i < L; ++i)
    {
        nonzero |= a[i] != 0;
    }
    uint32_t masked[ORC_MAX_LIMBS];
    for (int i = 0; i < L; ++i)
    {
        masked[i] = nonzero ? m->q[i] : 0u;
    }
    big_sub(out, masked, a, L);
}

/* mod.hpp:165-189: values of at most 32*L bits are multiplied by R^2 and
 * reduced once; wider values are reduced with R' = 2^(32*value_limbs) first
 * and then multiplied by (R' * R^2 mod Q) and reduced again. */
void orc_from_uint(const orc_modulus* m, uint32_t* out, const uint32_t* value, int value_limbs)
{
    int L = m->limbs;
    int width = bit_width_words(value, value_limbs);
    if (width <= 32 * L)
    {
        uint32_t v[ORC_MAX_LIMBS] = {0};
        memcpy(v, value, sizeof(uint32_t) * (size_t)(value_limbs < L ? value_limbs : L));
        uint32_t prod[2 * ORC_MAX_LIMBS];
        big_mul(prod, v, L, m->r2, L);
        orc_redc(m, out, prod, 2 * L, L);
        return;
    }
    uint32_t y[ORC_MAX_LIMBS];
    orc_redc(m, y, value, value_limbs, value_limbs);
    /* c = R' * R^2 mod Q */
    uint32_t wide[3 * ORC_MAX_LIMBS + 1];
    memset(wide, 0, sizeof wide);
    memcpy(wide + value_limbs, m->r2, sizeof(uint32_t) * (size_t)L);
    uint32_t c[ORC_MAX_LIMBS];
    big_mod(c, wide, value_limbs + L, m->q, L);
    uint32_t prod[2 * ORC_MAX_LIMBS];
    big_mul(prod, y, L, c, L);
    orc_redc(m, out, prod, 2 * L, L);
}

/* mod.hpp:356-361 */
void orc_to_uint(const orc_modulus* m, uint32_t* out, const uint32_t* x)
{
    orc_redc(m, out, x, m->limbs, m->limbs);
}

/* mod.hpp:219-226 (small signed: Q + v when v < 0, then as unsigned) */
void orc_from_int64(const orc_modulus* m, uint32_t* out, int64_t v)
{
    int L = m->limbs;
    uint32_t mag[ORC_MAX_LIMBS + 2] = {0};
    uint64_t a = v < 0 ? (uint64_t)(-(v + 1)) + 1u : (uint64_t)v;
    mag[0] = (uint32_t)a;
    mag[1] = (uint32_t)(a >> 32);
    int n = L > 2 ? L : 2;
    uint32_t r[ORC_MAX_LIMBS + 2];
    big_mod(r, mag, n, m->q, L);
    if (v < 0)
    {
        int zero = 1;
        for (int i = 0; i < L; ++i)
        {
            zero &= r[i] == 0;
        }
        if (!zero)
        {
            big_sub(r, m->q, r, L);
        }
    }
    orc_from_uint(m, out, r, L);
}

/* mod.hpp:259-307: integer value of x mod src; when it exceeds src/2 shift it
 * by (dst - src) (dst > src) or by the offset to the next multiple of dst
 * (dst < src); then convert as an unsigned integer. */
void orc_cast(const orc_modulus* dst, const orc_modulus* src, uint32_t* out, const uint32_t* x)
{
    int Ls = src->limbs;
    int Ld = dst->limbs;
    int n = (Ls > Ld ? Ls : Ld) + 1;
    uint32_t integer[ORC_MAX_LIMBS + 1] = {0};
    orc_to_uint(src, integer, x);
    uint32_t sq[ORC_MAX_LIMBS + 1] = {0};
    uint32_t dq[ORC_MAX_LIMBS + 1] = {0};
    uint32_t sh[ORC_MAX_LIMBS + 1] = {0};
    memcpy(sq, src->q, sizeof(uint32_t) * (size_t)Ls);
    memcpy(dq, dst->q, sizeof(uint32_t) * (size_t)Ld);
    memcpy(sh, src->half, sizeof(uint32_t) * (size_t)Ls);
    int above_half = big_cmp(integer, sh, n) > 0;
    uint32_t normalized[ORC_MAX_LIMBS + 1] = {0};
    if (big_cmp(dq, sq, n) > 0)
    {
        uint32_t offset[ORC_MAX_LIMBS + 1] = {0};
        big_sub(offset, dq, sq, n);
        if (above_half)
        {
            big_add(normalized, integer, offset, n);
        }
        else
        {
            memcpy(normalized, integer, sizeof normalized);
        }
    }
    else
    {
        uint32_t rem[ORC_MAX_LIMBS + 1] = {0};
        big_mod(rem, sq, n, dq, Ld);
        uint32_t offset[ORC_MAX_LIMBS + 1] = {0};
        int zero = 1;
        for (int i = 0; i < Ld; ++i)
        {
            zero &= rem[i] == 0;
        }
        if (!zero)
        {
            big_sub(offset, dq, rem, n);
        }
        if (above_half)
        {
            big_add(normalized, integer, offset, n);
        }
        else
        {
            memcpy(normalized, integer, sizeof normalized);
        }
    }
    orc_from_uint(dst, out, normalized, n);
}

/* square and multiply over the exponent bits (mod.hpp:409-434) */
void orc_pow(const orc_modulus* m, uint32_t* out, const uint32_t* x, const uint32_t* e, int e_limbs)
{
    int L = m->limbs;
    uint32_t result[ORC_MAX_LIMBS];
    uint32_t value[ORC_MAX_LIMBS];
    memcpy(result, m->one, sizeof(uint32_t) * (size_t)L);
    memcpy(value, x, sizeof(uint32_t) * (size_t)L);
    int bits = bit_width_words(e, e_limbs);
    for (int i = 0; i < bits; ++i)
    {
        if ((e[i / 32] >> (i % 32)) & 1u)
        {
            orc_mul(m, result, result, value);
        }
        orc_mul(m, value, value, value);
    }
    memcpy(out, result, sizeof(uint32_t) * (size_t)L);
}

void orc_invert(const orc_modulus* m, uint32_t* out, const uint32_t* x)
{
    uint32_t e[ORC_MAX_LIMBS] = {0};
    uint32_t two[ORC_MAX_LIMBS] = {2};
    big_sub(e, m->q, two, m->limbs);
    orc_pow(m, out, x, e, m->limbs);
}

/* --------------------------------------------------------------- chacha -- */

static uint32_t rotl32(uint32_t v, int c)
{
    return (v << c) | (v >> (32 - c));
}

/* crypto/chacha.hpp:13-30 */
void orc_chacha_quarter_round(uint32_t* a, uint32_t* b, uint32_t* c, uint32_t* d)
{
    *a += *b;
    *d ^= *a;
    *d = rotl32(*d, 16);
    *c += *d;
    *b ^= *c;
    *b = rotl32(*b, 12);
    *a += *b;
    *d ^= *a;
    *d = rotl32(*d, 8);
    *c += *d;
    *b ^= *c;
    *b = rotl32(*b, 7);
}

/* crypto/chacha.hpp:32-46 (double round), :91-115 (state), :144-166 (block) */
void orc_chacha20_block(const uint32_t key[8], uint32_t counter, const uint32_t nonce[3], uint32_t out[16])
{
    uint32_t s[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u};
    for (int i = 0; i < 8; ++i)
    {
        s[4 + i] = key[i];
    }
    s[12] = counter;
    s[13] = nonce[0];
    s[14] = nonce[1];
    s[15] = nonce[2];
    uint32_t x[16];
    memcpy(x, s, sizeof x);
    for (int r = 0; r < 10; ++r)
    {
        orc_chacha_quarter_round(&x[0], &x[4], &x[8], &x[12]);
        orc_chacha_quarter_round(&x[1], &x[5], &x[9], &x[13]);
        orc_chacha_quarter_round(&x[2], &x[6], &x[10], &x[14]);
        orc_chacha_quarter_round(&x[3], &x[7], &x[11], &x[15]);
        orc_chacha_quarter_round(&x[0], &x[5], &x[10], &x[15]);
        orc_chacha_quarter_round(&x[1], &x[6], &x[11], &x[12]);
        orc_chacha_quarter_round(&x[2], &x[7], &x[8], &x[13]);
        orc_chacha_quarter_round(&x[3], &x[4], &x[9], &x[14]);
    }
    for (int i = 0; i < 16; ++i)
    {
        out[i] = x[i] + s[i];
    }
}

/* random/number_generator.hpp:42-104: the first block is produced on
 * construction, one word per limb is consumed, and the next block (counter
 * + 1) is produced as soon as word 15 has been used. */
void orc_generator_init(orc_generator* g, const uint32_t key[8], const uint32_t nonce[3], uint32_t counter)
{
    memcpy(g->key, key, sizeof g->key);
    memcpy(g->nonce, nonce, sizeof g->nonce);
    orc_chacha20_block(g->key, counter, g->nonce, g->block);
    g->counter = counter + 1;
    g->index = 0;
}

uint32_t orc_generator_next(orc_generator* g)
{
    uint32_t w = g->block[g->index++];
    if (g->index == 16)
    {
        orc_chacha20_block(g->key, g->counter, g->nonce, g->block);
        g->counter += 1;
        g->index = 0;
    }
    return w;
}

/* random/binomial.hpp:29-86 (popcount of the low 4V bits of ceil(4V/32)
 * words, top word masked) and :110-122 (minus 2V) */
int64_t orc_sample_cbd(orc_generator* g, int variance_x2)
{
    int count = 2 * variance_x2;
    int words = (count + 31) / 32;
    int64_t sum = 0;
    for (int w = 0; w < words; ++w)
    {
        uint32_t word = orc_generator_next(g);
        if (w == words - 1 && (count % 32) != 0)
        {
            word &= (1u << (count % 32)) - 1u;
        }
        sum += __builtin_popcount(word);
    }
    return sum - variance_x2;
}

/* random/uniform.hpp:35-47,62-66 and ints/mod.hpp:210-215: draw
 * bit_width(Q-1)+security bits, then one reduction with
 * R' = 2^(32*max(L, words)). */
void orc_sample_uniform(const orc_modulus* m, orc_generator* g, uint32_t* out, int security)
{
    int bits = m->bits + security;
    int words = (bits + 31) / 32;
    uint32_t v[ORC_T_LIMBS];
    for (int w = 0; w < words; ++w)
    {
        v[w] = orc_generator_next(g);
    }
    if (bits % 32)
    {
        v[words - 1] &= (1u << (bits % 32)) - 1u;
    }
    int r = words > m->limbs ? words : m->limbs;
    orc_redc(m, out, v, words, r);
}

void orc_nonce_add(uint32_t nonce[3], uint64_t v)
{
    uint64_t s = (uint64_t)nonce[0] + (uint32_t)v;
    nonce[0] = (uint32_t)s;
    s = (uint64_t)nonce[1] + (uint32_t)(v >> 32) + (s >> 32);
    nonce[1] = (uint32_t)s;
    nonce[2] += (uint32_t)(s >> 32);
}

/* ---------------------------------------------------------------- roots -- */

static uint32_t bit_reverse(uint32_t v, int bits)
{
    uint32_t r = 0;
    for (int i = 0; i < bits; ++i)
    {
        r |= ((v >> i) & 1u) << (bits - 1 - i);
    }
    return r;
}

/* ints/num/theory/root_of_unity.hpp:20-54: candidates are L words of the
 * ChaCha stream with all-zero key, nonce and counter (top limb masked to
 * bit_width(Q-1) bits, minus Q when above Q-1, zero skipped); the first
 * g = x^((Q-1)/degree) with g^(degree/2) != 1 and g^degree == 1 wins. */
int orc_root_of_unity(const orc_modulus* m, uint64_t degree, uint32_t* out)
{
    int L = m->limbs;
    if (degree < 2 || (degree & (degree - 1)))
    {
        return 1;
    }
    uint32_t qm1[ORC_MAX_LIMBS] = {0};
    uint32_t one_word[ORC_MAX_LIMBS] = {1};
    big_sub(qm1, m->q, one_word, L);
    int shift = __builtin_ctzll(degree);
    /* exponent = (Q-1) / degree, exact */
    for (int i = 0; i < shift; ++i)
    {
        if (qm1[0] & 1u)
        {
            return 2;
        }
        for (int j = 0; j < L; ++j)
        {
            qm1[j] = (qm1[j] >> 1) | (j + 1 < L ? (qm1[j + 1] << 31) : 0u);
        }
    }
    uint32_t half_exp[2] = {(uint32_t)(degree / 2), (uint32_t)((degree / 2) >> 32)};
    uint32_t full_exp[2] = {(uint32_t)degree, (uint32_t)(degree >> 32)};
    uint32_t zeros[12] = {0};
    orc_generator g;
    orc_generator_init(&g, zeros, zeros, 0);
    uint32_t qm1_full[ORC_MAX_LIMBS] = {0};
    big_sub(qm1_full, m->q, one_word, L);
    for (long attempt = 0; attempt < 100000; ++attempt)
    {
        uint32_t x[ORC_MAX_LIMBS];
        for (int j = 0; j < L; ++j)
        {
            x[j] = orc_generator_next(&g);
        }
        if (m->bits % 32)
        {
            x[L - 1] &= (1u << (m->bits % 32)) - 1u;
        }
        if (big_cmp(x, qm1_full, L) > 0)
        {
            big_sub(x, x, m->q, L);
        }
        int zero = 1;
        for (int j = 0; j < L; ++j)
        {
            zero &= x[j] == 0;
        }
        if (zero)
        {
            continue;
        }
        uint32_t gpow[ORC_MAX_LIMBS];
        orc_pow(m, gpow, x, qm1, L);
        uint32_t t1[ORC_MAX_LIMBS];
        uint32_t t2[ORC_MAX_LIMBS];
        orc_pow(m, t1, gpow, half_exp, 2);
        orc_pow(m, t2, gpow, full_exp, 2);
        if (big_cmp(t1, m->one, L) != 0 && big_cmp(t2, m->one, L) == 0)
        {
            memcpy(out, gpow, sizeof(uint32_t) * (size_t)L);
            return 0;
        }
    }
    return 3;
}

/* number_theoretic_transform.hpp:35-88 */
int orc_twiddles(const orc_modulus* m, uint64_t n, int inverse, uint32_t* table)
{
    int L = m->limbs;
    if (n < 4 || (n & (n - 1)) || n > (1ull << 31))
    {
        return 1;
    }
    int bits = __builtin_ctzll(n);
    uint32_t root[ORC_MAX_LIMBS];
    int rc = orc_root_of_unity(m, 2 * n, root);
    if (rc)
    {
        return 10 + rc;
    }
    if (inverse)
    {
        orc_invert(m, root, root);
    }
    uint32_t nword[ORC_MAX_LIMBS] = {(uint32_t)n};
    uint32_t nmont[ORC_MAX_LIMBS];
    uint32_t normalization[ORC_MAX_LIMBS];
    orc_from_uint(m, nmont, nword, 1);
    orc_invert(m, normalization, nmont);
    memcpy(table, inverse ? normalization : m->one, sizeof(uint32_t) * (size_t)L);
    memcpy(table + (size_t)bit_reverse(1, bits) * L, root, sizeof(uint32_t) * (size_t)L);
    uint32_t power[ORC_MAX_LIMBS];
    memcpy(power, root, sizeof power);
    for (uint64_t i = 2; i < n; ++i)
    {
        orc_mul(m, power, power, root);
        uint32_t j = bit_reverse((uint32_t)i, bits);
        if (inverse && j == 1)
        {
            orc_mul(m, table + (size_t)j * L, power, normalization);
        }
        else
        {
            memcpy(table + (size_t)j * L, power, sizeof(uint32_t) * (size_t)L);
        }
    }
    return 0;
}

/* ------------------------------------------------------------------ NTT -- */

static void load_planar(const uint32_t* t, uint64_t elements, uint64_t e, int L, uint32_t* out)
{
    for (int j = 0; j < L; ++j)
    {
        out[j] = t[(uint64_t)j * elements + e];
    }
}

static void store_planar(uint32_t* t, uint64_t elements, uint64_t e, int L, const uint32_t* in)
{
    for (int j = 0; j < L; ++j)
    {
        t[(uint64_t)j * elements + e] = in[j];
    }
}

/* Produce the two inputs of one stage-0 butterfly.  Both come from ONE
 * capability object built from the first input's linear index, drawn one
 * after the other (number_theoretic_transform.hpp:316-329, :478-489;
 * comp/queue.hpp:191-212). */
static void produce_pair(const orc_modulus* m, const orc_producer* pr, uint64_t elements, uint64_t index,
                         uint64_t index_step, uint32_t* u, uint32_t* v)
{
    int L = m->limbs;
    switch (pr->kind)
    {
    case ORC_PRODUCER_TENSOR:
        load_planar(pr->src, elements, index, L, u);
        load_planar(pr->src, elements, index_step, L, v);
        break;
    case ORC_PRODUCER_CAST:
    {
        uint32_t x[ORC_MAX_LIMBS];
        load_planar(pr->src, elements, index, pr->src_modulus->limbs, x);
        orc_cast(m, pr->src_modulus, u, x);
        load_planar(pr->src, elements, index_step, pr->src_modulus->limbs, x);
        orc_cast(m, pr->src_modulus, v, x);
        break;
    }
    case ORC_PRODUCER_CBD:
    {
        orc_generator g;
        orc_generator_init(&g, pr->key, pr->nonce, (uint32_t)index);
        orc_from_int64(m, u, orc_sample_cbd(&g, pr->variance_x2));
        orc_from_int64(m, v, orc_sample_cbd(&g, pr->variance_x2));
        break;
    }
    case ORC_PRODUCER_UNIFORM:
    {
        orc_generator g;
        orc_generator_init(&g, pr->key, pr->nonce, (uint32_t)index);
        orc_sample_uniform(m, &g, u, pr->security);
        orc_sample_uniform(m, &g, v, pr->security);
        break;
    }
    default:
        break;
    }
}

/* Forward: number_theoretic_transform.hpp:144-197 (inner stages) and
 * :262-393 (first and last kernel).  Stage s: length = 2^s,
 * step = N/(2*length), psi = T[length + tid/step],
 * target = (tid/step)*2*step + tid%step; v *= psi; (u+v, u-v).
 * Inverse: :90-142 and :419-549.  Stage s: length = N >> (s+1),
 * step = 2^s; (u+v, (u-v)*psi); the last stage multiplies u+v by T[0] = N^-1
 * and u-v by T[1] (pre-multiplied by N^-1).
 * Work is element-major per polynomial (work[(i*N + k)*L + j]). */
int orc_ntt(const orc_modulus* m, uint64_t n, uint64_t batch, int inverse, const orc_producer* producer,
            uint32_t* out, int threads)
{
    int L = m->limbs;
    if (n < 4 || (n & (n - 1)))
    {
        return 1;
    }
    int bits = __builtin_ctzll(n);
    uint64_t elements = n * batch;
    uint32_t* table = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(n * (uint64_t)L));
    uint32_t* work = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(elements * (uint64_t)L));
    if (!table || !work)
    {
        free(table);
        free(work);
        return 2;
    }
    int rc = orc_twiddles(m, n, inverse, table);
    if (rc)
    {
        free(table);
        free(work);
        return rc;
    }
#ifdef _OPENMP
    if (threads > 0)
    {
        omp_set_num_threads(threads);
    }
#else
    (void)threads;
#endif
    int64_t pairs = (int64_t)(batch * (n / 2));
    for (int s = 0; s < bits; ++s)
    {
        uint64_t length = inverse ? (n >> (s + 1)) : (1ull << s);
        uint64_t step = inverse ? (1ull << s) : (n / length / 2);
        int first = s == 0;
        int last = s == bits - 1;
#pragma omp parallel for schedule(static)
        for (int64_t id = 0; id < pairs; ++id)
        {
            uint64_t i = (uint64_t)id / (n / 2);
            uint64_t tid = (uint64_t)id % (n / 2);
            uint64_t psi_step = tid / step;
            uint64_t target = psi_step * step * 2 + tid % step;
            const uint32_t* psi = table + (length + psi_step) * (uint64_t)L;
            uint32_t* pu = work + (i * n + target) * (uint64_t)L;
            uint32_t* pv = work + (i * n + target + step) * (uint64_t)L;
            uint32_t u[ORC_MAX_LIMBS];
            uint32_t v[ORC_MAX_LIMBS];
            uint32_t t[ORC_MAX_LIMBS];
            if (first)
            {
                produce_pair(m, producer, elements, i * n + target, i * n + target + step, u, v);
            }
            else
            {
                memcpy(u, pu, sizeof(uint32_t) * (size_t)L);
                memcpy(v, pv, sizeof(uint32_t) * (size_t)L);
            }
            if (!inverse)
            {
                orc_mul(m, v, v, psi);
                orc_add(m, pu, u, v);
                orc_sub(m, pv, u, v);
            }
            else if (!last)
            {
                orc_add(m, pu, u, v);
                orc_sub(m, t, u, v);
                orc_mul(m, pv, t, psi);
            }
            else
            {
                orc_add(m, t, u, v);
                orc_mul(m, pu, t, table);
                orc_sub(m, t, u, v);
                orc_mul(m, pv, t, table + L);
            }
        }
    }
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < (int64_t)elements; ++e)
    {
        store_planar(out, elements, (uint64_t)e, L, work + (uint64_t)e * L);
    }
    free(table);
    free(work);
    return 0;
}

/* --------------------------------------------------------- elementwise -- */

static void set_threads(int threads)
{
#ifdef _OPENMP
    if (threads > 0)
    {
        omp_set_num_threads(threads);
    }
#else
    (void)threads;
#endif
}

/* examples/fma.cpp:56-67: x[i] = a[i] * b[i] + c[i] */
void orc_fma(const orc_modulus* m, uint64_t elements, const uint32_t* a, const uint32_t* b, const uint32_t* c,
             uint32_t* d, int threads)
{
    int L = m->limbs;
    set_threads(threads);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < (int64_t)elements; ++e)
    {
        uint32_t x[ORC_MAX_LIMBS], y[ORC_MAX_LIMBS], z[ORC_MAX_LIMBS], t[ORC_MAX_LIMBS];
        load_planar(a, elements, (uint64_t)e, L, x);
        load_planar(b, elements, (uint64_t)e, L, y);
        load_planar(c, elements, (uint64_t)e, L, z);
        orc_mul(m, t, x, y);
        orc_add(m, t, t, z);
        store_planar(d, elements, (uint64_t)e, L, t);
    }
}

void orc_binary(const orc_modulus* m, int op, uint64_t elements, const uint32_t* a, uint64_t a_elements,
                const uint32_t* b, uint64_t b_elements, uint32_t* out, int threads)
{
    int L = m->limbs;
    set_threads(threads);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < (int64_t)elements; ++e)
    {
        uint32_t x[ORC_MAX_LIMBS] = {0}, y[ORC_MAX_LIMBS] = {0}, t[ORC_MAX_LIMBS];
        load_planar(a, a_elements, (uint64_t)e % a_elements, L, x);
        load_planar(b, b_elements, (uint64_t)e % b_elements, L, y);
        if (op == ORC_OP_ADD)
        {
            orc_add(m, t, x, y);
        }
        else if (op == ORC_OP_SUB)
        {
            orc_sub(m, t, x, y);
        }
        else
        {
            orc_mul(m, t, x, y);
        }
        store_planar(out, elements, (uint64_t)e, L, t);
    }
}

/* expr/matrix_vector_product.hpp:88-140: output element (b, i, c) is the
 * fold over k of matrix(b, i, k, c) * vector(b, k, c) with mod<Q>'s product
 * and sum; the matrix index inserts k after (b, i), the vector index replaces
 * i by k (:101-113).  A batch extent of one broadcasts (:7-23). */
void orc_matvec(const orc_modulus* m, uint64_t batch, uint64_t rows, uint64_t cols, uint64_t coeffs,
                const uint32_t* mat, uint64_t m_batch, const uint32_t* x, uint64_t x_batch, uint32_t* z,
                int threads)
{
    int L = m->limbs;
    uint64_t m_el = m_batch * rows * cols * coeffs;
    uint64_t x_el = x_batch * cols * coeffs;
    uint64_t z_el = batch * rows * coeffs;
    set_threads(threads);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < (int64_t)z_el; ++e)
    {
        uint64_t c = (uint64_t)e % coeffs, t = (uint64_t)e / coeffs;
        uint64_t i = t % rows, b = t / rows;
        uint64_t bm = m_batch == 1 ? 0 : b, bx = x_batch == 1 ? 0 : b;
        uint32_t acc[ORC_MAX_LIMBS] = {0}, a[ORC_MAX_LIMBS], v[ORC_MAX_LIMBS], p[ORC_MAX_LIMBS];
        for (uint64_t k = 0; k < cols; ++k)
        {
            load_planar(mat, m_el, ((bm * rows + i) * cols + k) * coeffs + c, L, a);
            load_planar(x, x_el, (bx * cols + k) * coeffs + c, L, v);
            orc_mul(m, p, a, v);
            orc_add(m, acc, acc, p);
        }
        store_planar(z, z_el, (uint64_t)e, L, acc);
    }
}

/* expr/bit_monomial.hpp:28-104: coefficient c of X^d * x is x[(c - d) mod n],
 * negated when c - d (as an unsigned 64-bit difference) has bit log2(n) set
 * (one wrap past X^n = -1); no monomial contributes zero (:98-101). */
void orc_matvec_monomial(const orc_modulus* m, uint64_t n, uint64_t batch, uint64_t rows, uint64_t cols,
                         const int64_t* degrees, uint64_t d_batch, const uint32_t* x, uint64_t x_batch,
                         uint32_t* z, int threads)
{
    int L = m->limbs;
    int bits = __builtin_ctzll(n);
    uint64_t x_el = x_batch * cols * n;
    uint64_t z_el = batch * rows * n;
    set_threads(threads);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < (int64_t)z_el; ++e)
    {
        uint64_t c = (uint64_t)e % n, t = (uint64_t)e / n;
        uint64_t i = t % rows, b = t / rows;
        uint64_t bd = d_batch == 1 ? 0 : b, bx = x_batch == 1 ? 0 : b;
        uint32_t acc[ORC_MAX_LIMBS] = {0}, v[ORC_MAX_LIMBS];
        for (uint64_t k = 0; k < cols; ++k)
        {
            int64_t d = degrees[(bd * rows + i) * cols + k];
            if (d < 0)
            {
                continue;
            }
            uint64_t difference = c - (uint64_t)d;
            uint64_t src = difference & (n - 1);
            int negative = (int)((difference >> bits) & 1u);
            load_planar(x, x_el, (bx * cols + k) * n + src, L, v);
            if (negative)
            {
                orc_neg(m, v, v);
            }
            orc_add(m, acc, acc, v);
        }
        store_planar(z, z_el, (uint64_t)e, L, acc);
    }
}

/* expr/reduce.hpp:206-250 over mod<Q>: sycl::plus / sycl::multiplies on
 * mod's operators, identities integer_traits<mod>::zero and ::one (the
 * Montgomery form of 1, R mod Q; ints/integer_traits.hpp:75-76). */
int orc_reduce_mod(const orc_modulus* m, int op, uint64_t elements, const uint32_t* in, uint32_t* out)
{
    int L = m->limbs;
    uint32_t acc[ORC_MAX_LIMBS] = {0}, v[ORC_MAX_LIMBS];
    if (op == ORC_REDUCE_MULTIPLY)
    {
        memcpy(acc, m->one, sizeof(uint32_t) * (size_t)L);
    }
    else if (op != ORC_REDUCE_ADD)
    {
        return 1;
    }
    for (uint64_t e = 0; e < elements; ++e)
    {
        load_planar(in, elements, e, L, v);
        if (op == ORC_REDUCE_ADD)
        {
            orc_add(m, acc, acc, v);
        }
        else
        {
            orc_mul(m, acc, acc, v);
        }
    }
    memcpy(out, acc, sizeof(uint32_t) * (size_t)L);
    return 0;
}

static void mask_bits(uint32_t* x, int limbs, int bits)
{
    if (bits % 32)
    {
        x[limbs - 1] &= (1u << (bits % 32)) - 1u;
    }
}

/* expr/reduce.hpp:206-250 over uint<bits> (ints/uint.hpp): identities of
 * ints/integer_traits.hpp:39-46 (zero, one, all_ones = compl all_zeros,
 * max = all_ones, min = zero); the accumulator is a uint<bits>, so sums and
 * products keep their low `bits` bits. */
int orc_reduce_uint(int op, int bits, uint64_t elements, const uint32_t* in, uint32_t* out)
{
    if (bits < 1 || bits > 32 * ORC_MAX_LIMBS || op < ORC_REDUCE_ADD || op > ORC_REDUCE_MAX)
    {
        return 1;
    }
    int L = (bits + 31) / 32;
    uint32_t acc[ORC_MAX_LIMBS] = {0}, v[ORC_MAX_LIMBS], wide[2 * ORC_MAX_LIMBS];
    if (op == ORC_REDUCE_MULTIPLY)
    {
        acc[0] = 1;
    }
    else if (op == ORC_REDUCE_BIT_AND || op == ORC_REDUCE_MIN)
    {
        memset(acc, 0xff, sizeof(uint32_t) * (size_t)L);
        mask_bits(acc, L, bits);
    }
    for (uint64_t e = 0; e < elements; ++e)
    {
        load_planar(in, elements, e, L, v);
        mask_bits(v, L, bits);
        switch (op)
        {
        case ORC_REDUCE_ADD:
            big_add(acc, acc, v, L);
            break;
        case ORC_REDUCE_MULTIPLY:
            big_mul(wide, acc, L, v, L);
            memcpy(acc, wide, sizeof(uint32_t) * (size_t)L);
            break;
        case ORC_REDUCE_BIT_AND:
            for (int j = 0; j < L; ++j) acc[j] &= v[j];
            break;
        case ORC_REDUCE_BIT_OR:
            for (int j = 0; j < L; ++j) acc[j] |= v[j];
            break;
        case ORC_REDUCE_BIT_XOR:
            for (int j = 0; j < L; ++j) acc[j] ^= v[j];
            break;
        case ORC_REDUCE_MIN:
            if (big_cmp(v, acc, L) < 0) memcpy(acc, v, sizeof(uint32_t) * (size_t)L);
            break;
        default:
            if (big_cmp(v, acc, L) > 0) memcpy(acc, v, sizeof(uint32_t) * (size_t)L);
            break;
        }
        mask_bits(acc, L, bits);
    }
    memcpy(out, acc, sizeof(uint32_t) * (size_t)L);
    return 0;
}

/* binary_expression.hpp with operator== (core/equal_to.hpp): one hmpc::bit per element */
void orc_equal(int limbs, uint64_t elements, const uint32_t* a, const uint32_t* b, uint32_t* out)
{
    for (uint64_t e = 0; e < elements; ++e)
    {
        uint32_t eq = 1;
        for (int j = 0; j < limbs; ++j)
        {
            eq &= a[(uint64_t)j * elements + e] == b[(uint64_t)j * elements + e];
        }
        out[e] = eq;
    }
}

/* expr/random/uniform.hpp:41-45 with the capability of comp/queue.hpp:191-212 */
void orc_sample_uniform_tensor(const orc_modulus* m, uint64_t elements, const uint32_t key[8],
                               const uint32_t nonce[3], int security, uint32_t* out, int threads)
{
    int L = m->limbs;
    set_threads(threads);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < (int64_t)elements; ++e)
    {
        orc_generator g;
        uint32_t t[ORC_MAX_LIMBS];
        orc_generator_init(&g, key, nonce, (uint32_t)e);
        orc_sample_uniform(m, &g, t, security);
        store_planar(out, elements, (uint64_t)e, L, t);
    }
}

/* expr/random/binomial.hpp:207-211 */
void orc_sample_cbd_tensor(const orc_modulus* m, uint64_t elements, const uint32_t key[8], const uint32_t nonce[3],
                           int variance_x2, uint32_t* out, int threads)
{
    int L = m->limbs;
    set_threads(threads);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < (int64_t)elements; ++e)
    {
        orc_generator g;
        uint32_t t[ORC_MAX_LIMBS];
        orc_generator_init(&g, key, nonce, (uint32_t)e);
        orc_from_int64(m, t, orc_sample_cbd(&g, variance_x2));
        store_planar(out, elements, (uint64_t)e, L, t);
    }
}

void orc_cast_tensor(const orc_modulus* dst, const orc_modulus* src, uint64_t elements, const uint32_t* x,
                     uint32_t* out, int threads)
{
    set_threads(threads);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < (int64_t)elements; ++e)
    {
        uint32_t a[ORC_MAX_LIMBS], t[ORC_MAX_LIMBS];
        load_planar(x, elements, (uint64_t)e, src->limbs, a);
        orc_cast(dst, src, t, a);
        store_planar(out, elements, (uint64_t)e, dst->limbs, t);
    }
}

void orc_to_uint_tensor(const orc_modulus* m, uint64_t elements, const uint32_t* x, uint32_t* out, int threads)
{
    set_threads(threads);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < (int64_t)elements; ++e)
    {
        uint32_t a[ORC_MAX_LIMBS], t[ORC_MAX_LIMBS];
        load_planar(x, elements, (uint64_t)e, m->limbs, a);
        orc_to_uint(m, t, a);
        store_planar(out, elements, (uint64_t)e, m->limbs, t);
    }
}

void orc_from_uint_tensor(const orc_modulus* m, uint64_t elements, const uint32_t* x, uint32_t* out, int threads)
{
    set_threads(threads);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < (int64_t)elements; ++e)
    {
        uint32_t a[ORC_MAX_LIMBS], t[ORC_MAX_LIMBS];
        load_planar(x, elements, (uint64_t)e, m->limbs, a);
        orc_from_uint(m, t, a, m->limbs);
        store_planar(out, elements, (uint64_t)e, m->limbs, t);
    }
}

/* ------------------------------------------------------------------ LHE -- */

static orc_producer sampler(int kind, int variance_x2, const uint32_t key[8], const uint32_t nonce[3])
{
    orc_producer pr;
    memset(&pr, 0, sizeof pr);
    pr.kind = kind;
    pr.variance_x2 = variance_x2;
    pr.security = 80;
    memcpy(pr.key, key, sizeof pr.key);
    memcpy(pr.nonce, nonce, sizeof pr.nonce);
    return pr;
}

/* expr/crypto/lhe/enc.hpp:19-69 with randomness.hpp:196-226; the cache plan
 * (expr/cache.hpp:226-271) runs NTT(u), NTT(v), [INTT_p(x)], NTT_q(msg), c0,
 * NTT(w), c1 and every kernel with a sampler advances the nonce by its
 * element count (comp/queue.hpp:241-253). */
int orc_lhe_enc(const orc_modulus* q, const orc_modulus* p, uint64_t n, uint64_t batch, const uint32_t* key_a,
                const uint32_t* key_b, const uint32_t* plaintext, int plaintext_ntt, const uint32_t key[8],
                uint32_t nonce[3], uint32_t* c0, uint32_t* c1, int threads)
{
    int L = q->limbs;
    uint64_t elements = n * batch;
    size_t bytes = sizeof(uint32_t) * (size_t)(elements * (uint64_t)L);
    uint32_t* u = (uint32_t*)malloc(bytes);
    uint32_t* v = (uint32_t*)malloc(bytes);
    uint32_t* w = (uint32_t*)malloc(bytes);
    uint32_t* msg = (uint32_t*)malloc(bytes);
    uint32_t* coeff = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(elements * (uint64_t)p->limbs));
    int rc = 0;
    if (!u || !v || !w || !msg || !coeff)
    {
        rc = 2;
        goto done;
    }
    orc_producer pr = sampler(ORC_PRODUCER_CBD, 1, key, nonce);
    if ((rc = orc_ntt(q, n, batch, 0, &pr, u, threads)))
        goto done;
    orc_nonce_add(nonce, elements);
    pr = sampler(ORC_PRODUCER_CBD, 20, key, nonce);
    if ((rc = orc_ntt(q, n, batch, 0, &pr, v, threads)))
        goto done;
    orc_nonce_add(nonce, elements);
    const uint32_t* coefficients = plaintext;
    if (plaintext_ntt)
    {
        orc_producer tp;
        memset(&tp, 0, sizeof tp);
        tp.kind = ORC_PRODUCER_TENSOR;
        tp.src = plaintext;
        if ((rc = orc_ntt(p, n, batch, 1, &tp, coeff, threads)))
            goto done;
        coefficients = coeff;
    }
    orc_producer cp;
    memset(&cp, 0, sizeof cp);
    cp.kind = ORC_PRODUCER_CAST;
    cp.src = coefficients;
    cp.src_modulus = p;
    if ((rc = orc_ntt(q, n, batch, 0, &cp, msg, threads)))
        goto done;
    {
        /* p as a constant mod q (enc.hpp:59-63) */
        uint32_t pmont[ORC_MAX_LIMBS];
        orc_from_uint(q, pmont, p->q, p->limbs);
        set_threads(threads);
#pragma omp parallel for schedule(static)
        for (int64_t e = 0; e < (int64_t)elements; ++e)
        {
            uint64_t k = (uint64_t)e % n;
            uint32_t a[ORC_MAX_LIMBS], x[ORC_MAX_LIMBS], y[ORC_MAX_LIMBS], t[ORC_MAX_LIMBS];
            load_planar(key_a, n, k, L, a);
            load_planar(u, elements, (uint64_t)e, L, x);
            orc_mul(q, t, a, x);
            load_planar(v, elements, (uint64_t)e, L, y);
            orc_mul(q, y, y, pmont);
            orc_add(q, t, t, y);
            load_planar(msg, elements, (uint64_t)e, L, y);
            orc_add(q, t, t, y);
            store_planar(c0, elements, (uint64_t)e, L, t);
        }
        pr = sampler(ORC_PRODUCER_CBD, 20, key, nonce);
        if ((rc = orc_ntt(q, n, batch, 0, &pr, w, threads)))
            goto done;
        orc_nonce_add(nonce, elements);
#pragma omp parallel for schedule(static)
        for (int64_t e = 0; e < (int64_t)elements; ++e)
        {
            uint64_t k = (uint64_t)e % n;
            uint32_t b[ORC_MAX_LIMBS], x[ORC_MAX_LIMBS], y[ORC_MAX_LIMBS], t[ORC_MAX_LIMBS];
            load_planar(key_b, n, k, L, b);
            load_planar(u, elements, (uint64_t)e, L, x);
            orc_mul(q, t, b, x);
            load_planar(w, elements, (uint64_t)e, L, y);
            orc_mul(q, y, y, pmont);
            orc_add(q, t, t, y);
            store_planar(c1, elements, (uint64_t)e, L, t);
        }
    }
done:
    free(u);
    free(v);
    free(w);
    free(msg);
    free(coeff);
    return rc;
}

/* expr/crypto/lhe/dec.hpp:13-45 */
int orc_lhe_dec(const orc_modulus* q, const orc_modulus* p, uint64_t n, uint64_t batch, const uint32_t* s,
                const uint32_t* c0, const uint32_t* c1, int plaintext_ntt, uint32_t* out, int threads)
{
    int L = q->limbs;
    uint64_t elements = n * batch;
    uint32_t* x = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(elements * (uint64_t)L));
    uint32_t* coeff = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(elements * (uint64_t)L));
    int rc = 0;
    if (!x || !coeff)
    {
        rc = 2;
        goto done;
    }
    set_threads(threads);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < (int64_t)elements; ++e)
    {
        uint64_t k = (uint64_t)e % n;
        uint32_t a[ORC_MAX_LIMBS], b[ORC_MAX_LIMBS], sk[ORC_MAX_LIMBS], t[ORC_MAX_LIMBS];
        load_planar(c0, elements, (uint64_t)e, L, a);
        load_planar(c1, elements, (uint64_t)e, L, b);
        load_planar(s, n, k, L, sk);
        orc_mul(q, t, sk, b);
        orc_sub(q, t, a, t);
        store_planar(x, elements, (uint64_t)e, L, t);
    }
    orc_producer tp;
    memset(&tp, 0, sizeof tp);
    tp.kind = ORC_PRODUCER_TENSOR;
    tp.src = x;
    if ((rc = orc_ntt(q, n, batch, 1, &tp, coeff, threads)))
        goto done;
    if (plaintext_ntt)
    {
        orc_producer cp;
        memset(&cp, 0, sizeof cp);
        cp.kind = ORC_PRODUCER_CAST;
        cp.src = coeff;
        cp.src_modulus = q;
        rc = orc_ntt(p, n, batch, 0, &cp, out, threads);
    }
    else
    {
        orc_cast_tensor(p, q, elements, coeff, out, threads);
    }
done:
    free(x);
    free(coeff);
    return rc;
}

int orc_lhe_keygen(const orc_modulus* q, const orc_modulus* p, uint64_t n, const uint32_t key[8], uint32_t nonce[3],
                   uint32_t* s, uint32_t* a, uint32_t* b, int threads)
{
    int L = q->limbs;
    uint32_t* e = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(n * (uint64_t)L));
    if (!e)
    {
        return 2;
    }
    orc_sample_uniform_tensor(q, n, key, nonce, 80, b, threads);
    orc_nonce_add(nonce, n);
    orc_producer pr = sampler(ORC_PRODUCER_CBD, 1, key, nonce);
    int rc = orc_ntt(q, n, 1, 0, &pr, s, threads);
    orc_nonce_add(nonce, n);
    if (!rc)
    {
        pr = sampler(ORC_PRODUCER_CBD, 20, key, nonce);
        rc = orc_ntt(q, n, 1, 0, &pr, e, threads);
        orc_nonce_add(nonce, n);
    }
    if (!rc)
    {
        uint32_t pmont[ORC_MAX_LIMBS];
        orc_from_uint(q, pmont, p->q, p->limbs);
        for (uint64_t k = 0; k < n; ++k)
        {
            uint32_t x[ORC_MAX_LIMBS], y[ORC_MAX_LIMBS], t[ORC_MAX_LIMBS];
            load_planar(b, n, k, L, x);
            load_planar(s, n, k, L, y);
            orc_mul(q, t, x, y);
            load_planar(e, n, k, L, x);
            orc_mul(q, x, x, pmont);
            orc_add(q, t, t, x);
            store_planar(a, n, k, L, t);
        }
    }
    free(e);
    return rc;
}

/* ---------------------------------------------------------------- cipher -- */

/* expr/crypto/cipher.hpp:128-173: the work is cut into batches of
 * lcm(16, limbs) words; batch b starts a generator at counter
 * b * (batch / 16) and consumes one word per limb of its elements in order --
 * so word w of the element-major output uses word w % 16 of block w / 16. */
static uint64_t gcd_u64(uint64_t a, uint64_t b)
{
    while (b)
    {
        uint64_t t = a % b;
        a = b;
        b = t;
    }
    return a;
}

static void cipher_batches(const uint32_t key[8], const uint32_t nonce[3], uint64_t elements, int limbs,
                           const uint32_t* in, uint32_t* out, int decrypt)
{
    const uint64_t batch = 16 / gcd_u64(16, (uint64_t)limbs) * (uint64_t)limbs;
    const uint64_t per_batch = batch / (uint64_t)limbs;
    const uint64_t blocks = batch / 16;
    const uint64_t count = (elements * (uint64_t)limbs + batch - 1) / batch;
#pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < (int64_t)count; ++b)
    {
        orc_generator g;
        orc_generator_init(&g, key, nonce, (uint32_t)((uint64_t)b * blocks));
        for (uint64_t e = 0; e < per_batch; ++e)
        {
            uint64_t i = (uint64_t)b * per_batch + e;
            if (i >= elements)
            {
                break;
            }
            for (int j = 0; j < limbs; ++j)
            {
                uint32_t mask = orc_generator_next(&g);
                if (!decrypt)
                {
                    out[i * (uint64_t)limbs + (uint64_t)j] = in[(uint64_t)j * elements + i] ^ mask;
                }
                else
                {
                    out[(uint64_t)j * elements + i] = in[i * (uint64_t)limbs + (uint64_t)j] ^ mask;
                }
            }
        }
    }
}

void orc_cipher_enc(const uint32_t key[8], const uint32_t nonce[3], uint64_t elements, int limbs,
                    const uint32_t* planar_in, uint32_t* flat_out)
{
    cipher_batches(key, nonce, elements, limbs, planar_in, flat_out, 0);
}

void orc_cipher_dec(const uint32_t key[8], const uint32_t nonce[3], uint64_t elements, int limbs,
                    const uint32_t* flat_in, uint32_t* planar_out)
{
    cipher_batches(key, nonce, elements, limbs, flat_in, planar_out, 1);
}
