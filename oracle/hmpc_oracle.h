/*
 * hmpc_oracle.h -- CPU restatement of hmpc's data-parallel hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path and
 * the timed CPU baseline; the product (hmpc_gb300) never links, loads or calls
 * it.  Every function restates an algorithm of the reference hmpc v0.5.2 and
 * cites the file:line it follows (paths relative to the hmpc source tree).
 *
 * Conventions shared with the reference:
 *   - limbs are 32-bit words, least significant first (hmpc/config.hpp:72);
 *   - a residue is stored as its fully reduced Montgomery representative
 *     x*R mod Q with R = 2^(32*L), L = ceil(bit_width(Q-1)/32)
 *     (hmpc/ints/mod.hpp:90-93);
 *   - tensors are limb-planar: limb j of element e lives at [j*elements + e]
 *     (hmpc/comp/tensor.hpp:21,25-29; hmpc/comp/accessor.hpp:191-197).
 */
#ifndef HMPC_ORACLE_H
#define HMPC_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_LIMBS 16

typedef struct orc_modulus
{
    int limbs;                      /* L */
    int bits;                       /* bit_width(Q - 1) */
    uint32_t ninv;                  /* -Q^{-1} mod 2^32 (mod.hpp:98-103) */
    uint32_t q[ORC_MAX_LIMBS];      /* Q */
    uint32_t half[ORC_MAX_LIMBS];   /* Q >> 1 (mod.hpp:79) */
    uint32_t one[ORC_MAX_LIMBS];    /* R mod Q (mod.hpp:114) */
    uint32_t r2[ORC_MAX_LIMBS];     /* R^2 mod Q (mod.hpp:117) */
} orc_modulus;

/* Returns 0 on success, nonzero if Q is even, zero, or too wide. */
int orc_modulus_init(orc_modulus* m, const uint32_t* q, int q_limbs);

/* Separated word-by-word Montgomery reduction with R = 2^(32*r). */
void orc_redc(const orc_modulus* m, uint32_t* out, const uint32_t* value, int value_limbs, int r);
void orc_mul(const orc_modulus* m, uint32_t* out, const uint32_t* a, const uint32_t* b);
void orc_add(const orc_modulus* m, uint32_t* out, const uint32_t* a, const uint32_t* b);
void orc_sub(const orc_modulus* m, uint32_t* out, const uint32_t* a, const uint32_t* b);
void orc_neg(const orc_modulus* m, uint32_t* out, const uint32_t* a);
/* canonical integer (any width) -> Montgomery representative */
void orc_from_uint(const orc_modulus* m, uint32_t* out, const uint32_t* value, int value_limbs);
/* Montgomery representative -> canonical integer in [0, Q) */
void orc_to_uint(const orc_modulus* m, uint32_t* out, const uint32_t* x);
void orc_from_int64(const orc_modulus* m, uint32_t* out, int64_t v);
/* centred lift of a residue mod src into dst (mod.hpp:259-307) */
void orc_cast(const orc_modulus* dst, const orc_modulus* src, uint32_t* out, const uint32_t* x);
/* x^e in Montgomery arithmetic, e given as e_limbs words */
void orc_pow(const orc_modulus* m, uint32_t* out, const uint32_t* x, const uint32_t* e, int e_limbs);
/* multiplicative inverse through Fermat (Q prime); returns Montgomery form */
void orc_invert(const orc_modulus* m, uint32_t* out, const uint32_t* x);

/* ChaCha20, state [const x4, key x8, counter x1, nonce x3] (crypto/chacha.hpp:146-166) */
void orc_chacha20_block(const uint32_t key[8], uint32_t counter, const uint32_t nonce[3], uint32_t out[16]);
void orc_chacha_quarter_round(uint32_t* a, uint32_t* b, uint32_t* c, uint32_t* d);

typedef struct orc_generator
{
    uint32_t key[8];
    uint32_t nonce[3];
    uint32_t counter;
    uint32_t block[16];
    int index;
} orc_generator;

void orc_generator_init(orc_generator* g, const uint32_t key[8], const uint32_t nonce[3], uint32_t counter);
uint32_t orc_generator_next(orc_generator* g);
/* centred binomial with variance V, variance_x2 = 2V (random/binomial.hpp:110-122) */
int64_t orc_sample_cbd(orc_generator* g, int variance_x2);
/* uniform<mod<Q>> with statistical security `security` (random/uniform.hpp:62-66) */
void orc_sample_uniform(const orc_modulus* m, orc_generator* g, uint32_t* out, int security);

/* 96-bit little-endian nonce += v (comp/queue.hpp:241-253) */
void orc_nonce_add(uint32_t nonce[3], uint64_t v);

/* primitive `degree`-th root of unity, Montgomery form (root_of_unity.hpp:20-54).
 * Returns 0 on success. */
int orc_root_of_unity(const orc_modulus* m, uint64_t degree, uint32_t* out);
/* twiddle table of N entries, element-major: entry k at table[k*L .. k*L+L-1]
 * (number_theoretic_transform.hpp:35-88) */
int orc_twiddles(const orc_modulus* m, uint64_t n, int inverse, uint32_t* table);

enum
{
    ORC_PRODUCER_TENSOR = 0,
    ORC_PRODUCER_CBD = 1,
    ORC_PRODUCER_UNIFORM = 2,
    ORC_PRODUCER_CAST = 3,
};

/* What feeds stage 0 of a transform: a tensor (limb-planar, batch*N elements),
 * a sampler driven by the RNG capability (key, nonce; counter = element
 * index), or a tensor of another modulus lifted through a cast. */
typedef struct orc_producer
{
    int kind;
    const uint32_t* src;
    const orc_modulus* src_modulus;
    int variance_x2;
    int security;
    uint32_t key[8];
    uint32_t nonce[3];
} orc_producer;

/* Batched negacyclic NTT (inverse=0) or INTT (inverse=1) of `batch`
 * polynomials of degree n; out is limb-planar with batch*n elements.
 * threads <= 0 uses the OpenMP default.  Returns 0 on success. */
int orc_ntt(const orc_modulus* m, uint64_t n, uint64_t batch, int inverse, const orc_producer* producer,
            uint32_t* out, int threads);

/* d = a*b + c over limb-planar tensors (examples/fma.cpp:56-67) */
void orc_fma(const orc_modulus* m, uint64_t elements, const uint32_t* a, const uint32_t* b, const uint32_t* c,
             uint32_t* d, int threads);

enum
{
    ORC_OP_ADD = 0,
    ORC_OP_SUB = 1,
    ORC_OP_MUL = 2,
};
/* out[e] = a[e % a_elements] OP b[e % b_elements]  (broadcast of a single
 * polynomial over a batch, expr/unsqueeze.hpp + binary_expression.hpp:118-136) */
void orc_binary(const orc_modulus* m, int op, uint64_t elements, const uint32_t* a, uint64_t a_elements,
                const uint32_t* b, uint64_t b_elements, uint32_t* out, int threads);

/* elementwise samplers: element e uses the generator (key, nonce, counter=e) */
void orc_sample_uniform_tensor(const orc_modulus* m, uint64_t elements, const uint32_t key[8],
                               const uint32_t nonce[3], int security, uint32_t* out, int threads);
void orc_sample_cbd_tensor(const orc_modulus* m, uint64_t elements, const uint32_t key[8], const uint32_t nonce[3],
                           int variance_x2, uint32_t* out, int threads);
void orc_cast_tensor(const orc_modulus* dst, const orc_modulus* src, uint64_t elements, const uint32_t* x,
                     uint32_t* out, int threads);
/* canonical <-> Montgomery over limb-planar tensors */
void orc_to_uint_tensor(const orc_modulus* m, uint64_t elements, const uint32_t* x, uint32_t* out, int threads);
void orc_from_uint_tensor(const orc_modulus* m, uint64_t elements, const uint32_t* x, uint32_t* out, int threads);

/* Matrix-vector product (expr/matrix_vector_product.hpp:88-140) of mod<Q>
 * tensors: z[b][i][c] = sum_k m[b][i][k][c] * x[b][k][c], c < coeffs (the
 * coefficients of NTT-form polynomials, whose ring product is elementwise).
 * m_batch and x_batch are batch or 1 (a batch of one is broadcast, the
 * common_extent of matrix_vector_product.hpp:7-23). */
void orc_matvec(const orc_modulus* m, uint64_t batch, uint64_t rows, uint64_t cols, uint64_t coeffs,
                const uint32_t* mat, uint64_t m_batch, const uint32_t* x, uint64_t x_batch, uint32_t* z,
                int threads);
/* The same product with a matrix of bit monomials X^d (expr/bit_monomial.hpp:
 * 18-104) times polynomials of degree n in coefficient form mod Q:
 * degrees[b][i][k] < 0 stands for std::nullopt (no monomial). */
void orc_matvec_monomial(const orc_modulus* m, uint64_t n, uint64_t batch, uint64_t rows, uint64_t cols,
                         const int64_t* degrees, uint64_t d_batch, const uint32_t* x, uint64_t x_batch,
                         uint32_t* z, int threads);

enum
{
    ORC_REDUCE_ADD = 0,
    ORC_REDUCE_MULTIPLY = 1,
    ORC_REDUCE_BIT_AND = 2,
    ORC_REDUCE_BIT_OR = 3,
    ORC_REDUCE_BIT_XOR = 4,
    ORC_REDUCE_MIN = 5,
    ORC_REDUCE_MAX = 6,
};
/* Reduction of every element to one value (expr/reduce.hpp:206-250).
 * mod<Q>: add or multiply (returns 1 for other operations); out has L words. */
int orc_reduce_mod(const orc_modulus* m, int op, uint64_t elements, const uint32_t* in, uint32_t* out);
/* uint<bits> in ceil(bits/32) limb planes: every operation; sums and products
 * wrap modulo 2^bits.  Returns 1 for a bad operation or width. */
int orc_reduce_uint(int op, int bits, uint64_t elements, const uint32_t* in, uint32_t* out);
/* out[e] = 1 if a[e] == b[e] (every limb) else 0: the hmpc::bit of x == y */
void orc_equal(int limbs, uint64_t elements, const uint32_t* a, const uint32_t* b, uint32_t* out);

/* Linear BGV (expr/crypto/lhe/enc.hpp:19-69): given key (a, b) in NTT form
 * mod q (one polynomial each) and `batch` plaintexts mod p, compute the
 * ciphertexts with the reference's execution order
 *   NTT(u), NTT(v), NTT(msg), c0, NTT(w), c1
 * advancing `nonce` as the queue does.  plaintext_ntt selects whether the
 * plaintext is in NTT representation mod p (then INTT_p is applied first). */
int orc_lhe_enc(const orc_modulus* q, const orc_modulus* p, uint64_t n, uint64_t batch, const uint32_t* key_a,
                const uint32_t* key_b, const uint32_t* plaintext, int plaintext_ntt, const uint32_t key[8],
                uint32_t nonce[3], uint32_t* c0, uint32_t* c1, int threads);
/* dec (expr/crypto/lhe/dec.hpp:13-45): c0 - s*c1 -> INTT_q -> cast to p
 * (-> NTT_p when plaintext_ntt). */
int orc_lhe_dec(const orc_modulus* q, const orc_modulus* p, uint64_t n, uint64_t batch, const uint32_t* s,
                const uint32_t* c0, const uint32_t* c1, int plaintext_ntt, uint32_t* out, int threads);
/* key generation (no counterpart in the reference): b <- uniform (NTT form),
 * s <- NTT(CBD(1/2)), e <- NTT(CBD(10)), a = b*s + p*e; nonce order b, s, e. */
int orc_lhe_keygen(const orc_modulus* q, const orc_modulus* p, uint64_t n, const uint32_t key[8], uint32_t nonce[3],
                   uint32_t* s, uint32_t* a, uint32_t* b, int threads);

/* ChaCha20 stream cipher over a tensor (expr/crypto/cipher.hpp:59-173,
 * crypto/cipher.hpp:29-44): element i's limbs (limb-planar input, `limbs`
 * words each) are XORed with keystream words i*limbs .. i*limbs+limbs-1 of
 * ChaCha20(key, nonce, counter from 0) and written element-major
 * (out[i*limbs + j]).  dec reads element-major and writes limb-planar. */
void orc_cipher_enc(const uint32_t key[8], const uint32_t nonce[3], uint64_t elements, int limbs,
                    const uint32_t* planar_in, uint32_t* flat_out);
void orc_cipher_dec(const uint32_t key[8], const uint32_t nonce[3], uint64_t elements, int limbs,
                    const uint32_t* flat_in, uint32_t* planar_out);

#ifdef __cplusplus
}
#endif

#endif
