/*
 * hmpc_gb300.h -- C ABI of the GB300 (sm_103a) implementation of hmpc's
 * data-parallel hot path: multi-limb Montgomery arithmetic, the negacyclic
 * NTT/INTT, the elementwise modular FMA, the ChaCha20 samplers and linear BGV.
 *
 * This is the device boundary that hmpc's SYCL device path crosses inside
 * hmpc::comp::queue (hmpc/comp/queue.hpp:313-414): where the reference submits
 * a parallel_for per expression node, a host front end calls these entry
 * points instead.  Conventions shared with the reference:
 *
 *  - A residue mod Q is L = ceil(bit_width(Q-1)/32) 32-bit limbs, least
 *    significant first, holding the fully reduced Montgomery representative
 *    x*R mod Q, R = 2^(32L) (hmpc/ints/mod.hpp:73-193).
 *  - Tensors are caller-owned device buffers in the reference's limb-planar
 *    layout: limb j of element e at [j*elements + e]
 *    (hmpc/comp/tensor.hpp:21,25-29; hmpc/comp/accessor.hpp:191-197).  A batch
 *    of polynomials of degree N stores element e = i*N + k.
 *  - The RNG capability is the queue's: an 8-word ChaCha20 key and a 96-bit
 *    nonce; a sampler launch uses the current nonce and then advances it by
 *    its element count (hmpc/comp/queue.hpp:175-253).  Element e's generator
 *    is ChaCha20(key, nonce, counter = low 32 bits of e).
 *
 * Every entry point returns HMPC_OK (0) or an error code and never throws;
 * hmpc_last_error() describes the last failure of the calling thread.  Work is
 * asynchronous on the context's stream; hmpc_context_synchronize() waits
 * (the reference's queue.wait(), hmpc/comp/queue.hpp:531-534).
 */
#ifndef HMPC_GB300_H
#define HMPC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HMPC_OK 0
#define HMPC_ERROR_INVALID_ARGUMENT 1
#define HMPC_ERROR_UNSUPPORTED 2
#define HMPC_ERROR_CUDA 3
#define HMPC_ERROR_OUT_OF_MEMORY 4
#define HMPC_ERROR_NO_ROOT 5
#define HMPC_ERROR_TIMEOUT 6
#define HMPC_ERROR_REJECTED 7

typedef struct hmpc_context hmpc_context;
typedef struct hmpc_modulus hmpc_modulus;

/* Description of the calling thread's last failure ("" when none). */
const char* hmpc_last_error(void);
/* Library version; returns HMPC_OK. */
int hmpc_version(int* major, int* minor);

/* --- context: device, stream and RNG capability -------------------------
 * Replaces hmpc::comp::queue's constructors (hmpc/comp/queue.hpp:229-239):
 * `key` is the 8-word ChaCha20 key (the reference draws it from
 * std::random_device when none is given); the nonce starts at 0.  `stream` is
 * a cudaStream_t (NULL: the legacy default stream). */
int hmpc_context_create(int device, const uint32_t key[8], void* stream, hmpc_context** out);
int hmpc_context_destroy(hmpc_context* ctx);
int hmpc_context_set_stream(hmpc_context* ctx, void* stream);
int hmpc_context_get_nonce(const hmpc_context* ctx, uint32_t nonce[3]);
int hmpc_context_set_nonce(hmpc_context* ctx, const uint32_t nonce[3]);
/* Number of kernels launched through this context so far (no counterpart in
 * the reference; used to report launches per timed step). */
int hmpc_context_launch_count(const hmpc_context* ctx, uint64_t* count);
/* hmpc::comp::queue::wait (hmpc/comp/queue.hpp:531-534).  Also reports
 * HMPC_ERROR_TIMEOUT when a tensor-core transform launched since the last
 * call gave up one of its bounded waits (and clears that state). */
int hmpc_context_synchronize(hmpc_context* ctx);
/* Test hook for the bounded waits of the tensor-core transform (no
 * counterpart in the reference): every wait of its group kernels gives up
 * after `polls` polls of an mbarrier (0: the default 2^20, each poll suspending
 * for at most about a microsecond); with stall != 0 the thread that issues the
 * MMAs of each launch first waits on a barrier that nothing arrives at, so
 * that wait runs out: every launch returns early with its output incomplete,
 * having waited for its copies in flight and freed its tensor memory, and
 * hmpc_context_synchronize reports HMPC_ERROR_TIMEOUT.  stall = 0 restores
 * normal operation; the context stays usable throughout. */
int hmpc_context_set_test_wait(hmpc_context* ctx, uint32_t polls, int stall);

/* --- moduli ---------------------------------------------------------------
 * mod<Q>'s compile-time constants (hmpc/ints/mod.hpp:90-127), computed at
 * run time: Q is given as q_words little-endian 32-bit words.  Supported:
 * odd Q with 2 <= bit_width(Q-1) <= 288 (1..9 limbs). */
int hmpc_modulus_create(hmpc_context* ctx, const uint32_t* q, int q_words, hmpc_modulus** out);
int hmpc_modulus_destroy(hmpc_modulus* mod);
/* limbs (L), bit_width(Q-1), and R mod Q (Montgomery one, L words, may be NULL) */
int hmpc_modulus_info(const hmpc_modulus* mod, int* limbs, int* bits, uint32_t* one);
/* Build (once) and cache on the device the forward and inverse twiddle tables
 * for ring degree n (hmpc/expr/number_theoretic_transform.hpp:35-88, the
 * reference caches them per (type, N) in the queue: comp/queue.hpp:364-381).
 * The transforms call this themselves; calling it ahead keeps the host work
 * out of a timed or captured region. */
int hmpc_modulus_prepare(hmpc_modulus* mod, uint64_t n);
/* psi (inverse = 0) or psi^-1 (inverse = 1) for degree n, Montgomery form,
 * L words (hmpc/ints/num/theory/root_of_unity.hpp:20-54). */
int hmpc_modulus_root(hmpc_modulus* mod, uint64_t n, int inverse, uint32_t* root);
/* Tile shape of the transforms of degree n over `batch` polynomials in one
 * direction: register radix bits (2 or 3: 4 or 8 elements per thread), tile
 * bits (log2 elements a CTA stages; 0 = by shared-memory budget) and column
 * bits (coalescing width) -- or radix bits 0: the tensor-core engine (exact
 * fp16 MMAs over 8-bit digits, moduli of 2 to 8 limbs below
 * 0.996 * 2^(32L); tensor, CBD(V) and forward uniform producers, the
 * uniform draws written to the output by one launch before the groups run in
 * place; other calls of that shape run the default tiles), whose local_bits
 * selects the output split (1 or 2,
 * 0 = 1) of the group with contiguous rows; or radix bits 1: one thread-block
 * cluster of 8 CTAs per polynomial holding it in distributed shared memory,
 * one launch per transform (degrees 2^10..2^14, tensor producer; other calls
 * run the default tiles).  No counterpart in the reference (its transform
 * has one schedule).  hmpc_modulus_tune times the candidates on the device
 * (scratch buffers, values irrelevant to the cost) and keeps the fastest. */
int hmpc_modulus_set_plan(hmpc_modulus* mod, uint64_t n, uint64_t batch, int inverse, int radix_bits, int local_bits,
                          int col_bits);
int hmpc_modulus_tune(hmpc_modulus* mod, uint64_t n, uint64_t batch, int inverse, float* best_ms);
/* The tile shape the transforms of (n, batch, inverse) run with: the one set
 * or tuned for them, else the default (radix bits 3, tile bits 0, column
 * bits 4). */
int hmpc_modulus_get_plan(hmpc_modulus* mod, uint64_t n, uint64_t batch, int inverse, int* radix_bits, int* local_bits,
                          int* col_bits);
/* Cost model of one tensor-core transform (no counterpart in the reference):
 * kernel launches, algorithmic DRAM bytes (digit / limb planes read and
 * written once per group, constant images read once per block) and dense
 * fp16 MMA flops, for `batch` polynomials of degree n fed by `producer_kind`
 * (HMPC_PRODUCER_TENSOR or HMPC_PRODUCER_CBD) with the output split
 * `splits` (1 or 2).  HMPC_ERROR_UNSUPPORTED when the engine does not cover
 * the modulus. */
typedef struct hmpc_tc_cost
{
    uint32_t launches;
    double bytes;
    double flops;
} hmpc_tc_cost;
int hmpc_modulus_tc_cost(hmpc_modulus* mod, uint64_t n, uint64_t batch, int inverse, int producer_kind, int splits,
                         hmpc_tc_cost* out);
/* Exactness margin of the tensor-core engine (no counterpart in the
 * reference).  A group fed by the digits of the group before it carries its
 * column sums in two float operations per digit, exact while every sum stays
 * below 2^22 - 2^15 in magnitude: with input digits of at most 128 in
 * magnitude that holds when each column of the group's constant images has a
 * sum of |digit| of at most 32512.  The engine checks this when it builds a
 * modulus's constants for (n, direction, splits) and refuses the modulus for
 * that transform if it fails (HMPC_ERROR_UNSUPPORTED; the CUDA-core tiles
 * still run it).  hmpc_modulus_tc_column_max builds the constants if needed and
 * reports their largest column sum; hmpc_context_set_tc_column_bound lowers
 * the bound applied to constants built afterwards through this context
 * (bound <= 32512), which lets a test drive the refusal. */
int hmpc_modulus_tc_column_max(hmpc_modulus* mod, uint64_t n, int inverse, int splits, uint32_t* column_max);
int hmpc_context_set_tc_column_bound(hmpc_context* ctx, uint32_t bound);
/* Copy a cached twiddle table (n*L words, element-major) to host memory. */
int hmpc_modulus_twiddles(hmpc_modulus* mod, uint64_t n, int inverse, uint32_t* host_table);

/* --- device memory helpers (optional: any device allocation works) ------ */
int hmpc_tensor_alloc(hmpc_context* ctx, uint64_t words, uint32_t** out);
int hmpc_tensor_free(hmpc_context* ctx, uint32_t* ptr);
int hmpc_tensor_upload(hmpc_context* ctx, uint32_t* dst, const uint32_t* host, uint64_t words);
int hmpc_tensor_download(hmpc_context* ctx, uint32_t* host, const uint32_t* src, uint64_t words);

/* --- transforms -------------------------------------------------------------
 * What feeds stage 0 of a forward transform.  The reference fuses the inner
 * expression of number_theoretic_transform(...) into its first kernel
 * (hmpc/expr/number_theoretic_transform.hpp:262-335): a tensor, a centred
 * binomial sampler (expr/random/binomial.hpp:176-236) or a uniform sampler
 * (expr/random/uniform.hpp:10-58).  For a sampler both inputs of a stage-0
 * butterfly come from one generator (counter = element index of the first),
 * drawn one after the other, and the launch advances the nonce by batch*n. */
#define HMPC_PRODUCER_TENSOR 0
#define HMPC_PRODUCER_CBD 1
#define HMPC_PRODUCER_UNIFORM 2
typedef struct hmpc_producer
{
    int kind;
    const uint32_t* src;    /* HMPC_PRODUCER_TENSOR: batch*n elements, limb-planar */
    uint32_t variance_x2;   /* HMPC_PRODUCER_CBD: 2V (1 for V = 1/2, 20 for V = 10), 1..64 */
    uint32_t security;      /* HMPC_PRODUCER_UNIFORM: statistical security, 80 */
} hmpc_producer;

/* number_theoretic_transform_expression (number_theoretic_transform.hpp:226-394):
 * batch polynomials of degree n (power of two, n >= 4) in natural order ->
 * bit-reversed order.  out may equal producer->src. */
int hmpc_ntt_forward(hmpc_context* ctx, hmpc_modulus* mod, uint64_t n, uint64_t batch, const hmpc_producer* producer,
                     uint32_t* out);
/* inverse_number_theoretic_transform_expression (:396-550). out may equal in. */
int hmpc_ntt_inverse(hmpc_context* ctx, hmpc_modulus* mod, uint64_t n, uint64_t batch, const uint32_t* in,
                     uint32_t* out);

/* The plain transform: one launch per stage over global memory, one thread
 * per butterfly -- the schedule of the reference's SYCL kernels
 * (number_theoretic_transform.hpp:90-197, 262-549) on this GPU; the comparator
 * the tiled passes are measured against.  Same arguments and bit-identical
 * results as hmpc_ntt_forward / hmpc_ntt_inverse. */
int hmpc_ntt_forward_plain(hmpc_context* ctx, hmpc_modulus* mod, uint64_t n, uint64_t batch,
                           const hmpc_producer* producer, uint32_t* out);
int hmpc_ntt_inverse_plain(hmpc_context* ctx, hmpc_modulus* mod, uint64_t n, uint64_t batch, const uint32_t* in,
                           uint32_t* out);

/* --- batched transforms of uneven degree -------------------------------------
 * A batch of polynomials of different degrees (powers of two >= 8), each in
 * its own limb-planar buffer, transformed from ONE captured CUDA graph.  The
 * reference runs one transform per polynomial type (the degree is a template
 * parameter, poly_mod.hpp:12-75).  Two engines:
 *  - CUDA cores: one persistent kernel launch over every polynomial; its
 *    register radix (4 or 8 elements per thread), stages per shared-memory
 *    pass and coalescing width are a tile shape;
 *  - tensor cores (moduli the tensor-core transform covers, every degree
 *    >= 16, buffers 16-byte aligned): the polynomials bucketed by degree, each
 *    bucket one tensor-core transform whose first group reads and last group
 *    writes the polynomials' own buffers through device pointer tables.
 * autotune: HMPC_BATCH_DEFAULT (the CUDA-core default tile shape),
 * HMPC_BATCH_AUTOTUNE (time every CUDA-core tile shape and the tensor-core
 * engine on the device at creation and keep the fastest) or
 * HMPC_BATCH_TENSOR_CORES (the tensor-core engine; HMPC_ERROR_UNSUPPORTED
 * when it does not cover the batch).  Same results as hmpc_ntt_forward /
 * hmpc_ntt_inverse per polynomial. */
#define HMPC_BATCH_DEFAULT 0
#define HMPC_BATCH_AUTOTUNE 1
#define HMPC_BATCH_TENSOR_CORES 2
typedef struct hmpc_ntt_batch hmpc_ntt_batch;
int hmpc_ntt_batch_create(hmpc_context* ctx, hmpc_modulus* mod, uint64_t count, const uint64_t* degrees, int inverse,
                          int autotune, hmpc_ntt_batch** out);
/* in[i] / out[i]: degrees[i]*L words each (in[i] may equal out[i]); ordered
 * on the context's stream. */
int hmpc_ntt_batch_run(hmpc_ntt_batch* batch, const uint32_t* const* in, uint32_t* const* out);
/* The engine and tile shape the batch runs with (radix_bits 0: the
 * tensor-core engine, local_bits its split), the CUDA-core kernel's work
 * items or the tensor-core graph's kernel launches, and the tuned time. */
int hmpc_ntt_batch_info(const hmpc_ntt_batch* batch, int* radix_bits, int* local_bits, int* col_bits, uint32_t* items,
                        float* tuned_ms);
/* After a run: waits for it and reports whether every work item finished
 * (HMPC_ERROR_TIMEOUT and the 1-based failing item when a bounded wait ran
 * out). */
int hmpc_ntt_batch_status(hmpc_ntt_batch* batch, uint32_t* failed_item);
/* Test hook for the bounded waits (no counterpart in the reference): a
 * later-pass work item waits at most `polls` polls of about 64 ns (0: the
 * default, about a second) for the earlier passes of its polynomial; with
 * withheld_item != 0 that work item (1-based; it must belong to the last pass,
 * after the first, of its polynomial) waits for one signal more than the
 * earlier passes give, so its wait runs out: the run leaves that polynomial's
 * output incomplete and hmpc_ntt_batch_status reports HMPC_ERROR_TIMEOUT with
 * the item.  withheld_item = 0 restores the work list. */
int hmpc_ntt_batch_set_test_wait(hmpc_ntt_batch* batch, uint32_t polls, uint32_t withheld_item);
int hmpc_ntt_batch_destroy(hmpc_ntt_batch* batch);

/* --- elementwise ----------------------------------------------------------- */
/* d = a*b + c (examples/fma.cpp:56-67) */
int hmpc_fma(hmpc_context* ctx, hmpc_modulus* mod, uint64_t elements, const uint32_t* a, const uint32_t* b,
             const uint32_t* c, uint32_t* d);
#define HMPC_OP_ADD 0
#define HMPC_OP_SUB 1
#define HMPC_OP_MUL 2
/* out[e] = a[e % a_elements] OP b[e % b_elements]: the binary expressions of
 * hmpc/expr/binary_expression.hpp:149-163 with broadcasting of an unsqueezed
 * operand (hmpc/expr/unsqueeze.hpp:9-61).  a_elements and b_elements must
 * divide elements. */
int hmpc_binary(hmpc_context* ctx, hmpc_modulus* mod, int op, uint64_t elements, const uint32_t* a,
                uint64_t a_elements, const uint32_t* b, uint64_t b_elements, uint32_t* out);
/* uniform<mod<Q>>(shape) evaluated elementwise (expr/random/uniform.hpp:11-46);
 * advances the nonce by elements. security must be 80. */
int hmpc_sample_uniform(hmpc_context* ctx, hmpc_modulus* mod, uint64_t elements, uint32_t security, uint32_t* out);
/* centered_binomial<mod<Q>>(shape, V) (expr/random/binomial.hpp:176-236), 2V = variance_x2 */
int hmpc_sample_cbd(hmpc_context* ctx, hmpc_modulus* mod, uint64_t elements, uint32_t variance_x2, uint32_t* out);
/* cast<mod<dst>>(x) of residues mod src: the centred lift of
 * hmpc/ints/mod.hpp:259-307 (expr/cast.hpp:10-53). */
int hmpc_cast(hmpc_context* ctx, hmpc_modulus* dst, hmpc_modulus* src, uint64_t elements, const uint32_t* in,
              uint32_t* out);
/* canonical integers in [0, Q) <-> Montgomery representatives
 * (mod.hpp:197-204 and :356-361) */
int hmpc_to_montgomery(hmpc_context* ctx, hmpc_modulus* mod, uint64_t elements, const uint32_t* in, uint32_t* out);
int hmpc_from_montgomery(hmpc_context* ctx, hmpc_modulus* mod, uint64_t elements, const uint32_t* in, uint32_t* out);

/* --- matrix-vector products and reductions ------------------------------------
 * The consumers of NTT-form data after the transform.  All tensors are
 * limb-planar and row-major. */
/* z[b][i][c] = sum_k m[b][i][k][c] * x[b][k][c] mod Q for b < batch, i < rows,
 * k < cols, c < coeffs: hmpc::expr::matrix_vector_product of mod<Q> tensors
 * (hmpc/expr/matrix_vector_product.hpp:88-140).  coeffs is 1 for a matrix of
 * residues, or the degree for NTT-form polynomials, whose ring product is
 * elementwise.  m holds m_batch matrices of rows x cols x coeffs elements and
 * x holds x_batch vectors of cols x coeffs elements; each of m_batch and
 * x_batch is batch or 1 (broadcast: the common_extent of
 * matrix_vector_product.hpp:7-23).  z holds batch x rows x coeffs elements. */
int hmpc_matvec(hmpc_context* ctx, hmpc_modulus* mod, uint64_t batch, uint64_t rows, uint64_t cols, uint64_t coeffs,
                const uint32_t* m, uint64_t m_batch, const uint32_t* x, uint64_t x_batch, uint32_t* z);
/* z[b][i] = sum_k X^degrees[b][i][k] * x[b][k] in Z_Q[X]/(X^n + 1) for
 * polynomials of degree n (a power of two) in coefficient form: a matrix of
 * hmpc::expr::bit_monomial<n> times polynomials (hmpc/expr/bit_monomial.hpp:
 * 18-104 inside matrix_vector_product.hpp:88-140).  degrees is a device array
 * of d_batch x rows x cols int64 values; a negative degree stands for
 * std::nullopt (no monomial); a degree d acts as X^(d mod 2n).  x holds
 * x_batch x cols polynomials, z batch x rows polynomials. */
int hmpc_matvec_monomial(hmpc_context* ctx, hmpc_modulus* mod, uint64_t n, uint64_t batch, uint64_t rows,
                         uint64_t cols, const int64_t* degrees, uint64_t d_batch, const uint32_t* x,
                         uint64_t x_batch, uint32_t* z);
#define HMPC_REDUCE_ADD 0
#define HMPC_REDUCE_MULTIPLY 1
#define HMPC_REDUCE_BIT_AND 2
#define HMPC_REDUCE_BIT_OR 3
#define HMPC_REDUCE_BIT_XOR 4
#define HMPC_REDUCE_MIN 5
#define HMPC_REDUCE_MAX 6
/* out (device, L words) = the sum or product of every residue of in:
 * hmpc::expr::sum / product of a mod<Q> tensor (hmpc/expr/reduce.hpp:206-277);
 * op is HMPC_REDUCE_ADD or HMPC_REDUCE_MULTIPLY.  An empty tensor gives the
 * identity (0, or the Montgomery form of 1). */
int hmpc_reduce(hmpc_context* ctx, hmpc_modulus* mod, int op, uint64_t elements, const uint32_t* in, uint32_t* out);
/* The same over uint<bits> values in ceil(bits / 32) limb planes (bits <= 288):
 * every HMPC_REDUCE_* operation of hmpc::reduction (reduce.hpp:8-53); sums and
 * products keep their low `bits` bits, as a uint<bits> accumulator does, and
 * the identities are ints/integer_traits.hpp:39-46.  On one-bit values
 * BIT_AND and BIT_OR are hmpc::expr::all and any. */
int hmpc_reduce_uint(hmpc_context* ctx, int op, int bits, uint64_t elements, const uint32_t* in, uint32_t* out);
/* out[e] = 1 if a[e] == b[e] in every limb, else 0: the hmpc::bit tensor of
 * x == y (hmpc/expr/binary_expression.hpp) that all / any reduce. */
int hmpc_equal(hmpc_context* ctx, int limbs, uint64_t elements, const uint32_t* a, const uint32_t* b, uint32_t* out);

/* --- linear BGV (hmpc/expr/crypto/lhe) ---------------------------------------
 * Keys and ciphertext components are polynomials of degree n mod q in NTT
 * representation; plaintexts are mod p (coefficient representation, or NTT
 * when plaintext_ntt != 0). */
/* enc (expr/crypto/lhe/enc.hpp:19-69) with randomness<Rq>(shape{batch})
 * (randomness.hpp:196-226): c0 = a*u + v*p + NTT_q(lift(m)), c1 = b*u + w*p
 * with u = NTT(CBD(1/2)), v, w = NTT(CBD(10)).  Nonce order of the reference's
 * execution plan: u, v, w each advance the nonce by batch*n. */
int hmpc_lhe_enc(hmpc_context* ctx, hmpc_modulus* q, hmpc_modulus* p, uint64_t n, uint64_t batch,
                 const uint32_t* key_a, const uint32_t* key_b, const uint32_t* plaintext, int plaintext_ntt,
                 uint32_t* c0, uint32_t* c1);
/* hmpc_lhe_enc without any device allocation.  No counterpart in the
 * reference.  For callers that cannot allocate device memory: a serving
 * process whose memory is reserved up front by its own pool, or a
 * latency-critical loop that must not pay the device-wide synchronisation that
 * cudaMalloc/cudaFree can cause.  Same arguments and bit-identical results as
 * hmpc_lhe_enc; the intermediates live in one fixed 32 MiB array of device
 * memory in this library (held by every GPU that loads it until exit), so
 * 3*batch*n*L_q (+ batch*n*L_p for NTT-form plaintexts) must not exceed
 * 8 Mi words -- larger batches are rejected with HMPC_ERROR_INVALID_ARGUMENT.
 * The twiddle tables must already exist (hmpc_modulus_prepare) -- the call
 * refuses to build them.  Its transforms run on the CUDA-core tiles whatever
 * plan q has (the tensor-core engine allocates digit buffers and constant
 * images of its own), so it is slower than hmpc_lhe_enc where q's plan is the
 * tensor-core engine; the ciphertexts are the same bits either way.  The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress); make that first call before any
 * stream capture.  All calls on a device share the array: calls that overlap
 * on the GPU (other streams, other contexts) race and must be serialised by
 * the caller. */
int hmpc_lhe_enc_noalloc(hmpc_context* ctx, hmpc_modulus* q, hmpc_modulus* p, uint64_t n, uint64_t batch,
                         const uint32_t* key_a, const uint32_t* key_b, const uint32_t* plaintext, int plaintext_ntt,
                         uint32_t* c0, uint32_t* c1);
/* dec<Plaintext>(s, ct) (expr/crypto/lhe/dec.hpp:13-45): c0 - s*c1 -> INTT_q
 * -> cast to p (-> NTT_p when plaintext_ntt). */
int hmpc_lhe_dec(hmpc_context* ctx, hmpc_modulus* q, hmpc_modulus* p, uint64_t n, uint64_t batch,
                 const uint32_t* s, const uint32_t* c0, const uint32_t* c1, int plaintext_ntt, uint32_t* out);
/* Decryption of a degree-2 ciphertext (c0, c1, c2), the result of
 * hmpc_lhe_ct_mul: c0 - s*c1 + s^2*c2 -> INTT_q -> cast to p (-> NTT_p).  No
 * counterpart in the reference. */
int hmpc_lhe_dec2(hmpc_context* ctx, hmpc_modulus* q, hmpc_modulus* p, uint64_t n, uint64_t batch,
                  const uint32_t* s, const uint32_t* c0, const uint32_t* c1, const uint32_t* c2, int plaintext_ntt,
                  uint32_t* out);
/* Ciphertext x ciphertext in NTT form: the tensor product
 * (d0, d1, d2) = (a0*b0, a0*b1 + a1*b0, a1*b1) over `elements` residues.  No
 * counterpart in the reference, whose ciphertexts are linear only
 * (expr/crypto/lhe/ciphertext.hpp:49-81). */
int hmpc_lhe_ct_mul(hmpc_context* ctx, hmpc_modulus* q, uint64_t elements, const uint32_t* a0, const uint32_t* a1,
                    const uint32_t* b0, const uint32_t* b1, uint32_t* d0, uint32_t* d1, uint32_t* d2);
/* Key generation; no counterpart in the reference, whose keys are plain
 * tensors (comp/crypto/lhe/key.hpp:7-12).  b <- uniform mod q (NTT form),
 * s <- NTT(CBD(1/2)), e <- NTT(CBD(10)), a = b*s + p*e, so that
 * dec(s, enc((a, b), m)) = m.  Nonce order: b, s, e (n each). */
int hmpc_lhe_keygen(hmpc_context* ctx, hmpc_modulus* q, hmpc_modulus* p, uint64_t n, uint32_t* s, uint32_t* a,
                    uint32_t* b);

/* --- stream cipher -----------------------------------------------------------
 * enc(cipher(key, nonce), x) / dec<T>(cipher(key, nonce), y) of
 * hmpc/expr/crypto/cipher.hpp:59-319: element i's `limbs` words are XORed with
 * keystream words i*limbs .. i*limbs+limbs-1 of ChaCha20(key, nonce, counter
 * from 0).  enc reads a limb-planar tensor and writes the reference's
 * element-major limb tensor (flat_out[i*limbs + j]); dec is the reverse.
 * Independent of the context's RNG capability (explicit key and nonce). */
int hmpc_cipher_enc(hmpc_context* ctx, const uint32_t key[8], const uint32_t nonce[3], uint64_t elements, int limbs,
                    const uint32_t* planar_in, uint32_t* flat_out);
int hmpc_cipher_dec(hmpc_context* ctx, const uint32_t key[8], const uint32_t nonce[3], uint64_t elements, int limbs,
                    const uint32_t* flat_in, uint32_t* planar_out);

/* --- serving ---------------------------------------------------------------
 * A request loop with continuous batching (no counterpart in the reference).
 * Clients submit requests from any thread and get a ticket; a scheduler
 * thread groups compatible pending requests (same kind, modulus, degree and
 * key) into one dispatch per free lane (a device stream), so requests that
 * arrive while others run are admitted as lanes and memory free up and their
 * work overlaps on the device.  Scratch comes from a device pool reserved at
 * creation (memory_budget_bytes): a dispatch waits until its scratch fits, a
 * request that cannot fit even alone is rejected (HMPC_ERROR_REJECTED).  Keys
 * and twiddle tables stay resident.  A request's result equals the result it
 * has alone: an encryption draws its randomness from its own nonce with
 * coefficient indices local to the request, exactly as hmpc_lhe_enc on a
 * context whose nonce is the request's nonce. */
typedef struct hmpc_server hmpc_server;
typedef struct hmpc_server_config
{
    uint64_t memory_budget_bytes;    /* device pool for dispatch scratch */
    uint32_t lanes;                  /* device streams, one dispatch each */
    uint32_t max_batch;              /* requests per dispatch (1: no batching) */
    uint32_t max_batch_polynomials;  /* polynomials per dispatch (0: 4096) */
    uint32_t batch_window_us;        /* hold a group smaller than max_batch until its oldest request has */
                                     /* waited this long, so compatible arrivals join it (0: at once) */
} hmpc_server_config;

#define HMPC_REQUEST_NTT 0       /* out0 = NTT(in0): count polynomials of degree n mod q */
#define HMPC_REQUEST_ENCRYPT 1   /* (out0, out1) = enc(key, in0): count plaintexts mod p, own nonce */
#define HMPC_REQUEST_CT_MUL 2    /* (out0, out1, out2) = (in0, in1) x (in2, in3), count ciphertexts */
typedef struct hmpc_request
{
    int kind;
    uint32_t key_id;             /* HMPC_REQUEST_ENCRYPT: from hmpc_server_add_key */
    hmpc_modulus* q;             /* NTT / CT_MUL modulus (ENCRYPT: the key's) */
    uint64_t n;                  /* ring degree */
    uint64_t count;              /* polynomials / plaintexts / ciphertexts */
    const uint32_t* in0;
    const uint32_t* in1;
    const uint32_t* in2;
    const uint32_t* in3;
    uint32_t* out0;
    uint32_t* out1;
    uint32_t* out2;
    uint32_t nonce[3];           /* HMPC_REQUEST_ENCRYPT: the request's RNG nonce */
} hmpc_request;

#define HMPC_REQUEST_QUEUED 0
#define HMPC_REQUEST_RUNNING 1
#define HMPC_REQUEST_DONE 2
#define HMPC_REQUEST_FAILED (-2)

typedef struct hmpc_server_stats
{
    uint64_t submitted, completed, rejected, failed, dispatches, launches;
    double mean_batch;           /* requests per dispatch */
    double p50_us, p99_us, mean_us;  /* submit -> completion observed, completed requests */
} hmpc_server_stats;

int hmpc_server_create(hmpc_context* ctx, const hmpc_server_config* config, hmpc_server** out);
/* keep a public key (a, b: n words x L each, device memory) resident; the
 * server copies it */
int hmpc_server_add_key(hmpc_server* server, hmpc_modulus* q, hmpc_modulus* p, uint64_t n, const uint32_t* a,
                        const uint32_t* b, uint32_t* key_id);
/* non-blocking; the buffers must stay valid until the request is done */
int hmpc_server_submit(hmpc_server* server, const hmpc_request* request, uint64_t* ticket);
/* state: HMPC_REQUEST_*; latency_us (may be NULL): submit -> completion */
int hmpc_server_poll(hmpc_server* server, uint64_t ticket, int* state, double* latency_us);
/* wait until every submitted request has finished */
int hmpc_server_drain(hmpc_server* server, uint32_t timeout_ms);
int hmpc_server_get_stats(hmpc_server* server, hmpc_server_stats* out);
int hmpc_server_destroy(hmpc_server* server);

/* ------------------------------------------------------------------ wire
 * Messages of hmpc's network layer (hmpc-rs/src/net.rs:205-400,
 * docs/networking.md "Message Format", format version 0), packed and unpacked
 * on the device; the payload of a tensor is its limb-planar storage
 * (hmpc/net/queue.hpp:60-88).  No counterpart in the reference's device code:
 * it serialises on the host from a host accessor.  Header, little-endian:
 * version u8 = 0, feature flags u8 (bit 0 sessions: a 16-byte session id
 * follows the header; bit 1 signing: not supported), kind u8 (send 1 ..
 * all-to-all 6, consistency checks | 0x10), datatype u8 (bit width | 1 for
 * little-endian: 0x21 for 32-bit limbs), sender u16, receiver u16, message id
 * u64. */
#define HMPC_WIRE_SEND 1
#define HMPC_WIRE_BROADCAST 2
#define HMPC_WIRE_SCATTER 3
#define HMPC_WIRE_GATHER 4
#define HMPC_WIRE_ALL_GATHER 5
#define HMPC_WIRE_ALL_TO_ALL 6
#define HMPC_WIRE_FLAG_SESSIONS 1
#define HMPC_WIRE_FLAG_SIGNING 2
#define HMPC_WIRE_DATATYPE_U32 0x21

typedef struct hmpc_wire_message
{
    uint8_t kind;
    uint8_t datatype;
    uint16_t sender;
    uint16_t receiver;
    uint64_t id;
    const void* payload;   /* device memory (pack: read; unpack: ignored) */
    uint64_t bytes;        /* payload bytes */
    uint32_t planes;       /* 0 or 1: contiguous; else the payload is `planes` equal parts of a */
    uint64_t plane_stride; /* multiple of 16 bytes, plane_stride bytes apart in the tensor (one */
                           /* polynomial's limb planes inside a batch tensor; unpack: the destination) */
} hmpc_wire_message;

/* Byte offset of each message in a packed buffer (slots start on 16-byte
 * boundaries, header + payload) and the buffer's size. */
int hmpc_wire_layout(const hmpc_wire_message* messages, uint64_t count, uint8_t flags, uint64_t* offsets,
                     uint64_t* total_bytes);
/* Write `count` messages (header + payload) into device buffer `out` at
 * `offsets` in one launch on the context's stream. */
int hmpc_wire_pack(hmpc_context* ctx, const hmpc_wire_message* messages, uint64_t count, uint8_t flags,
                   const uint8_t session[16], const uint64_t* offsets, uint8_t* out);
/* Check each received message (device buffer `in`, message i at offsets[i],
 * sizes[i] bytes) against `expected` (kind, datatype, sender, receiver, id,
 * payload bytes; version 0, `flags`, the session id) and copy the payloads of
 * those that match into payloads[i] (device).  status (device, one word per
 * message) receives 0 or the first mismatching field: 1 version, 2 flags,
 * 3 kind, 4 datatype, 5 sender, 6 receiver, 7 id, 8 session, 9 size.
 * Returns when the copies are complete. */
int hmpc_wire_unpack(hmpc_context* ctx, const uint8_t* in, const uint64_t* offsets, const uint64_t* sizes,
                     uint64_t count, uint8_t flags, const uint8_t session[16], const hmpc_wire_message* expected,
                     void* const* payloads, uint32_t* status);
/* Message id of an operation (hmpc-rs/src/net/queue.rs:108-135): the first
 * eight bytes, little-endian, of SHA-256(senders || kind || datatype ||
 * member || receivers) plus `counter` (1 for the first operation with that
 * hash, then 2, ...); a communicator hashes as its size (u64) and its distinct
 * party ids (u16) ascending; `member` is the sender (broadcast) or receiver
 * (gather), none (members = 0) for all-gather and all-to-all. */
int hmpc_wire_message_id(uint8_t kind, uint8_t datatype, const uint16_t* member, int members,
                         const uint16_t* senders, int sender_count, const uint16_t* receivers, int receiver_count,
                         uint64_t counter, uint64_t* id);
/* SHA-256 of host bytes (FIPS 180-4), as the message id and the signing
 * feature's payload hash use it. */
int hmpc_wire_sha256(const void* data, uint64_t bytes, uint8_t digest[32]);

#ifdef __cplusplus
}
#endif

#endif
