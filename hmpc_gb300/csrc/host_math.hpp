// Host-side precomputation for a registered modulus: Montgomery constants,
// the primitive 2N-th root of unity, twiddle tables and cast constants.
// Runs once per (modulus, degree) and caches on the device, the way hmpc's
// queue caches its root tables (hmpc/comp/queue.hpp:364-381).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace hmpc_gb300::host
{
    using words = std::vector<uint32_t>;

    constexpr int max_limbs = 16;

    int bit_width(const words& a);
    int compare(const words& a, const words& b);           // over max(size)
    words add(const words& a, const words& b, int n);      // (a + b) mod 2^(32n)
    words sub(const words& a, const words& b, int n);      // (a - b) mod 2^(32n)
    words mul(const words& a, const words& b);              // full product
    words mod(const words& a, const words& q);              // a mod q
    words resize(words a, int n);

    struct ModulusConstants
    {
        int limbs = 0;
        int bits = 0;
        uint32_t ninv = 0;
        words q, half, one, r2;
    };

    // Returns false when Q is even, below 3 or wider than max_limbs words.
    bool make_constants(const words& q, ModulusConstants& out, std::string& error);

    words mont_mul(const ModulusConstants& m, const words& a, const words& b);
    words mont_pow(const ModulusConstants& m, const words& x, const words& e);
    words to_mont(const ModulusConstants& m, const words& v);  // any width
    words from_mont(const ModulusConstants& m, const words& x);
    words invert(const ModulusConstants& m, const words& x);   // Fermat, Q prime

    void chacha20_block(const uint32_t key[8], uint32_t counter, const uint32_t nonce[3], uint32_t out[16]);

    // primitive `degree`-th root of unity in Montgomery form
    // (hmpc/ints/num/theory/root_of_unity.hpp:20-54)
    bool root_of_unity(const ModulusConstants& m, uint64_t degree, words& root, std::string& error);

    // element-major table [n][L] (hmpc/expr/number_theoretic_transform.hpp:35-88)
    bool twiddle_table(const ModulusConstants& m, uint64_t n, bool inverse, std::vector<uint32_t>& table,
                       words& root, std::string& error);
}
