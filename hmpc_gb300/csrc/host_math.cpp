#include "host_math.hpp"

#include <algorithm>

namespace hmpc_gb300::host
{
    words resize(words a, int n)
    {
        a.resize(static_cast<size_t>(n), 0u);
        return a;
    }

    static void trim(words& a)
    {
        while (a.size() > 1 && a.back() == 0u)
        {
            a.pop_back();
        }
    }

    int bit_width(const words& a)
    {
        for (int i = static_cast<int>(a.size()) - 1; i >= 0; --i)
        {
            if (a[static_cast<size_t>(i)])
            {
                return 32 * i + (32 - __builtin_clz(a[static_cast<size_t>(i)]));
            }
        }
        return 0;
    }

    int compare(const words& a, const words& b)
    {
        const size_t n = std::max(a.size(), b.size());
        for (size_t k = n; k-- > 0;)
        {
            const uint32_t x = k < a.size() ? a[k] : 0u;
            const uint32_t y = k < b.size() ? b[k] : 0u;
            if (x != y)
            {
                return x > y ? 1 : -1;
            }
        }
        return 0;
    }

    words add(const words& a, const words& b, int n)
    {
        words r(static_cast<size_t>(n));
        uint64_t carry = 0;
        for (size_t i = 0; i < r.size(); ++i)
        {
            const uint64_t s = static_cast<uint64_t>(i < a.size() ? a[i] : 0u) + (i < b.size() ? b[i] : 0u) + carry;
            r[i] = static_cast<uint32_t>(s);
            carry = s >> 32;
        }
        return r;
    }

    words sub(const words& a, const words& b, int n)
    {
        words r(static_cast<size_t>(n));
        uint64_t borrow = 0;
        for (size_t i = 0; i < r.size(); ++i)
        {
            const uint64_t d = static_cast<uint64_t>(i < a.size() ? a[i] : 0u) - (i < b.size() ? b[i] : 0u) - borrow;
            r[i] = static_cast<uint32_t>(d);
            borrow = (d >> 63) & 1u;
        }
        return r;
    }

    words mul(const words& a, const words& b)
    {
        words r(a.size() + b.size(), 0u);
        for (size_t i = 0; i < b.size(); ++i)
        {
            uint64_t carry = 0;
            for (size_t j = 0; j < a.size(); ++j)
            {
                const uint64_t t = static_cast<uint64_t>(a[j]) * b[i] + r[i + j] + carry;
                r[i + j] = static_cast<uint32_t>(t);
                carry = t >> 32;
            }
            r[i + a.size()] = static_cast<uint32_t>(carry);
        }
        return r;
    }

    words mod(const words& a, const words& q)
    {
        const int nq = static_cast<int>(q.size());
        words r(static_cast<size_t>(nq + 1), 0u);
        const words qq = resize(q, nq + 1);
        for (int bit = 32 * static_cast<int>(a.size()) - 1; bit >= 0; --bit)
        {
            uint32_t top = (a[static_cast<size_t>(bit / 32)] >> (bit % 32)) & 1u;
            for (auto& w : r)
            {
                const uint32_t next = w >> 31;
                w = (w << 1) | top;
                top = next;
            }
            if (compare(r, qq) >= 0)
            {
                r = sub(r, qq, nq + 1);
            }
        }
        return resize(r, nq);
    }

    bool make_constants(const words& q_in, ModulusConstants& m, std::string& error)
    {
        words q = q_in;
        trim(q);
        if (bit_width(q) < 2 || (q[0] & 1u) == 0u)
        {
            error = "modulus must be odd and at least 3";
            return false;
        }
        const words qm1 = sub(q, words{1u}, static_cast<int>(q.size()));
        m.bits = bit_width(qm1);
        m.limbs = (m.bits + 31) / 32;
        if (m.limbs > max_limbs)
        {
            error = "modulus wider than 512 bits";
            return false;
        }
        const int L = m.limbs;
        m.q = resize(q, L);
        m.half.assign(static_cast<size_t>(L), 0u);
        for (int i = 0; i < L; ++i)
        {
            m.half[static_cast<size_t>(i)] =
                (m.q[static_cast<size_t>(i)] >> 1) | (i + 1 < L ? (m.q[static_cast<size_t>(i + 1)] << 31) : 0u);
        }
        uint32_t inv = 1u;
        for (int i = 0; i < 6; ++i)
        {
            inv *= 2u - m.q[0] * inv;
        }
        m.ninv = 0u - inv;
        words R(static_cast<size_t>(L + 1), 0u);
        R[static_cast<size_t>(L)] = 1u;
        m.one = mod(R, m.q);
        words R2(static_cast<size_t>(2 * L + 1), 0u);
        R2[static_cast<size_t>(2 * L)] = 1u;
        m.r2 = mod(R2, m.q);
        return true;
    }

    words mont_mul(const ModulusConstants& m, const words& a, const words& b)
    {
        const int L = m.limbs;
        words t(static_cast<size_t>(L + 2), 0u);
        for (int i = 0; i < L; ++i)
        {
            uint64_t carry = 0;
            const uint64_t bi = b[static_cast<size_t>(i)];
            for (int j = 0; j < L; ++j)
            {
                const uint64_t s = a[static_cast<size_t>(j)] * bi + t[static_cast<size_t>(j)] + carry;
                t[static_cast<size_t>(j)] = static_cast<uint32_t>(s);
                carry = s >> 32;
            }
            uint64_t s = static_cast<uint64_t>(t[static_cast<size_t>(L)]) + carry;
            t[static_cast<size_t>(L)] = static_cast<uint32_t>(s);
            t[static_cast<size_t>(L + 1)] = static_cast<uint32_t>(s >> 32);
            const uint64_t mq = static_cast<uint32_t>(t[0] * m.ninv);
            carry = (mq * m.q[0] + t[0]) >> 32;
            for (int j = 1; j < L; ++j)
            {
                const uint64_t u = mq * m.q[static_cast<size_t>(j)] + t[static_cast<size_t>(j)] + carry;
                t[static_cast<size_t>(j - 1)] = static_cast<uint32_t>(u);
                carry = u >> 32;
            }
            s = static_cast<uint64_t>(t[static_cast<size_t>(L)]) + carry;
            t[static_cast<size_t>(L - 1)] = static_cast<uint32_t>(s);
            t[static_cast<size_t>(L)] = t[static_cast<size_t>(L + 1)] + static_cast<uint32_t>(s >> 32);
            t[static_cast<size_t>(L + 1)] = 0u;
        }
        words r = resize(t, L + 1);
        if (compare(r, m.q) >= 0)
        {
            r = sub(r, m.q, L + 1);
        }
        return resize(r, L);
    }

    words mont_pow(const ModulusConstants& m, const words& x, const words& e)
    {
        words result = m.one;
        words v = x;
        const int bits = bit_width(e);
        for (int i = 0; i < bits; ++i)
        {
            if ((e[static_cast<size_t>(i / 32)] >> (i % 32)) & 1u)
            {
                result = mont_mul(m, result, v);
            }
            v = mont_mul(m, v, v);
        }
        return result;
    }

    words to_mont(const ModulusConstants& m, const words& v)
    {
        return mont_mul(m, mod(v.empty() ? words{0u} : v, m.q), m.r2);
    }

    words from_mont(const ModulusConstants& m, const words& x)
    {
        words one(static_cast<size_t>(m.limbs), 0u);
        one[0] = 1u;
        return mont_mul(m, x, one);
    }

    words invert(const ModulusConstants& m, const words& x)
    {
        return mont_pow(m, x, sub(m.q, words{2u}, m.limbs));
    }

    static uint32_t rotl(uint32_t v, int c)
    {
        return (v << c) | (v >> (32 - c));
    }

    static void quarter(uint32_t& a, uint32_t& b, uint32_t& c, uint32_t& d)
    {
        a += b;
        d = rotl(d ^ a, 16);
        c += d;
        b = rotl(b ^ c, 12);
        a += b;
        d = rotl(d ^ a, 8);
        c += d;
        b = rotl(b ^ c, 7);
    }

    void chacha20_block(const uint32_t key[8], uint32_t counter, const uint32_t nonce[3], uint32_t out[16])
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
        std::copy(s, s + 16, x);
        for (int r = 0; r < 10; ++r)
        {
            quarter(x[0], x[4], x[8], x[12]);
            quarter(x[1], x[5], x[9], x[13]);
            quarter(x[2], x[6], x[10], x[14]);
            quarter(x[3], x[7], x[11], x[15]);
            quarter(x[0], x[5], x[10], x[15]);
            quarter(x[1], x[6], x[11], x[12]);
            quarter(x[2], x[7], x[8], x[13]);
            quarter(x[3], x[4], x[9], x[14]);
        }
        for (int i = 0; i < 16; ++i)
        {
            out[i] = x[i] + s[i];
        }
    }

    bool root_of_unity(const ModulusConstants& m, uint64_t degree, words& root, std::string& error)
    {
        const int L = m.limbs;
        if (degree < 2 || (degree & (degree - 1)) != 0)
        {
            error = "root degree must be a power of two";
            return false;
        }
        words qm1 = sub(m.q, words{1u}, L);
        words exponent = qm1;
        const int shift = __builtin_ctzll(degree);
        for (int i = 0; i < shift; ++i)
        {
            if (exponent[0] & 1u)
            {
                error = "Q - 1 is not divisible by the root degree (Q is not NTT friendly for this N)";
                return false;
            }
            for (int j = 0; j < L; ++j)
            {
                exponent[static_cast<size_t>(j)] =
                    (exponent[static_cast<size_t>(j)] >> 1) |
                    (j + 1 < L ? (exponent[static_cast<size_t>(j + 1)] << 31) : 0u);
            }
        }
        const words half_degree{static_cast<uint32_t>(degree / 2), static_cast<uint32_t>((degree / 2) >> 32)};
        const words full_degree{static_cast<uint32_t>(degree), static_cast<uint32_t>(degree >> 32)};
        // the candidate stream: ChaCha20 with zero key, nonce and counter,
        // L words per candidate, top limb masked to bit_width(Q-1) bits
        const uint32_t zero_key[8] = {};
        const uint32_t zero_nonce[3] = {};
        uint32_t block[16];
        uint32_t counter = 0;
        int index = 16;
        for (long attempt = 0; attempt < 100000; ++attempt)
        {
            words x(static_cast<size_t>(L));
            for (int j = 0; j < L; ++j)
            {
                if (index == 16)
                {
                    chacha20_block(zero_key, counter++, zero_nonce, block);
                    index = 0;
                }
                x[static_cast<size_t>(j)] = block[index++];
            }
            if (m.bits % 32)
            {
                x[static_cast<size_t>(L - 1)] &= (1u << (m.bits % 32)) - 1u;
            }
            if (compare(x, qm1) > 0)
            {
                x = sub(x, m.q, L);
            }
            if (bit_width(x) == 0)
            {
                continue;
            }
            const words g = mont_pow(m, x, exponent);
            if (compare(mont_pow(m, g, half_degree), m.one) != 0 && compare(mont_pow(m, g, full_degree), m.one) == 0)
            {
                root = g;
                return true;
            }
        }
        error = "no root of unity found (is Q prime?)";
        return false;
    }

    static uint32_t bit_reverse(uint32_t v, int bits)
    {
        uint32_t r = 0u;
        for (int i = 0; i < bits; ++i)
        {
            r |= ((v >> i) & 1u) << (bits - 1 - i);
        }
        return r;
    }

    bool twiddle_table(const ModulusConstants& m, uint64_t n, bool inverse, std::vector<uint32_t>& table,
                       words& root_out, std::string& error)
    {
        const int L = m.limbs;
        if (n < 4 || (n & (n - 1)) != 0 || n > (1ull << 30))
        {
            error = "ring degree must be a power of two in [4, 2^30]";
            return false;
        }
        const int bits = __builtin_ctzll(n);
        words root;
        if (!root_of_unity(m, 2 * n, root, error))
        {
            return false;
        }
        if (inverse)
        {
            root = invert(m, root);
        }
        root_out = root;
        const words normalization = invert(m, to_mont(m, words{static_cast<uint32_t>(n)}));
        table.assign(static_cast<size_t>(n) * static_cast<size_t>(L), 0u);
        auto put = [&](uint64_t j, const words& v) {
            std::copy(v.begin(), v.begin() + L, table.begin() + static_cast<std::ptrdiff_t>(j * static_cast<uint64_t>(L)));
        };
        put(0, inverse ? normalization : m.one);
        put(bit_reverse(1, bits), root);
        words power = root;
        for (uint64_t i = 2; i < n; ++i)
        {
            power = mont_mul(m, power, root);
            const uint32_t j = bit_reverse(static_cast<uint32_t>(i), bits);
            put(j, (inverse && j == 1) ? mont_mul(m, power, normalization) : power);
        }
        return true;
    }
}
