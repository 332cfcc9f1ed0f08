// Exercises the C++ front end (include/hmpc_gb300/hmpc.hpp) the way hmpc code
// uses hmpc::comp::queue: lazy expressions evaluated in the reference's plan
// order.  Writes the results as raw little-endian words for the Python test
// to compare against the oracle; checks the BGV round trip itself.
#include <cstdio>
#include <fstream>
#include <vector>

#include "hmpc_gb300/hmpc.hpp"

static void dump(const char* dir, const char* name, const std::vector<uint32_t>& w)
{
    std::string path = std::string(dir) + "/" + name;
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char*>(w.data()), static_cast<std::streamsize>(w.size() * 4));
}

int main(int argc, char** argv)
{
    const char* dir = argc > 1 ? argv[1] : ".";
    using namespace hmpc::expr::operators;
    namespace expr = hmpc::expr;
    // q 256-bit and p 64-bit, little-endian words
    const std::vector<uint32_t> q_words = {0x56740001u, 0x85f3a1f1u, 0x0b577d27u, 0x53e20d92u,
                                           0xd7ae005du, 0xaf55bca0u, 0xb12ccf05u, 0xcff479b9u};
    const std::vector<uint32_t> p_words = {0x23320001u, 0x8822d806u};
    const uint64_t n = 1024, batch = 3;

    hmpc::comp::queue queue({1, 2, 3, 4, 5, 6, 7, 8});
    auto& q = queue.modulus(q_words);
    auto& p = queue.modulus(p_words);

    // a tensor of raw representatives below q (x_i = i + 1 in the low limb)
    auto x = hmpc::comp::make_tensor(queue, q, {batch}, n);
    std::vector<uint32_t> host(x.words(), 0u);
    for (uint64_t e = 0; e < batch * n; ++e)
    {
        host[e] = static_cast<uint32_t>(e + 1);
    }
    x.upload(host);
    auto y = queue(expr::number_theoretic_transform(expr::tensor(x)));
    dump(dir, "ntt.bin", y.download());

    // two sampled transforms in one queue call: nonces 0 and batch*n
    auto [u, v] = queue(expr::number_theoretic_transform(expr::centered_binomial(q, {batch}, n, expr::half)),
                        expr::number_theoretic_transform(expr::centered_binomial(q, {batch}, n, expr::ten)));
    dump(dir, "u.bin", u.download());
    dump(dir, "v.bin", v.download());
    auto nonce = queue.nonce();
    if (nonce[0] != 2 * batch * n)
    {
        std::fprintf(stderr, "nonce %u, expected %llu\n", nonce[0], static_cast<unsigned long long>(2 * batch * n));
        return 1;
    }

    // a*u + v (broadcast of one polynomial over the batch), then back
    auto a = hmpc::comp::make_tensor(queue, q, {}, n);
    a.upload(std::vector<uint32_t>(host.begin(), host.begin() + static_cast<long>(n * q.limbs())));
    auto w = queue(expr::inverse_number_theoretic_transform(expr::tensor(a) * expr::tensor(u) + expr::tensor(v)));
    dump(dir, "w.bin", w.download());

    // a 2 x 3 matrix of NTT-form polynomials times the 3 polynomials of y
    // (broadcast over a batch of one), and the sum and product of y
    auto mat = hmpc::comp::make_tensor(queue, q, {1, 2, batch}, n);
    std::vector<uint32_t> mhost(mat.words(), 0u);
    for (uint64_t e = 0; e < 2 * batch * n; ++e)
    {
        mhost[e] = static_cast<uint32_t>(3 * e + 7);
    }
    mat.upload(mhost);
    auto vec = hmpc::comp::make_tensor(queue, q, {1, batch}, n);
    vec.upload(y.download());
    auto [z, total, prod] = queue(expr::matrix_vector_product(expr::tensor(mat), expr::tensor(vec)),
                                  expr::sum(expr::tensor(y)), expr::product(expr::tensor(y)));
    dump(dir, "matvec.bin", z.download());
    dump(dir, "sum.bin", total.download());
    dump(dir, "product.bin", prod.download());

    // BGV round trip through the lhe front end
    auto [s, key] = hmpc::crypto::lhe::keygen(queue, q, p, n);
    auto m = queue(expr::uniform(p, {batch}, n));
    auto ct = hmpc::crypto::lhe::enc(queue, key, m, q);
    auto back = hmpc::crypto::lhe::dec(queue, s, ct, p);
    if (back.download() != m.download())
    {
        std::fprintf(stderr, "BGV round trip failed\n");
        return 1;
    }
    queue.wait();
    std::printf("frontend ok\n");
    return 0;
}
