// Wire format for shipping tensors (ciphertexts) between parties, packed and
// unpacked on the device.
//
// hmpc's network layer (hmpc-rs/src/net.rs:205-400, docs/networking.md
// "Message Format") writes one message per (operation, receiver):
//   version u8 (0) | feature flags u8 (bit 0 sessions, bit 1 signing) |
//   kind u8 | datatype u8 | sender u16 | receiver u16 | message id u64 |
//   [session id u128] | payload | [signature, 64 bytes]
// all little-endian; the payload of a tensor is its limb-planar storage as is
// (hmpc/net/queue.hpp:60-88: the host accessor's bytes).  The message id is
// the first eight bytes (little-endian) of SHA-256(senders || kind ||
// datatype || metadata member || receivers) plus a per-(kind, datatype, hash)
// operation counter starting at 1 (hmpc-rs/src/net/queue.rs:108-135,
// hmpc-rs/src/net/metadata.rs:3-76); a communicator hashes as its size (u64)
// and its party ids (u16) in ascending order.
//
// Packing many messages is one launch: every thread copies 16-byte pieces of
// a payload into its message's slot (slots start on 16-byte boundaries) and
// the first piece's thread writes the header.  Unpacking validates each
// header against the expected metadata on the device, then copies the
// payloads of the messages that passed.  The signing feature (Ed25519 over the
// metadata and SHA-256 of the payload) needs the parties' keys and is not
// implemented: flags with bit 1 set are rejected.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.hpp"

using namespace hmpc_gb300;
using namespace hmpc_gb300::detail;

namespace
{
    constexpr uint64_t piece = 16;

    struct WireSlot
    {
        uint64_t first_piece;  // prefix sum of pieces over the messages before this one
        uint64_t offset;       // of the message in the packed buffer
        uint64_t bytes;        // payload bytes
        uint64_t plane_bytes;  // the payload is planes of this size ...
        uint64_t plane_stride; // ... this far apart in the tensor
        const uint8_t* src;    // pack: payload; unpack: packed message
        uint8_t* dst;          // pack: packed message; unpack: payload
        uint8_t header[32];    // pack: the header to write; unpack: the expected header
        uint32_t header_bytes;
    };

    __device__ __forceinline__ uint32_t find_slot(const WireSlot* slots, uint32_t count, uint64_t pc)
    {
        uint32_t lo = 0, hi = count;
        while (hi - lo > 1)
        {
            const uint32_t mid = (lo + hi) / 2;
            if (slots[mid].first_piece <= pc)
            {
                lo = mid;
            }
            else
            {
                hi = mid;
            }
        }
        return lo;
    }

    // copy `len` (<= 16) bytes; both ends 16-byte aligned when len == 16
    __device__ __forceinline__ void copy_piece(uint8_t* dst, const uint8_t* src, uint64_t len)
    {
        if (len == piece && (reinterpret_cast<uintptr_t>(src) & 15u) == 0)
        {
            *reinterpret_cast<uint4*>(dst) = __ldg(reinterpret_cast<const uint4*>(src));
        }
        else
        {
            for (uint64_t i = 0; i < len; ++i)
            {
                dst[i] = src[i];
            }
        }
    }

    __global__ void wire_pack_kernel(const WireSlot* slots, uint32_t count, uint64_t pieces)
    {
        for (uint64_t pc = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; pc < pieces;
             pc += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        {
            const WireSlot& s = slots[find_slot(slots, count, pc)];
            const uint64_t k = pc - s.first_piece;
            uint8_t* msg = s.dst + s.offset;
            if (k == 0)
            {
                for (uint32_t i = 0; i < s.header_bytes; ++i)
                {
                    msg[i] = s.header[i];
                }
            }
            const uint64_t at = k * piece;
            if (at < s.bytes)
            {
                const uint64_t len = s.bytes - at < piece ? s.bytes - at : piece;
                const uint64_t plane = at / s.plane_bytes;
                copy_piece(msg + s.header_bytes + at, s.src + plane * s.plane_stride + (at - plane * s.plane_bytes), len);
            }
        }
    }

    // status[i]: 0 valid, else the first mismatching field (1 version, 2 flags,
    // 3 kind, 4 datatype, 5 sender, 6 receiver, 7 id, 8 session, 9 size)
    __global__ void wire_check_kernel(const WireSlot* slots, uint32_t count, const uint64_t* sizes,
                                      uint32_t* status)
    {
        const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= count)
        {
            return;
        }
        const WireSlot& s = slots[i];
        uint32_t code = 0;
        if (sizes[i] != s.header_bytes + s.bytes)
        {
            code = 9;
        }
        else
        {
            const uint8_t* msg = s.src + s.offset;
            // field boundaries: version 0, flags 1, kind 2, datatype 3, sender 4-5,
            // receiver 6-7, id 8-15, session 16-31
            const uint8_t field_end[8] = {1, 2, 3, 4, 6, 8, 16, 32};
            uint32_t field = 0;
            for (uint32_t b = 0; b < s.header_bytes && !code; ++b)
            {
                while (b >= field_end[field])
                {
                    ++field;
                }
                if (msg[b] != s.header[b])
                {
                    code = field + 1;
                }
            }
        }
        status[i] = code;
    }

    __global__ void wire_unpack_kernel(const WireSlot* slots, uint32_t count, uint64_t pieces,
                                       const uint32_t* status)
    {
        for (uint64_t pc = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; pc < pieces;
             pc += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        {
            const uint32_t m = find_slot(slots, count, pc);
            if (status[m])
            {
                continue;
            }
            const WireSlot& s = slots[m];
            const uint64_t at = (pc - s.first_piece) * piece;
            if (at < s.bytes)
            {
                const uint64_t len = s.bytes - at < piece ? s.bytes - at : piece;
                const uint8_t* src = s.src + s.offset + s.header_bytes + at;
                const uint64_t plane = at / s.plane_bytes;
                uint8_t* dst = s.dst + plane * s.plane_stride + (at - plane * s.plane_bytes);
                if (len == piece && ((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) & 15u) == 0)
                {
                    *reinterpret_cast<uint4*>(dst) = *reinterpret_cast<const uint4*>(src);
                }
                else
                {
                    for (uint64_t b = 0; b < len; ++b)
                    {
                        dst[b] = src[b];
                    }
                }
            }
        }
    }

    // ------------------------------------------------------------ SHA-256
    // FIPS 180-4.  The round constants are the first 32 fractional bits of the
    // cube roots of the first 64 primes and the initial state those of the
    // square roots of the first 8, computed here rather than tabulated.
    struct Sha256
    {
        uint32_t k[64], h[8];
        std::vector<uint8_t> data;

        Sha256()
        {
            int primes[64], n = 0;
            for (int c = 2; n < 64; ++c)
            {
                bool prime = true;
                for (int d = 2; d * d <= c; ++d)
                {
                    prime = prime && (c % d != 0);
                }
                if (prime)
                {
                    primes[n++] = c;
                }
            }
            for (int i = 0; i < 64; ++i)
            {
                k[i] = frac32(std::cbrt(static_cast<long double>(primes[i])), primes[i], 3);
            }
            for (int i = 0; i < 8; ++i)
            {
                h[i] = frac32(std::sqrt(static_cast<long double>(primes[i])), primes[i], 2);
            }
        }

        // floor(frac(x) * 2^32) for x = prime^(1/e), corrected against integer
        // arithmetic so the long double rounding cannot leak into the result
        static uint32_t frac32(long double x, int prime, int e)
        {
            const unsigned long long whole = static_cast<unsigned long long>(x);
            unsigned long long f = static_cast<unsigned long long>((x - static_cast<long double>(whole)) * 4294967296.0L);
            // (whole * 2^32 + f)^e <= prime * 2^(32 e) < (whole * 2^32 + f + 1)^e
            auto fits = [&](unsigned long long frac) {
                // compare (w + frac / 2^32)^e with prime using 128-bit integers
                const unsigned __int128 v = (static_cast<unsigned __int128>(whole) << 32) + frac;
                unsigned __int128 p = 1;
                for (int i = 0; i < e; ++i)
                {
                    p *= v;  // v < 2^35, v^3 < 2^105
                }
                const unsigned __int128 target = static_cast<unsigned __int128>(prime) << (32 * e);
                return p <= target;
            };
            while (f > 0 && !fits(f))
            {
                --f;
            }
            while (f + 1 < (1ull << 32) && fits(f + 1))
            {
                ++f;
            }
            return static_cast<uint32_t>(f);
        }

        static uint32_t rotr(uint32_t x, int n)
        {
            return (x >> n) | (x << (32 - n));
        }

        void update(const void* p, size_t n)
        {
            const uint8_t* b = static_cast<const uint8_t*>(p);
            data.insert(data.end(), b, b + n);
        }

        void finish(uint8_t out[32])
        {
            const uint64_t bits = static_cast<uint64_t>(data.size()) * 8;
            data.push_back(0x80);
            while (data.size() % 64 != 56)
            {
                data.push_back(0);
            }
            for (int i = 7; i >= 0; --i)
            {
                data.push_back(static_cast<uint8_t>(bits >> (8 * i)));
            }
            uint32_t s[8];
            std::memcpy(s, h, sizeof s);
            for (size_t blk = 0; blk < data.size(); blk += 64)
            {
                uint32_t w[64];
                for (int i = 0; i < 16; ++i)
                {
                    w[i] = (static_cast<uint32_t>(data[blk + 4 * i]) << 24) |
                           (static_cast<uint32_t>(data[blk + 4 * i + 1]) << 16) |
                           (static_cast<uint32_t>(data[blk + 4 * i + 2]) << 8) | data[blk + 4 * i + 3];
                }
                for (int i = 16; i < 64; ++i)
                {
                    const uint32_t s0 = rotr(w[i - 15], 7) ^ rotr(w[i - 15], 18) ^ (w[i - 15] >> 3);
                    const uint32_t s1 = rotr(w[i - 2], 17) ^ rotr(w[i - 2], 19) ^ (w[i - 2] >> 10);
                    w[i] = w[i - 16] + s0 + w[i - 7] + s1;
                }
                uint32_t a = s[0], b = s[1], c = s[2], d = s[3], e = s[4], f = s[5], g = s[6], hh = s[7];
                for (int i = 0; i < 64; ++i)
                {
                    const uint32_t t1 = hh + (rotr(e, 6) ^ rotr(e, 11) ^ rotr(e, 25)) + ((e & f) ^ (~e & g)) + k[i] + w[i];
                    const uint32_t t2 = (rotr(a, 2) ^ rotr(a, 13) ^ rotr(a, 22)) + ((a & b) ^ (a & c) ^ (b & c));
                    hh = g;
                    g = f;
                    f = e;
                    e = d + t1;
                    d = c;
                    c = b;
                    b = a;
                    a = t1 + t2;
                }
                s[0] += a; s[1] += b; s[2] += c; s[3] += d; s[4] += e; s[5] += f; s[6] += g; s[7] += hh;
            }
            for (int i = 0; i < 8; ++i)
            {
                for (int j = 0; j < 4; ++j)
                {
                    out[4 * i + j] = static_cast<uint8_t>(s[i] >> (24 - 8 * j));
                }
            }
        }
    };

    uint32_t header_bytes(uint8_t flags)
    {
        return (flags & 1u) ? 32u : 16u;
    }

    void write_header(uint8_t* h, uint8_t flags, const hmpc_wire_message& m, const uint8_t* session)
    {
        h[0] = 0;  // message format version
        h[1] = flags;
        h[2] = m.kind;
        h[3] = m.datatype;
        h[4] = static_cast<uint8_t>(m.sender);
        h[5] = static_cast<uint8_t>(m.sender >> 8);
        h[6] = static_cast<uint8_t>(m.receiver);
        h[7] = static_cast<uint8_t>(m.receiver >> 8);
        for (int i = 0; i < 8; ++i)
        {
            h[8 + i] = static_cast<uint8_t>(m.id >> (8 * i));
        }
        if (flags & 1u)
        {
            std::memcpy(h + 16, session, 16);
        }
    }

    // a payload of `planes` equal parts `plane_stride` bytes apart (one
    // ciphertext's limb planes inside a batch tensor); 0 or 1 plane: contiguous
    int set_planes(WireSlot& s, const hmpc_wire_message& m)
    {
        if (m.planes <= 1)
        {
            s.plane_bytes = m.bytes ? m.bytes : 1;
            s.plane_stride = 0;
            return HMPC_OK;
        }
        if (m.bytes % m.planes || (m.bytes / m.planes) % piece || m.plane_stride < m.bytes / m.planes)
        {
            return fail(HMPC_ERROR_INVALID_ARGUMENT, "payload planes must be equal multiples of 16 bytes");
        }
        s.plane_bytes = m.bytes / m.planes;
        s.plane_stride = m.plane_stride;
        return HMPC_OK;
    }

    int check_flags(uint8_t flags, const uint8_t* session)
    {
        if (flags & ~3u)
        {
            return fail(HMPC_ERROR_INVALID_ARGUMENT, "unknown feature flags");
        }
        if (flags & 2u)
        {
            return fail(HMPC_ERROR_UNSUPPORTED, "the signing feature needs the parties' Ed25519 keys");
        }
        if ((flags & 1u) && !session)
        {
            return fail(HMPC_ERROR_INVALID_ARGUMENT, "the sessions feature needs a session id");
        }
        return HMPC_OK;
    }

    int upload_slots(hmpc_context* ctx, const std::vector<WireSlot>& slots, WireSlot** out)
    {
        const size_t bytes = slots.size() * sizeof(WireSlot);
        uint32_t* ws = ctx->scratch((bytes + 3) / 4);
        if (!ws)
        {
            return fail(HMPC_ERROR_OUT_OF_MEMORY, "allocating the message table");
        }
        HMPC_CUDA(cudaMemcpyAsync(ws, slots.data(), bytes, cudaMemcpyHostToDevice, ctx->stream), "uploading messages");
        *out = reinterpret_cast<WireSlot*>(ws);
        return HMPC_OK;
    }

    unsigned copy_grid(uint64_t pieces)
    {
        const uint64_t g = (pieces + 255) / 256;
        return static_cast<unsigned>(std::max<uint64_t>(1, std::min<uint64_t>(g, 152ull * 32ull)));
    }
}

int hmpc_wire_layout(const hmpc_wire_message* messages, uint64_t count, uint8_t flags, uint64_t* offsets,
                     uint64_t* total_bytes)
{
    if ((count && (!messages || !offsets)) || !total_bytes)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
    }
    uint64_t at = 0;
    for (uint64_t i = 0; i < count; ++i)
    {
        offsets[i] = at;
        at += (header_bytes(flags) + messages[i].bytes + piece - 1) / piece * piece;
    }
    *total_bytes = at;
    return HMPC_OK;
}

int hmpc_wire_pack(hmpc_context* ctx, const hmpc_wire_message* messages, uint64_t count, uint8_t flags,
                   const uint8_t session[16], const uint64_t* offsets, uint8_t* out)
{
    if (int rc = enter(ctx))
    {
        return rc;
    }
    if (int rc = check_flags(flags, session))
    {
        return rc;
    }
    if (count == 0)
    {
        return HMPC_OK;
    }
    if (!messages || !offsets || !out)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
    }
    std::vector<WireSlot> slots(count);
    uint64_t pieces = 0;
    for (uint64_t i = 0; i < count; ++i)
    {
        if ((offsets[i] & (piece - 1)) || (messages[i].bytes && !messages[i].payload))
        {
            return fail(HMPC_ERROR_INVALID_ARGUMENT, "message slots start on 16-byte boundaries");
        }
        WireSlot& s = slots[i];
        if (int rc = set_planes(s, messages[i]))
        {
            return rc;
        }
        s.first_piece = pieces;
        s.offset = offsets[i];
        s.bytes = messages[i].bytes;
        s.src = static_cast<const uint8_t*>(messages[i].payload);
        s.dst = out;
        s.header_bytes = header_bytes(flags);
        write_header(s.header, flags, messages[i], session);
        pieces += std::max<uint64_t>(1, (s.bytes + piece - 1) / piece);
    }
    WireSlot* d_slots = nullptr;
    if (int rc = upload_slots(ctx, slots, &d_slots))
    {
        return rc;
    }
    wire_pack_kernel<<<copy_grid(pieces), 256, 0, ctx->stream>>>(d_slots, static_cast<uint32_t>(count), pieces);
    HMPC_CUDA(cudaGetLastError(), "launching the message packer");
    ++ctx->launches;
    return HMPC_OK;
}

int hmpc_wire_unpack(hmpc_context* ctx, const uint8_t* in, const uint64_t* offsets, const uint64_t* sizes,
                     uint64_t count, uint8_t flags, const uint8_t session[16], const hmpc_wire_message* expected,
                     void* const* payloads, uint32_t* status)
{
    if (int rc = enter(ctx))
    {
        return rc;
    }
    if (int rc = check_flags(flags, session))
    {
        return rc;
    }
    if (count == 0)
    {
        return HMPC_OK;
    }
    if (!in || !offsets || !sizes || !expected || !payloads || !status)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
    }
    std::vector<WireSlot> slots(count);
    uint64_t pieces = 0;
    for (uint64_t i = 0; i < count; ++i)
    {
        WireSlot& s = slots[i];
        if (int rc = set_planes(s, expected[i]))
        {
            return rc;
        }
        s.first_piece = pieces;
        s.offset = offsets[i];
        s.bytes = expected[i].bytes;
        s.src = in;
        s.dst = static_cast<uint8_t*>(payloads[i]);
        s.header_bytes = header_bytes(flags);
        write_header(s.header, flags, expected[i], session);
        if (s.bytes && !s.dst)
        {
            return fail(HMPC_ERROR_INVALID_ARGUMENT, "null payload destination");
        }
        pieces += std::max<uint64_t>(1, (s.bytes + piece - 1) / piece);
    }
    // the sizes array is read on the device: stage it behind the slot table
    std::vector<uint64_t> host_sizes(sizes, sizes + count);
    const size_t slot_bytes = count * sizeof(WireSlot);
    const size_t total = slot_bytes + count * sizeof(uint64_t);
    uint32_t* ws = ctx->scratch((total + 3) / 4);
    if (!ws)
    {
        return fail(HMPC_ERROR_OUT_OF_MEMORY, "allocating the message table");
    }
    uint8_t* base = reinterpret_cast<uint8_t*>(ws);
    HMPC_CUDA(cudaMemcpyAsync(base, slots.data(), slot_bytes, cudaMemcpyHostToDevice, ctx->stream), "uploading messages");
    HMPC_CUDA(cudaMemcpyAsync(base + slot_bytes, host_sizes.data(), count * sizeof(uint64_t), cudaMemcpyHostToDevice,
                              ctx->stream),
              "uploading message sizes");
    const WireSlot* d_slots = reinterpret_cast<const WireSlot*>(base);
    const uint64_t* d_sizes = reinterpret_cast<const uint64_t*>(base + slot_bytes);
    wire_check_kernel<<<static_cast<unsigned>((count + 255) / 256), 256, 0, ctx->stream>>>(
        d_slots, static_cast<uint32_t>(count), d_sizes, status);
    HMPC_CUDA(cudaGetLastError(), "launching the message check");
    wire_unpack_kernel<<<copy_grid(pieces), 256, 0, ctx->stream>>>(d_slots, static_cast<uint32_t>(count), pieces,
                                                                   status);
    HMPC_CUDA(cudaGetLastError(), "launching the message unpacker");
    ctx->launches += 2;
    // the host staging vectors must outlive the asynchronous copies
    HMPC_CUDA(cudaStreamSynchronize(ctx->stream), "unpacking messages");
    return HMPC_OK;
}

int hmpc_wire_message_id(uint8_t kind, uint8_t datatype, const uint16_t* member, int members,
                         const uint16_t* senders, int sender_count, const uint16_t* receivers, int receiver_count,
                         uint64_t counter, uint64_t* id)
{
    if (!id || members < 0 || members > 1 || (members && !member) || sender_count < 0 || receiver_count < 0 ||
        (sender_count && !senders) || (receiver_count && !receivers))
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "invalid message id arguments");
    }
    auto put_communicator = [](Sha256& sha, const uint16_t* parties, int count) {
        std::vector<uint16_t> sorted(parties, parties + count);
        std::sort(sorted.begin(), sorted.end());
        sorted.erase(std::unique(sorted.begin(), sorted.end()), sorted.end());
        const uint64_t len = sorted.size();
        uint8_t b[8];
        for (int i = 0; i < 8; ++i)
        {
            b[i] = static_cast<uint8_t>(len >> (8 * i));
        }
        sha.update(b, 8);
        for (uint16_t p : sorted)
        {
            const uint8_t pb[2] = {static_cast<uint8_t>(p), static_cast<uint8_t>(p >> 8)};
            sha.update(pb, 2);
        }
    };
    Sha256 sha;
    put_communicator(sha, senders, sender_count);
    sha.update(&kind, 1);
    sha.update(&datatype, 1);
    if (members)
    {
        const uint8_t mb[2] = {static_cast<uint8_t>(*member), static_cast<uint8_t>(*member >> 8)};
        sha.update(mb, 2);
    }
    put_communicator(sha, receivers, receiver_count);
    uint8_t digest[32];
    sha.finish(digest);
    uint64_t initial = 0;
    for (int i = 0; i < 8; ++i)
    {
        initial |= static_cast<uint64_t>(digest[i]) << (8 * i);
    }
    *id = initial + counter;
    return HMPC_OK;
}

int hmpc_wire_sha256(const void* data, uint64_t bytes, uint8_t digest[32])
{
    if ((bytes && !data) || !digest)
    {
        return fail(HMPC_ERROR_INVALID_ARGUMENT, "null argument");
    }
    Sha256 sha;
    sha.update(data, bytes);
    sha.finish(digest);
    return HMPC_OK;
}
