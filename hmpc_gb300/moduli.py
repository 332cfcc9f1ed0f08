"""Named moduli of the workloads (the reference's example moduli and
NTT-friendly primes of 4..8 limbs) and a host ChaCha20 word stream that seeds
workload shapes (degrees, arrival times)."""

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
