// Keccak-f[1600] and the Keccak-256 / SHA3-256 sponges (keccak.hpp), written from the
// permutation's definition (theta, rho, pi, chi, iota on a 5 x 5 array of 64-bit lanes).
// The round constants and rotation offsets are derived at start-up from their definitions
// (the degree-8 LFSR x^8 + x^6 + x^5 + x^4 + 1 and the triangular offsets along the pi walk)
// rather than tabulated.
#include "keccak.hpp"

#include <string.h>

namespace gkrgpu {
namespace {

struct Tables {
    uint64_t rc[24];
    unsigned rot[5][5];  // rot[x][y]
    Tables() {
        // rc(t): output bit of the LFSR after t steps
        auto rc_bit = [](unsigned t) -> uint64_t {
            unsigned r = 1;
            for (unsigned i = 0; i < t % 255; i++) {
                r <<= 1;
                if (r & 0x100) r ^= 0x171;
            }
            return r & 1;
        };
        for (unsigned i = 0; i < 24; i++) {
            rc[i] = 0;
            for (unsigned j = 0; j < 7; j++) rc[i] |= rc_bit(j + 7 * i) << ((1u << j) - 1);
        }
        memset(rot, 0, sizeof(rot));
        unsigned x = 1, y = 0;
        for (unsigned t = 0; t < 24; t++) {
            rot[x][y] = ((t + 1) * (t + 2) / 2) % 64;
            const unsigned nx = y, ny = (2 * x + 3 * y) % 5;
            x = nx;
            y = ny;
        }
    }
};

const Tables& tables() {
    static const Tables t;
    return t;
}

inline uint64_t rotl(uint64_t v, unsigned n) { return n ? (v << n) | (v >> (64 - n)) : v; }

// a[x + 5 y]
void keccak_f(uint64_t a[25]) {
    const Tables& T = tables();
    for (int round = 0; round < 24; round++) {
        uint64_t c[5], b[25];
        for (int x = 0; x < 5; x++) c[x] = a[x] ^ a[x + 5] ^ a[x + 10] ^ a[x + 15] ^ a[x + 20];
        for (int x = 0; x < 5; x++) {
            const uint64_t d = c[(x + 4) % 5] ^ rotl(c[(x + 1) % 5], 1);
            for (int y = 0; y < 5; y++) a[x + 5 * y] ^= d;
        }
        for (int x = 0; x < 5; x++)
            for (int y = 0; y < 5; y++) b[y + 5 * ((2 * x + 3 * y) % 5)] = rotl(a[x + 5 * y], T.rot[x][y]);
        for (int x = 0; x < 5; x++)
            for (int y = 0; y < 5; y++)
                a[x + 5 * y] = b[x + 5 * y] ^ (~b[(x + 1) % 5 + 5 * y] & b[(x + 2) % 5 + 5 * y]);
        a[0] ^= T.rc[round];
    }
}

void sponge256(const uint8_t* in, size_t len, uint8_t domain, uint8_t out[32]) {
    constexpr size_t rate = 136;
    uint64_t a[25];
    memset(a, 0, sizeof(a));
    auto absorb = [&](const uint8_t* blk) {
        for (size_t i = 0; i < rate / 8; i++) {
            uint64_t w = 0;
            for (int k = 7; k >= 0; k--) w = (w << 8) | blk[8 * i + k];
            a[i] ^= w;
        }
        keccak_f(a);
    };
    while (len >= rate) {
        absorb(in);
        in += rate;
        len -= rate;
    }
    uint8_t last[rate];
    memset(last, 0, rate);
    if (len) memcpy(last, in, len);
    last[len] ^= domain;
    last[rate - 1] ^= 0x80;
    absorb(last);
    for (int i = 0; i < 4; i++)
        for (int k = 0; k < 8; k++) out[8 * i + k] = (uint8_t)(a[i] >> (8 * k));
}

}  // namespace

void keccak256(const uint8_t* in, size_t len, uint8_t out[32]) { sponge256(in, len, 0x01, out); }
void sha3_256(const uint8_t* in, size_t len, uint8_t out[32]) { sponge256(in, len, 0x06, out); }

}  // namespace gkrgpu

extern "C" {
// Exported for the tests (checked against a SHA3-256 implementation and known digests).
void gkrgpu_keccak256(const uint8_t* in, uint64_t len, uint8_t* out) { gkrgpu::keccak256(in, (size_t)len, out); }
void gkrgpu_sha3_256(const uint8_t* in, uint64_t len, uint8_t* out) { gkrgpu::sha3_256(in, (size_t)len, out); }
}
