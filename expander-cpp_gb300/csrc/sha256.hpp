// Host SHA-256 (FIPS 180-4) for the Fiat-Shamir transcript.
//
// The reference transcript hashes with Bitcoin Core's CSHA256 through SHA256Hasher
// (include/hash/hashes.hpp:22-33), i.e. plain SHA-256 of a byte string.  This
// implementation uses the ARMv8 SHA-2 instructions when the compiler targets them
// (__ARM_FEATURE_SHA2) and portable C++ otherwise; both give the standard digest.
#pragma once
#include <stddef.h>
#include <stdint.h>

namespace gkrgpu {

// Streaming hasher: init, any number of update() calls, final().
struct Sha256 {
    uint32_t h[8];
    uint8_t buf[64];
    uint64_t total;
    uint32_t fill;
    Sha256() { init(); }
    void init();
    void update(const uint8_t* p, size_t n);
    void final(uint8_t out[32]);
};

void sha256(const uint8_t* in, size_t n, uint8_t out[32]);

// SHA-256 of three messages of the same length (interleaved on ARMv8).
void sha256_x3(const uint8_t* const in[3], size_t n, uint8_t out[3][32]);

// Name of the compression path compiled in ("armv8-sha2" or "portable").
const char* sha256_impl_name();

}  // namespace gkrgpu
