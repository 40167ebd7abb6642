// Fiat-Shamir transcript of the reference prover (include/fiat_shamir/transcript.hpp:87-175).
//
// The proof is the byte stream of everything appended.  A challenge is SHA-256 of the
// bytes appended since the previous challenge, or of the previous digest when nothing
// was appended (:91-103) - the digest is not chained into new data.  The digest starts
// as 32 zero bytes (:118-125).  challenge_f reads the first 4 digest bytes as a
// little-endian u32 and reduces it mod p (M31::from_bytes, include/field/M31.hpp:111-116).
#pragma once
#include <stdint.h>
#include <string.h>

#include "m31.cuh"
#include "sha256.hpp"

namespace gkrgpu {

class Transcript {
   public:
    Transcript(uint8_t* buf, uint64_t cap) : buf_(buf), cap_(cap) { memset(digest_, 0, 32); }

    uint64_t size() const { return len_; }
    uint8_t* tail() { return buf_ + len_; }

    // Appends n bytes (the caller has checked the capacity: the proof size is exact).
    void append(const void* p, uint64_t n) {
        memcpy(buf_ + len_, p, n);
        len_ += n;
    }
    // Marks n bytes already written at tail() as appended.
    void appended(uint64_t n) { len_ += n; }

    uint32_t challenge() {
        if (len_ > hash_start_) {
            sha256(buf_ + hash_start_, len_ - hash_start_, digest_);
            hash_start_ = len_;
        } else {
            uint8_t d[32];
            sha256(digest_, 32, d);
            memcpy(digest_, d, 32);
        }
        uint32_t x;
        memcpy(&x, digest_, 4);
        return m31::from_u32(x);
    }

   private:
    uint8_t* buf_;
    uint64_t cap_;
    uint64_t len_ = 0;
    uint64_t hash_start_ = 0;
    uint8_t digest_[32];
};

// grind (include/LinearGKR/LinearGKR.hpp:13-32): 256/31 = 8 challenges written at 4-byte
// offsets form 32 bytes, which are re-hashed in place 2^grinding_bits times and appended.
inline void grind(Transcript& t, int grinding_bits) {
    uint8_t h[32];
    memset(h, 0, 32);
    for (int i = 0; i < 256 / 31; i++) {
        const uint32_t c = t.challenge();
        memcpy(h + 4 * i, &c, 4);
    }
    for (long i = 0; i < (1L << grinding_bits); i++) {
        uint8_t d[32];
        sha256(h, 32, d);
        memcpy(h, d, 32);
    }
    t.append(h, 32);
}

}  // namespace gkrgpu
