// Fiat-Shamir transcript of the reference prover (include/fiat_shamir/transcript.hpp:87-175).
//
// The proof is the byte stream of everything appended.  A challenge is SHA-256 of the
// bytes appended since the previous challenge, or of the previous digest when nothing
// was appended (:91-103) - the digest is not chained into new data.  The digest starts
// as 32 zero bytes (:118-125).  challenge_f reads the first 4 digest bytes as a
// little-endian u32 and reduces it mod p (M31::from_bytes, include/field/M31.hpp:111-116).
//
// The hash is SHA-256, the only one the reference's transcript implements (the prover
// asserts it, include/LinearGKR/LinearGKR.hpp:45).  Config::FS_hash also names Keccak256
// (include/configuration/config.hpp:18-24) without code behind it; selecting it here runs
// the same schedule with Keccak-256 (keccak.hpp) in every place SHA-256 is used.
#pragma once
#include <stdint.h>
#include <string.h>

#include "fr_host.hpp"
#include "keccak.hpp"
#include "m31.cuh"
#include "sha256.hpp"

namespace gkrgpu {

// FiatShamir_hash_type numbering (config.hpp:18-24).
enum FsHash : int { kFsSha256 = 0, kFsKeccak256 = 1 };

inline void fs_hash(int h, const uint8_t* p, uint64_t n, uint8_t out[32]) {
    if (h == kFsKeccak256)
        keccak256(p, (size_t)n, out);
    else
        sha256(p, n, out);
}

// Position of a transcript: bytes written, start of the not-yet-hashed bytes, digest, hash.
struct TranscriptState {
    uint64_t len = 0, hash_start = 0;
    uint8_t digest[32] = {};
    int hash = kFsSha256;
};

class Transcript {
   public:
    Transcript(uint8_t* buf, uint64_t cap, int hash = kFsSha256) : buf_(buf), cap_(cap) { s_.hash = hash; }
    // Resumes a transcript over the same buffer (e.g. on another thread).
    Transcript(uint8_t* buf, const TranscriptState& s) : buf_(buf), cap_(~0ull), s_(s) {}

    const TranscriptState& state() const { return s_; }
    uint64_t size() const { return s_.len; }
    uint8_t* tail() { return buf_ + s_.len; }

    // Appends n bytes (the caller has checked the capacity: the proof size is exact).
    void append(const void* p, uint64_t n) {
        memcpy(buf_ + s_.len, p, n);
        s_.len += n;
    }
    // Marks n bytes already written at tail() as appended.
    void appended(uint64_t n) { s_.len += n; }
    // Marks n bytes already written at tail() as appended when their SHA-256 `d` was computed
    // elsewhere (from the same bytes); the next challenge uses it if nothing else was appended.
    void appended_prehashed(uint64_t n, const uint8_t d[32]) {
        s_.len += n;
        memcpy(pre_, d, 32);
        pre_from_ = s_.len - n;
        pre_to_ = s_.len;
        has_pre_ = true;
    }

    // Appends three messages of n bytes, each followed by a challenge, exactly as three
    // append+challenge steps would when nothing else is pending; the three SHA-256 run
    // interleaved.  Returns false (and does nothing) when bytes are pending.
    bool append_challenge3(const uint8_t* const msgs[3], uint64_t n, uint32_t out[3]) {
        if (s_.len != s_.hash_start || has_pre_ || s_.hash != kFsSha256) return false;
        const uint8_t* at[3];
        for (int m = 0; m < 3; m++) {
            at[m] = buf_ + s_.len;
            append(msgs[m], n);
        }
        uint8_t d[3][32];
        sha256_x3(at, n, d);
        s_.hash_start = s_.len;
        memcpy(s_.digest, d[2], 32);
        for (int m = 0; m < 3; m++) {
            uint32_t x;
            memcpy(&x, d[m], 4);
            out[m] = m31::from_u32(x);
        }
        return true;
    }

    uint32_t challenge() {
        uint32_t x;
        memcpy(&x, next_digest(), 4);
        return m31::from_u32(x);
    }
    // BN254 challenge_f: the whole digest, read little-endian and reduced mod r.
    frh::Fr challenge_bn254() { return frh::from_bytes(next_digest()); }

    // The digest behind the next challenge (_hash_to_digest, transcript.hpp:91-103).
    const uint8_t* next_digest() {
        if (has_pre_ && s_.hash_start == pre_from_ && s_.len == pre_to_) {
            memcpy(s_.digest, pre_, 32);
            s_.hash_start = s_.len;
            has_pre_ = false;
        } else if (s_.len > s_.hash_start) {
            fs_hash(s_.hash, buf_ + s_.hash_start, s_.len - s_.hash_start, s_.digest);
            s_.hash_start = s_.len;
        } else {
            uint8_t d[32];
            fs_hash(s_.hash, s_.digest, 32, d);
            memcpy(s_.digest, d, 32);
        }
        return s_.digest;
    }

   private:
    uint8_t* buf_;
    uint64_t cap_;
    TranscriptState s_;
    uint8_t pre_[32];
    uint64_t pre_from_ = 0, pre_to_ = 0;
    bool has_pre_ = false;
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
        fs_hash(t.state().hash, h, 32, d);
        memcpy(h, d, 32);
    }
    t.append(h, 32);
}

// The same for BN254: 256/254 = 1 challenge, written as its 32 canonical bytes.
inline void grind_bn254(Transcript& t, int grinding_bits) {
    uint8_t h[32];
    frh::to_bytes(t.challenge_bn254(), h);
    for (long i = 0; i < (1L << grinding_bits); i++) {
        uint8_t d[32];
        fs_hash(t.state().hash, h, 32, d);
        memcpy(h, d, 32);
    }
    t.append(h, 32);
}

}  // namespace gkrgpu
