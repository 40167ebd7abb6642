// Host SHA-256, see sha256.hpp.
#include "sha256.hpp"

#include <string.h>

#if defined(__aarch64__) && defined(__ARM_FEATURE_SHA2)
#include <arm_neon.h>
#define GKR_SHA_ARMV8 1
#endif

namespace gkrgpu {

namespace {

alignas(16) const uint32_t K[64] = {
    0x428a2f98, 0x71374491, 0xb5c0fbcf, 0xe9b5dba5, 0x3956c25b, 0x59f111f1, 0x923f82a4, 0xab1c5ed5,
    0xd807aa98, 0x12835b01, 0x243185be, 0x550c7dc3, 0x72be5d74, 0x80deb1fe, 0x9bdc06a7, 0xc19bf174,
    0xe49b69c1, 0xefbe4786, 0x0fc19dc6, 0x240ca1cc, 0x2de92c6f, 0x4a7484aa, 0x5cb0a9dc, 0x76f988da,
    0x983e5152, 0xa831c66d, 0xb00327c8, 0xbf597fc7, 0xc6e00bf3, 0xd5a79147, 0x06ca6351, 0x14292967,
    0x27b70a85, 0x2e1b2138, 0x4d2c6dfc, 0x53380d13, 0x650a7354, 0x766a0abb, 0x81c2c92e, 0x92722c85,
    0xa2bfe8a1, 0xa81a664b, 0xc24b8b70, 0xc76c51a3, 0xd192e819, 0xd6990624, 0xf40e3585, 0x106aa070,
    0x19a4c116, 0x1e376c08, 0x2748774c, 0x34b0bcb5, 0x391c0cb3, 0x4ed8aa4a, 0x5b9cca4f, 0x682e6ff3,
    0x748f82ee, 0x78a5636f, 0x84c87814, 0x8cc70208, 0x90befffa, 0xa4506ceb, 0xbef9a3f7, 0xc67178f2};

#if defined(GKR_SHA_ARMV8)
// Four rounds per step: vsha256hq/vsha256h2q advance (a..d, e..h) by the four words of
// wk = W[4i..4i+3] + K[4i..4i+3]; vsha256su0q/vsha256su1q extend the message schedule.
void compress(uint32_t st[8], const uint8_t* p, size_t nblocks) {
    uint32x4_t s0 = vld1q_u32(st), s1 = vld1q_u32(st + 4);
    for (size_t b = 0; b < nblocks; b++, p += 64) {
        uint32x4_t m[4];
        for (int i = 0; i < 4; i++) m[i] = vreinterpretq_u32_u8(vrev32q_u8(vld1q_u8(p + 16 * i)));
        const uint32x4_t save0 = s0, save1 = s1;
        for (int i = 0; i < 16; i++) {
            const uint32x4_t wk = vaddq_u32(m[i & 3], vld1q_u32(K + 4 * i));
            if (i < 12)
                m[i & 3] = vsha256su1q_u32(vsha256su0q_u32(m[i & 3], m[(i + 1) & 3]), m[(i + 2) & 3], m[(i + 3) & 3]);
            const uint32x4_t abcd = s0;
            s0 = vsha256hq_u32(s0, s1, wk);
            s1 = vsha256h2q_u32(s1, abcd, wk);
        }
        s0 = vaddq_u32(s0, save0);
        s1 = vaddq_u32(s1, save1);
    }
    vst1q_u32(st, s0);
    vst1q_u32(st + 4, s1);
}
#else
inline uint32_t ror(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }
inline uint32_t be32(const uint8_t* p) {
    return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | (uint32_t)p[3];
}

void compress(uint32_t st[8], const uint8_t* p, size_t nblocks) {
    for (size_t b = 0; b < nblocks; b++, p += 64) {
        uint32_t w[64];
        for (int i = 0; i < 16; i++) w[i] = be32(p + 4 * i);
        for (int i = 16; i < 64; i++) {
            const uint32_t s0 = ror(w[i - 15], 7) ^ ror(w[i - 15], 18) ^ (w[i - 15] >> 3);
            const uint32_t s1 = ror(w[i - 2], 17) ^ ror(w[i - 2], 19) ^ (w[i - 2] >> 10);
            w[i] = w[i - 16] + s0 + w[i - 7] + s1;
        }
        uint32_t a = st[0], bb = st[1], c = st[2], d = st[3], e = st[4], f = st[5], g = st[6], h = st[7];
        for (int i = 0; i < 64; i++) {
            const uint32_t t1 = h + (ror(e, 6) ^ ror(e, 11) ^ ror(e, 25)) + ((e & f) ^ (~e & g)) + K[i] + w[i];
            const uint32_t t2 = (ror(a, 2) ^ ror(a, 13) ^ ror(a, 22)) + ((a & bb) ^ (a & c) ^ (bb & c));
            h = g; g = f; f = e; e = d + t1; d = c; c = bb; bb = a; a = t1 + t2;
        }
        st[0] += a; st[1] += bb; st[2] += c; st[3] += d; st[4] += e; st[5] += f; st[6] += g; st[7] += h;
    }
}
#endif

}  // namespace

void Sha256::init() {
    static const uint32_t H0[8] = {0x6a09e667, 0xbb67ae85, 0x3c6ef372, 0xa54ff53a,
                                   0x510e527f, 0x9b05688c, 0x1f83d9ab, 0x5be0cd19};
    memcpy(h, H0, sizeof(h));
    total = 0;
    fill = 0;
}

void Sha256::update(const uint8_t* p, size_t n) {
    total += n;
    if (fill) {
        size_t take = 64 - fill < n ? 64 - fill : n;
        memcpy(buf + fill, p, take);
        fill += (uint32_t)take;
        p += take;
        n -= take;
        if (fill < 64) return;
        compress(h, buf, 1);
        fill = 0;
    }
    const size_t nb = n / 64;
    if (nb) compress(h, p, nb);
    p += nb * 64;
    n -= nb * 64;
    if (n) {
        memcpy(buf, p, n);
        fill = (uint32_t)n;
    }
}

void Sha256::final(uint8_t out[32]) {
    const uint64_t bits = total * 8;
    uint8_t pad[72];
    memset(pad, 0, sizeof(pad));
    pad[0] = 0x80;
    const size_t padlen = (fill < 56) ? (56 - fill) : (120 - fill);
    for (int i = 0; i < 8; i++) pad[padlen + i] = (uint8_t)(bits >> (56 - 8 * i));
    const uint64_t keep = total;
    update(pad, padlen + 8);
    total = keep;
    for (int i = 0; i < 8; i++) {
        out[4 * i] = (uint8_t)(h[i] >> 24);
        out[4 * i + 1] = (uint8_t)(h[i] >> 16);
        out[4 * i + 2] = (uint8_t)(h[i] >> 8);
        out[4 * i + 3] = (uint8_t)h[i];
    }
}

void sha256(const uint8_t* in, size_t n, uint8_t out[32]) {
    Sha256 s;
    s.update(in, n);
    s.final(out);
}

namespace {

#if defined(GKR_SHA_ARMV8)
void put_digest(const uint32_t h[8], uint8_t out[32]) {
    for (int i = 0; i < 8; i++) {
        out[4 * i] = (uint8_t)(h[i] >> 24);
        out[4 * i + 1] = (uint8_t)(h[i] >> 16);
        out[4 * i + 2] = (uint8_t)(h[i] >> 8);
        out[4 * i + 3] = (uint8_t)h[i];
    }
}

// Three independent message streams in one loop: the SHA-2 instructions of one stream
// depend on each other, so interleaving three streams fills the pipeline.
void compress3(uint32_t st[3][8], const uint8_t* const p[3], size_t nblocks) {
    uint32x4_t s0[3], s1[3];
    for (int m = 0; m < 3; m++) {
        s0[m] = vld1q_u32(st[m]);
        s1[m] = vld1q_u32(st[m] + 4);
    }
    for (size_t b = 0; b < nblocks; b++) {
        uint32x4_t w[3][4], save0[3], save1[3];
        for (int m = 0; m < 3; m++) {
            for (int i = 0; i < 4; i++) w[m][i] = vreinterpretq_u32_u8(vrev32q_u8(vld1q_u8(p[m] + 64 * b + 16 * i)));
            save0[m] = s0[m];
            save1[m] = s1[m];
        }
        for (int i = 0; i < 16; i++) {
            const uint32x4_t k = vld1q_u32(K + 4 * i);
            for (int m = 0; m < 3; m++) {
                const uint32x4_t wk = vaddq_u32(w[m][i & 3], k);
                if (i < 12)
                    w[m][i & 3] = vsha256su1q_u32(vsha256su0q_u32(w[m][i & 3], w[m][(i + 1) & 3]), w[m][(i + 2) & 3],
                                                  w[m][(i + 3) & 3]);
                const uint32x4_t abcd = s0[m];
                s0[m] = vsha256hq_u32(s0[m], s1[m], wk);
                s1[m] = vsha256h2q_u32(s1[m], abcd, wk);
            }
        }
        for (int m = 0; m < 3; m++) {
            s0[m] = vaddq_u32(s0[m], save0[m]);
            s1[m] = vaddq_u32(s1[m], save1[m]);
        }
    }
    for (int m = 0; m < 3; m++) {
        vst1q_u32(st[m], s0[m]);
        vst1q_u32(st[m] + 4, s1[m]);
    }
}
#endif

}  // namespace

void sha256_x3(const uint8_t* const in[3], size_t n, uint8_t out[3][32]) {
#if defined(GKR_SHA_ARMV8)
    static const uint32_t H0[8] = {0x6a09e667, 0xbb67ae85, 0x3c6ef372, 0xa54ff53a,
                                   0x510e527f, 0x9b05688c, 0x1f83d9ab, 0x5be0cd19};
    uint32_t st[3][8];
    for (int m = 0; m < 3; m++) memcpy(st[m], H0, sizeof(H0));
    const size_t full = n / 64;
    compress3(st, in, full);
    // identical lengths give identical padding: build each tail and finish together
    const size_t rem = n - 64 * full;
    const size_t tl = (rem + 9 <= 64) ? 64 : 128;
    uint8_t tail[3][128];
    const uint64_t bits = (uint64_t)n * 8;
    for (int m = 0; m < 3; m++) {
        memset(tail[m], 0, sizeof(tail[m]));
        if (rem) memcpy(tail[m], in[m] + 64 * full, rem);
        tail[m][rem] = 0x80;
        for (int i = 0; i < 8; i++) tail[m][tl - 1 - i] = (uint8_t)(bits >> (8 * i));
    }
    const uint8_t* tp[3] = {tail[0], tail[1], tail[2]};
    compress3(st, tp, tl / 64);
    for (int m = 0; m < 3; m++) put_digest(st[m], out[m]);
#else
    for (int m = 0; m < 3; m++) sha256(in[m], n, out[m]);
#endif
}

const char* sha256_impl_name() {
#if defined(GKR_SHA_ARMV8)
    return "armv8-sha2";
#else
    return "portable";
#endif
}

}  // namespace gkrgpu
