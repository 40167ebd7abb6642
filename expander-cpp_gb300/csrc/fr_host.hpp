// Host arithmetic of the BN254 scalar field r = 0x30644e72...43e1f593f0000001 for the
// transcript side of the BN254 prover: challenges (a 32-byte digest read little-endian and
// reduced mod r), the last 2->1 folds of each sumcheck phase and Montgomery conversion of
// the values sent to the device.  4 x 64-bit limbs, Montgomery form x * 2^256 mod r with
// CIOS multiplication (Koc, Acar, Kaliski 1996).  Its memory image is the device's 8 x 32-bit
// limb layout (both hosts are little-endian).
#pragma once
#include <stdint.h>
#include <string.h>

namespace gkrgpu {
namespace frh {

struct Fr {
    uint64_t v[4];
};

typedef unsigned __int128 u128;

constexpr uint64_t kR[4] = {0x43e1f593f0000001ull, 0x2833e84879b97091ull, 0xb85045b68181585dull,
                            0x30644e72e131a029ull};
constexpr uint64_t kNP = 0xc2e1f593efffffffull;  // -r^-1 mod 2^64
constexpr uint64_t kR2[4] = {0x1bb8e645ae216da7ull, 0x53fe3ab1e35c59e3ull, 0x8c49833d53bb8085ull,
                             0x0216d0b17f4e44a5ull};  // 2^512 mod r

inline bool geq_r(const uint64_t* a) {
    for (int i = 3; i >= 0; i--) {
        if (a[i] != kR[i]) return a[i] > kR[i];
    }
    return true;
}
inline void sub_r(uint64_t* a) {
    uint64_t br = 0;
    for (int i = 0; i < 4; i++) {
        const u128 d = (u128)a[i] - kR[i] - br;
        a[i] = (uint64_t)d;
        br = (uint64_t)(d >> 64) & 1;
    }
}
inline Fr zero() { return Fr{{0, 0, 0, 0}}; }
inline Fr from_u32(uint32_t x) { return Fr{{x, 0, 0, 0}}; }
inline bool is_canonical(const Fr& a) { return !geq_r(a.v); }
inline bool eq(const Fr& a, const Fr& b) { return memcmp(a.v, b.v, 32) == 0; }

inline Fr add(const Fr& a, const Fr& b) {
    Fr s;
    uint64_t c = 0;
    for (int i = 0; i < 4; i++) {
        const u128 t = (u128)a.v[i] + b.v[i] + c;
        s.v[i] = (uint64_t)t;
        c = (uint64_t)(t >> 64);
    }
    if (c || geq_r(s.v)) sub_r(s.v);
    return s;
}
inline Fr sub(const Fr& a, const Fr& b) {
    Fr d;
    uint64_t br = 0;
    for (int i = 0; i < 4; i++) {
        const u128 t = (u128)a.v[i] - b.v[i] - br;
        d.v[i] = (uint64_t)t;
        br = (uint64_t)(t >> 64) & 1;
    }
    if (br) {
        uint64_t c = 0;
        for (int i = 0; i < 4; i++) {
            const u128 t = (u128)d.v[i] + kR[i] + c;
            d.v[i] = (uint64_t)t;
            c = (uint64_t)(t >> 64);
        }
    }
    return d;
}
// a * b * 2^-256 mod r for a, b < r.
inline Fr mont(const Fr& a, const Fr& b) {
    uint64_t t[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < 4; i++) {
        uint64_t c = 0;
        for (int j = 0; j < 4; j++) {
            const u128 p = (u128)a.v[j] * b.v[i] + t[j] + c;
            t[j] = (uint64_t)p;
            c = (uint64_t)(p >> 64);
        }
        u128 s = (u128)t[4] + c;
        t[4] = (uint64_t)s;
        t[5] = (uint64_t)(s >> 64);
        const uint64_t m = t[0] * kNP;
        u128 p = (u128)m * kR[0] + t[0];
        c = (uint64_t)(p >> 64);
        for (int j = 1; j < 4; j++) {
            p = (u128)m * kR[j] + t[j] + c;
            t[j - 1] = (uint64_t)p;
            c = (uint64_t)(p >> 64);
        }
        s = (u128)t[4] + c;
        t[3] = (uint64_t)s;
        t[4] = t[5] + (uint64_t)(s >> 64);
    }
    Fr r;
    memcpy(r.v, t, 32);
    if (t[4] || geq_r(r.v)) sub_r(r.v);
    return r;
}
inline Fr to_mont(const Fr& a) { return mont(a, Fr{{kR2[0], kR2[1], kR2[2], kR2[3]}}); }
// a * b mod r of canonical values (two Montgomery products)
inline Fr mul(const Fr& a, const Fr& b) { return to_mont(mont(a, b)); }
// (r + 1) / 2, the inverse of 2
constexpr uint64_t kInv2[4] = {0xa1f0fac9f8000001ull, 0x9419f4243cdcb848ull, 0xdc2822db40c0ac2eull,
                               0x183227397098d014ull};
inline Fr from_mont(const Fr& a) { return mont(a, Fr{{1, 0, 0, 0}}); }
// f0 + r (f1 - f0), all in the same (Montgomery) form.
inline Fr fold_mont(const Fr& f0, const Fr& f1, const Fr& r_mont) { return add(f0, mont(sub(f1, f0), r_mont)); }

// 32 little-endian bytes reduced mod r (2^256 < 6r: at most five subtractions).
inline Fr from_bytes(const uint8_t* in) {
    Fr r;
    for (int i = 0; i < 4; i++) {
        uint64_t x = 0;
        for (int k = 7; k >= 0; k--) x = (x << 8) | in[8 * i + k];
        r.v[i] = x;
    }
    while (geq_r(r.v)) sub_r(r.v);
    return r;
}
inline void to_bytes(const Fr& a, uint8_t* out) {
    for (int i = 0; i < 4; i++)
        for (int k = 0; k < 8; k++) out[8 * i + k] = (uint8_t)(a.v[i] >> (8 * k));
}
// Element of a little-endian u32 limb array (the device layout).
inline Fr load(const uint32_t* p) {
    Fr r;
    for (int i = 0; i < 4; i++) r.v[i] = (uint64_t)p[2 * i] | ((uint64_t)p[2 * i + 1] << 32);
    return r;
}
inline void store(const Fr& a, uint32_t* p) {
    for (int i = 0; i < 4; i++) {
        p[2 * i] = (uint32_t)a.v[i];
        p[2 * i + 1] = (uint32_t)(a.v[i] >> 32);
    }
}

}  // namespace frh
}  // namespace gkrgpu
