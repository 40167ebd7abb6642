/* Test infrastructure only: BN254 scalar field (r = 0x30644e72...f0000001) for the oracle.
 *
 * The reference declares a BN254 field type (include/configuration/config.hpp:12-16,53-55)
 * but ships no implementation (its field/bn254_fr.hpp is missing from the tree), so the
 * encoding here is this project's definition, shared by the oracle driver and checked
 * against Python big integers by tests/test_bn254.py:
 *   - an element is a canonical integer in [0, r), serialised as 32 little-endian bytes;
 *   - from_bytes reads 32 little-endian bytes and reduces the integer mod r (this is how a
 *     SHA-256 digest becomes a challenge);
 *   - arithmetic is modular; internally products use Montgomery reduction with R = 2^256.
 */
#ifndef ORACLE_BN254_H
#define ORACLE_BN254_H

#include <stdint.h>
#include <string.h>

typedef struct {
    uint64_t v[4];
} bn_t;

typedef unsigned __int128 bn_u128;

static const uint64_t BN_R[4] = {0x43e1f593f0000001ull, 0x2833e84879b97091ull, 0xb85045b68181585dull,
                                 0x30644e72e131a029ull};
static const uint64_t BN_NPRIME = 0xc2e1f593efffffffull; /* -r^-1 mod 2^64 */
static const uint64_t BN_R2[4] = {0x1bb8e645ae216da7ull, 0x53fe3ab1e35c59e3ull, 0x8c49833d53bb8085ull,
                                  0x0216d0b17f4e44a5ull}; /* 2^512 mod r */

static inline int bn_geq_r(const uint64_t a[4]) {
    for (int i = 3; i >= 0; i--) {
        if (a[i] > BN_R[i]) return 1;
        if (a[i] < BN_R[i]) return 0;
    }
    return 1;
}
static inline void bn_sub_r(uint64_t a[4]) {
    uint64_t borrow = 0;
    for (int i = 0; i < 4; i++) {
        bn_u128 d = (bn_u128)a[i] - BN_R[i] - borrow;
        a[i] = (uint64_t)d;
        borrow = (uint64_t)(d >> 64) & 1;
    }
}
static inline bn_t bn_add(bn_t a, bn_t b) {
    bn_t c;
    uint64_t carry = 0;
    for (int i = 0; i < 4; i++) {
        bn_u128 s = (bn_u128)a.v[i] + b.v[i] + carry;
        c.v[i] = (uint64_t)s;
        carry = (uint64_t)(s >> 64);
    }
    if (carry || bn_geq_r(c.v)) bn_sub_r(c.v);
    return c;
}
static inline bn_t bn_sub(bn_t a, bn_t b) {
    bn_t c;
    uint64_t borrow = 0;
    for (int i = 0; i < 4; i++) {
        bn_u128 d = (bn_u128)a.v[i] - b.v[i] - borrow;
        c.v[i] = (uint64_t)d;
        borrow = (uint64_t)(d >> 64) & 1;
    }
    if (borrow) {
        uint64_t carry = 0;
        for (int i = 0; i < 4; i++) {
            bn_u128 s = (bn_u128)c.v[i] + BN_R[i] + carry;
            c.v[i] = (uint64_t)s;
            carry = (uint64_t)(s >> 64);
        }
    }
    return c;
}
static inline bn_t bn_neg(bn_t a) {
    bn_t z = {{0, 0, 0, 0}};
    return bn_sub(z, a);
}
/* Montgomery product a*b*2^-256 mod r (CIOS), inputs < r. */
static inline bn_t bn_mont(bn_t a, bn_t b) {
    uint64_t t[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < 4; i++) {
        uint64_t c = 0;
        for (int j = 0; j < 4; j++) {
            bn_u128 p = (bn_u128)a.v[j] * b.v[i] + t[j] + c;
            t[j] = (uint64_t)p;
            c = (uint64_t)(p >> 64);
        }
        bn_u128 s = (bn_u128)t[4] + c;
        t[4] = (uint64_t)s;
        t[5] = (uint64_t)(s >> 64);
        uint64_t m = t[0] * BN_NPRIME;
        bn_u128 p = (bn_u128)m * BN_R[0] + t[0];
        c = (uint64_t)(p >> 64);
        for (int j = 1; j < 4; j++) {
            p = (bn_u128)m * BN_R[j] + t[j] + c;
            t[j - 1] = (uint64_t)p;
            c = (uint64_t)(p >> 64);
        }
        s = (bn_u128)t[4] + c;
        t[3] = (uint64_t)s;
        t[4] = t[5] + (uint64_t)(s >> 64);
    }
    bn_t r;
    memcpy(r.v, t, 32);
    if (t[4] || bn_geq_r(r.v)) bn_sub_r(r.v);
    return r;
}
/* a*b mod r for canonical a, b: (a*b*R^-1) * R^2 * R^-1. */
static inline bn_t bn_mul(bn_t a, bn_t b) {
    bn_t r2;
    memcpy(r2.v, BN_R2, 32);
    return bn_mont(bn_mont(a, b), r2);
}
static inline bn_t bn_from_u32(uint32_t x) {
    bn_t r = {{x, 0, 0, 0}};
    return r;
}
static inline void bn_to_bytes(bn_t a, uint8_t out[32]) {
    for (int i = 0; i < 4; i++)
        for (int k = 0; k < 8; k++) out[8 * i + k] = (uint8_t)(a.v[i] >> (8 * k));
}
/* 32 little-endian bytes reduced mod r (2^256 / r < 6, so at most 5 subtractions). */
static inline bn_t bn_from_bytes(const uint8_t in[32]) {
    bn_t r;
    for (int i = 0; i < 4; i++) {
        uint64_t x = 0;
        for (int k = 7; k >= 0; k--) x = (x << 8) | in[8 * i + k];
        r.v[i] = x;
    }
    while (bn_geq_r(r.v)) bn_sub_r(r.v);
    return r;
}
static inline int bn_eq(bn_t a, bn_t b) { return memcmp(a.v, b.v, 32) == 0; }

#endif
