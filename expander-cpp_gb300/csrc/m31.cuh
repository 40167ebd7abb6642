// M31 field arithmetic (p = 2^31 - 1) for host and device.
//
// Every function maps canonical inputs in [0, p) to the canonical result, which is the
// value the reference's scalar and packed operators produce (include/field/M31.hpp:64-93,
// include/field/M31_avx.tcc:97-176): field results are unique, so the proof bytes do
// not depend on how a sum is ordered or split across threads.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define GKR_HD __host__ __device__ __forceinline__
#else
#define GKR_HD inline
#endif

namespace m31 {

static constexpr uint32_t P = 2147483647u;

GKR_HD uint32_t umin(uint32_t a, uint32_t b) { return a < b ? a : b; }

// a + b: the sum is < 2^32; min(s, s - p) picks s - p exactly when s >= p.
GKR_HD uint32_t add(uint32_t a, uint32_t b) {
    uint32_t s = a + b;
    return umin(s, s - P);
}

// a - b: d wraps to a value > p when a < b, and then d + p (mod 2^32) is the smaller one.
GKR_HD uint32_t sub(uint32_t a, uint32_t b) {
    uint32_t d = a - b;
    return umin(d, d + P);
}

// Mersenne reduction of a 62-bit product: x = hi * 2^31 + lo == hi + lo (mod p).
// lo + hi <= p + 2^31 - 2 < 2p, so one conditional subtraction finishes it.
GKR_HD uint32_t reduce62(uint64_t x) {
    uint32_t s = (uint32_t)(x & P) + (uint32_t)(x >> 31);
    return umin(s, s - P);
}

GKR_HD uint32_t mul(uint32_t a, uint32_t b) { return reduce62((uint64_t)a * b); }

// Canonical form of an arbitrary u32 (M31::from_bytes, include/field/M31.hpp:111-116).
GKR_HD uint32_t from_u32(uint32_t x) {
    uint32_t s = (x & P) + (x >> 31);
    return umin(s, s - P);
}

// acc + a * b (mod p) for any acc < 2^32 and canonical a, b, left unreduced below 2^32:
// a * b <= (p - 1)^2 = 2^62 - 2^33 + 4, so t = acc + a * b < 2^62, t >> 31 < 2^31 and
// (t & p) + (t >> 31) <= 2^32 - 2.  Chains of these stay below 2^32; from_u32 finishes.
GKR_HD uint32_t mac_lazy(uint32_t acc, uint32_t a, uint32_t b) {
    const uint64_t t = (uint64_t)a * b + acc;
    return (uint32_t)(t & P) + (uint32_t)(t >> 31);
}

// a + (b - a) * r: the fold of a multilinear table at challenge r
// (SumcheckMultiLinearProdHelper::receive_challenge, sumcheck_helper.hpp:115,124-125).
GKR_HD uint32_t fold(uint32_t a, uint32_t b, uint32_t r) { return add(a, mul(sub(b, a), r)); }

// Evaluation at 2 of the degree-2 round polynomial from p0 = h(0), p1 = h(1) and
// p2raw = sum (f0+f1)(g0+g1) = 4 h(1/2): 6 p1 + 3 p0 - 2 p2raw (sumcheck_helper.hpp:100).
GKR_HD uint32_t eval_at_two(uint32_t p0, uint32_t p1, uint32_t p2raw) {
    return sub(add(mul(p1, 6), mul(p0, 3)), mul(p2raw, 2));
}

// The degree-2 polynomial through (0, v0), (1, v1), (2, v2) evaluated at x: the claim the
// next sumcheck round must meet (degree_2_eval, sumcheck_verifier_utils.hpp:10-18).  2^30 is
// the inverse of 2 (2 * 2^30 = p + 1).
GKR_HD uint32_t eval_degree2(uint32_t v0, uint32_t v1, uint32_t v2, uint32_t x) {
    const uint32_t c2 = mul(1u << 30, add(sub(v2, add(v1, v1)), v0));
    const uint32_t c1 = sub(sub(v1, v0), c2);
    return add(v0, mul(add(mul(c2, x), c1), x));
}

}  // namespace m31
