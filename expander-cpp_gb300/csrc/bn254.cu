// BN254 scalar-field kernels (see bn254.cuh).  Same algorithms as the M31 kernels in
// kernels.cu, for one repetition (R = 1 for BN254, include/configuration/config.hpp:61-65),
// with 256-bit elements: one thread per element of a row, Montgomery multiplication on
// 8 x 32-bit limbs (CIOS as PTX multiply-add carry chains).
#include "bn254.cuh"

namespace gkrgpu {
namespace bn {

namespace {

// r = 0x30644e72e131a029b85045b68181585d2833e84879b9709143e1f593f0000001 (little-endian
// limbs 0xf0000001, 0x43e1f593, ... appear as immediates in the PTX below), -r^-1 mod 2^32 =
// 0xefffffff.
__constant__ uint32_t kOne[8] = {0x4ffffffbu, 0xac96341cu, 0x9f60cd29u, 0x36fc7695u,
                                 0x7879462eu, 0x666ea36fu, 0x9a07df2fu, 0x0e0a77c1u};  // 2^256 mod r
__constant__ uint32_t kR2[8] = {0xae216da7u, 0x1bb8e645u, 0xe35c59e3u, 0x53fe3ab1u,
                                0x53bb8085u, 0x8c49833du, 0x7f4e44a5u, 0x0216d0b1u};  // 2^512 mod r
__constant__ uint32_t kInv2M[8] = {0x1ffffffeu, 0x783c14d8u, 0x0c8d1eddu, 0xaf982f6fu,
                                   0xfcfd4f45u, 0x8f5f7492u, 0x3d9cbfacu, 0x1f37631au};  // (r + 1) / 2 * 2^256 mod r

__device__ __forceinline__ Fr zero() {
    Fr z;
#pragma unroll
    for (int i = 0; i < 8; i++) z.l[i] = 0u;
    return z;
}
__device__ __forceinline__ Fr one() {
    Fr z;
#pragma unroll
    for (int i = 0; i < 8; i++) z.l[i] = kOne[i];
    return z;
}
// Field operations on canonical Montgomery forms (< r) as PTX carry chains (add.cc/addc,
// mad.lo.cc/madc.hi.cc); each asm block holds a whole chain, so no carry flag crosses
// statements.  The modulus limbs are immediates.

// x - r with a borrow chain; returns the borrow-out word (0xffffffff when x < r).
__device__ __forceinline__ uint32_t minus_r(const uint32_t* x, uint32_t* d) {
    uint32_t bw;
    asm("sub.cc.u32 %0, %9, 0xf0000001;\n\t"
        "subc.cc.u32 %1, %10, 0x43e1f593;\n\t"
        "subc.cc.u32 %2, %11, 0x79b97091;\n\t"
        "subc.cc.u32 %3, %12, 0x2833e848;\n\t"
        "subc.cc.u32 %4, %13, 0x8181585d;\n\t"
        "subc.cc.u32 %5, %14, 0xb85045b6;\n\t"
        "subc.cc.u32 %6, %15, 0xe131a029;\n\t"
        "subc.cc.u32 %7, %16, 0x30644e72;\n\t"
        "subc.u32 %8, 0, 0;"
        : "=r"(d[0]), "=r"(d[1]), "=r"(d[2]), "=r"(d[3]), "=r"(d[4]), "=r"(d[5]), "=r"(d[6]), "=r"(d[7]), "=r"(bw)
        : "r"(x[0]), "r"(x[1]), "r"(x[2]), "r"(x[3]), "r"(x[4]), "r"(x[5]), "r"(x[6]), "r"(x[7]));
    return bw;
}

__device__ __forceinline__ Fr add(const Fr& a, const Fr& b) {
    uint32_t s[8], d[8];
    // a + b < 2r < 2^255: no carry out of the top limb
    asm("add.cc.u32 %0, %8, %16;\n\t"
        "addc.cc.u32 %1, %9, %17;\n\t"
        "addc.cc.u32 %2, %10, %18;\n\t"
        "addc.cc.u32 %3, %11, %19;\n\t"
        "addc.cc.u32 %4, %12, %20;\n\t"
        "addc.cc.u32 %5, %13, %21;\n\t"
        "addc.cc.u32 %6, %14, %22;\n\t"
        "addc.u32 %7, %15, %23;"
        : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6]), "=r"(s[7])
        : "r"(a.l[0]), "r"(a.l[1]), "r"(a.l[2]), "r"(a.l[3]), "r"(a.l[4]), "r"(a.l[5]), "r"(a.l[6]), "r"(a.l[7]),
          "r"(b.l[0]), "r"(b.l[1]), "r"(b.l[2]), "r"(b.l[3]), "r"(b.l[4]), "r"(b.l[5]), "r"(b.l[6]), "r"(b.l[7]));
    const bool below = minus_r(s, d) != 0u;
    Fr o;
#pragma unroll
    for (int i = 0; i < 8; i++) o.l[i] = below ? s[i] : d[i];
    return o;
}
__device__ __forceinline__ Fr sub(const Fr& a, const Fr& b) {
    uint32_t d[8], bw;
    asm("sub.cc.u32 %0, %9, %17;\n\t"
        "subc.cc.u32 %1, %10, %18;\n\t"
        "subc.cc.u32 %2, %11, %19;\n\t"
        "subc.cc.u32 %3, %12, %20;\n\t"
        "subc.cc.u32 %4, %13, %21;\n\t"
        "subc.cc.u32 %5, %14, %22;\n\t"
        "subc.cc.u32 %6, %15, %23;\n\t"
        "subc.cc.u32 %7, %16, %24;\n\t"
        "subc.u32 %8, 0, 0;"
        : "=r"(d[0]), "=r"(d[1]), "=r"(d[2]), "=r"(d[3]), "=r"(d[4]), "=r"(d[5]), "=r"(d[6]), "=r"(d[7]), "=r"(bw)
        : "r"(a.l[0]), "r"(a.l[1]), "r"(a.l[2]), "r"(a.l[3]), "r"(a.l[4]), "r"(a.l[5]), "r"(a.l[6]), "r"(a.l[7]),
          "r"(b.l[0]), "r"(b.l[1]), "r"(b.l[2]), "r"(b.l[3]), "r"(b.l[4]), "r"(b.l[5]), "r"(b.l[6]), "r"(b.l[7]));
    // a < b: add r back (bw is all ones, masking r's limbs)
    Fr o;
    asm("{\n\t.reg .u32 m0, m1, m2, m3, m4, m5, m6, m7;\n\t"
        "and.b32 m0, %16, 0xf0000001;\n\t"
        "and.b32 m1, %16, 0x43e1f593;\n\t"
        "and.b32 m2, %16, 0x79b97091;\n\t"
        "and.b32 m3, %16, 0x2833e848;\n\t"
        "and.b32 m4, %16, 0x8181585d;\n\t"
        "and.b32 m5, %16, 0xb85045b6;\n\t"
        "and.b32 m6, %16, 0xe131a029;\n\t"
        "and.b32 m7, %16, 0x30644e72;\n\t"
        "add.cc.u32 %0, %8, m0;\n\t"
        "addc.cc.u32 %1, %9, m1;\n\t"
        "addc.cc.u32 %2, %10, m2;\n\t"
        "addc.cc.u32 %3, %11, m3;\n\t"
        "addc.cc.u32 %4, %12, m4;\n\t"
        "addc.cc.u32 %5, %13, m5;\n\t"
        "addc.cc.u32 %6, %14, m6;\n\t"
        "addc.u32 %7, %15, m7;\n\t"
        "}"
        : "=r"(o.l[0]), "=r"(o.l[1]), "=r"(o.l[2]), "=r"(o.l[3]), "=r"(o.l[4]), "=r"(o.l[5]), "=r"(o.l[6]),
          "=r"(o.l[7])
        : "r"(d[0]), "r"(d[1]), "r"(d[2]), "r"(d[3]), "r"(d[4]), "r"(d[5]), "r"(d[6]), "r"(d[7]), "r"(bw));
    return o;
}

// One CIOS step (Koc, Acar, Kaliski 1996): t += a * bi, then t += m * r with
// m = t0 * (-r^-1) mod 2^32, which clears t0.  t0..t9 are %0..%9, a is %10..%17, bi %18.
#define GKRGPU_BN_CIOS_STEP                      \
    "{\n\t.reg .u32 m;\n\t"                      \
    "mad.lo.cc.u32 %0, %10, %18, %0;\n\t"        \
    "madc.lo.cc.u32 %1, %11, %18, %1;\n\t"       \
    "madc.lo.cc.u32 %2, %12, %18, %2;\n\t"       \
    "madc.lo.cc.u32 %3, %13, %18, %3;\n\t"       \
    "madc.lo.cc.u32 %4, %14, %18, %4;\n\t"       \
    "madc.lo.cc.u32 %5, %15, %18, %5;\n\t"       \
    "madc.lo.cc.u32 %6, %16, %18, %6;\n\t"       \
    "madc.lo.cc.u32 %7, %17, %18, %7;\n\t"       \
    "addc.cc.u32 %8, %8, 0;\n\t"                 \
    "addc.u32 %9, 0, 0;\n\t"                     \
    "mad.hi.cc.u32 %1, %10, %18, %1;\n\t"        \
    "madc.hi.cc.u32 %2, %11, %18, %2;\n\t"       \
    "madc.hi.cc.u32 %3, %12, %18, %3;\n\t"       \
    "madc.hi.cc.u32 %4, %13, %18, %4;\n\t"       \
    "madc.hi.cc.u32 %5, %14, %18, %5;\n\t"       \
    "madc.hi.cc.u32 %6, %15, %18, %6;\n\t"       \
    "madc.hi.cc.u32 %7, %16, %18, %7;\n\t"       \
    "madc.hi.cc.u32 %8, %17, %18, %8;\n\t"       \
    "addc.u32 %9, %9, 0;\n\t"                    \
    "mul.lo.u32 m, %0, 0xefffffff;\n\t"          \
    "mad.lo.cc.u32 %0, m, 0xf0000001, %0;\n\t"   \
    "madc.lo.cc.u32 %1, m, 0x43e1f593, %1;\n\t"  \
    "madc.lo.cc.u32 %2, m, 0x79b97091, %2;\n\t"  \
    "madc.lo.cc.u32 %3, m, 0x2833e848, %3;\n\t"  \
    "madc.lo.cc.u32 %4, m, 0x8181585d, %4;\n\t"  \
    "madc.lo.cc.u32 %5, m, 0xb85045b6, %5;\n\t"  \
    "madc.lo.cc.u32 %6, m, 0xe131a029, %6;\n\t"  \
    "madc.lo.cc.u32 %7, m, 0x30644e72, %7;\n\t"  \
    "addc.cc.u32 %8, %8, 0;\n\t"                 \
    "addc.u32 %9, %9, 0;\n\t"                    \
    "mad.hi.cc.u32 %1, m, 0xf0000001, %1;\n\t"   \
    "madc.hi.cc.u32 %2, m, 0x43e1f593, %2;\n\t"  \
    "madc.hi.cc.u32 %3, m, 0x79b97091, %3;\n\t"  \
    "madc.hi.cc.u32 %4, m, 0x2833e848, %4;\n\t"  \
    "madc.hi.cc.u32 %5, m, 0x8181585d, %5;\n\t"  \
    "madc.hi.cc.u32 %6, m, 0xb85045b6, %6;\n\t"  \
    "madc.hi.cc.u32 %7, m, 0xe131a029, %7;\n\t"  \
    "madc.hi.cc.u32 %8, m, 0x30644e72, %8;\n\t"  \
    "addc.u32 %9, %9, 0;\n\t"                    \
    "}"

// Montgomery product a * b * 2^-256 mod r (inputs < r, output < r).
__device__ __forceinline__ Fr mul(const Fr& a, const Fr& b) {
    uint32_t t0 = 0, t1 = 0, t2 = 0, t3 = 0, t4 = 0, t5 = 0, t6 = 0, t7 = 0, t8 = 0, t9 = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        asm(GKRGPU_BN_CIOS_STEP
            : "+r"(t0), "+r"(t1), "+r"(t2), "+r"(t3), "+r"(t4), "+r"(t5), "+r"(t6), "+r"(t7), "+r"(t8), "+r"(t9)
            : "r"(a.l[0]), "r"(a.l[1]), "r"(a.l[2]), "r"(a.l[3]), "r"(a.l[4]), "r"(a.l[5]), "r"(a.l[6]),
              "r"(a.l[7]), "r"(b.l[i]));
        // divide by 2^32: t0 is zero
        t0 = t1; t1 = t2; t2 = t3; t3 = t4; t4 = t5; t5 = t6; t6 = t7; t7 = t8; t8 = t9; t9 = 0;
    }
    // t < 2r < 2^255, so t8 is 0: one conditional subtraction of r
    const uint32_t t[8] = {t0, t1, t2, t3, t4, t5, t6, t7};
    uint32_t d[8];
    const bool below = minus_r(t, d) != 0u;
    Fr o;
#pragma unroll
    for (int i = 0; i < 8; i++) o.l[i] = below ? t[i] : d[i];
    return o;
}
#undef GKRGPU_BN_CIOS_STEP
__device__ __forceinline__ Fr from_mont(const Fr& a) {
    Fr u = zero();
    u.l[0] = 1u;
    return mul(a, u);
}
__device__ __forceinline__ Fr to_mont(const Fr& a) {
    Fr r2;
#pragma unroll
    for (int i = 0; i < 8; i++) r2.l[i] = kR2[i];
    return mul(a, r2);
}
__device__ __forceinline__ Fr fold(const Fr& a, const Fr& b, const Fr& r) { return add(a, mul(sub(b, a), r)); }

// The canonical value of a sum of Montgomery forms given as 64-bit limb sums:
// T = sum_k s[k] 2^(32k) is the sum of the x_i R (R = 2^256), so REDC(T) = T R^-1 mod r is
// sum x_i, already canonical after one conditional subtraction (T < 2^266 keeps
// REDC(T) < 2r).  Eight reduction steps of CIOS on a ten-word window.
__device__ __forceinline__ Fr redc_sums(const unsigned long long* s) {
    uint32_t t0, t1, t2, t3, t4, t5, t6, t7, t8, t9;
    {
        uint32_t w[10];
        unsigned long long c = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const unsigned long long lo = c + (s[k] & 0xffffffffull);
            w[k] = (uint32_t)lo;
            c = (lo >> 32) + (s[k] >> 32);
        }
        w[8] = (uint32_t)c;
        w[9] = (uint32_t)(c >> 32);
        t0 = w[0]; t1 = w[1]; t2 = w[2]; t3 = w[3]; t4 = w[4];
        t5 = w[5]; t6 = w[6]; t7 = w[7]; t8 = w[8]; t9 = w[9];
    }
#pragma unroll
    for (int i = 0; i < 8; i++) {
        asm("{\n\t.reg .u32 m;\n\t"
            "mul.lo.u32 m, %0, 0xefffffff;\n\t"
            "mad.lo.cc.u32 %0, m, 0xf0000001, %0;\n\t"
            "madc.lo.cc.u32 %1, m, 0x43e1f593, %1;\n\t"
            "madc.lo.cc.u32 %2, m, 0x79b97091, %2;\n\t"
            "madc.lo.cc.u32 %3, m, 0x2833e848, %3;\n\t"
            "madc.lo.cc.u32 %4, m, 0x8181585d, %4;\n\t"
            "madc.lo.cc.u32 %5, m, 0xb85045b6, %5;\n\t"
            "madc.lo.cc.u32 %6, m, 0xe131a029, %6;\n\t"
            "madc.lo.cc.u32 %7, m, 0x30644e72, %7;\n\t"
            "addc.cc.u32 %8, %8, 0;\n\t"
            "addc.u32 %9, %9, 0;\n\t"
            "mad.hi.cc.u32 %1, m, 0xf0000001, %1;\n\t"
            "madc.hi.cc.u32 %2, m, 0x43e1f593, %2;\n\t"
            "madc.hi.cc.u32 %3, m, 0x79b97091, %3;\n\t"
            "madc.hi.cc.u32 %4, m, 0x2833e848, %4;\n\t"
            "madc.hi.cc.u32 %5, m, 0x8181585d, %5;\n\t"
            "madc.hi.cc.u32 %6, m, 0xb85045b6, %6;\n\t"
            "madc.hi.cc.u32 %7, m, 0xe131a029, %7;\n\t"
            "madc.hi.cc.u32 %8, m, 0x30644e72, %8;\n\t"
            "addc.u32 %9, %9, 0;\n\t"
            "}"
            : "+r"(t0), "+r"(t1), "+r"(t2), "+r"(t3), "+r"(t4), "+r"(t5), "+r"(t6), "+r"(t7), "+r"(t8), "+r"(t9));
        t0 = t1; t1 = t2; t2 = t3; t3 = t4; t4 = t5; t5 = t6; t6 = t7; t7 = t8; t8 = t9; t9 = 0;
    }
    const uint32_t t[8] = {t0, t1, t2, t3, t4, t5, t6, t7};
    uint32_t d[8];
    const bool below = minus_r(t, d) != 0u;
    Fr o;
#pragma unroll
    for (int i = 0; i < 8; i++) o.l[i] = below ? t[i] : d[i];
    return o;
}

__device__ __forceinline__ Fr ldf(const uint32_t* __restrict__ base, uint64_t row, uint32_t N, uint32_t lane) {
    const uint4* p = reinterpret_cast<const uint4*>(base + (row * N + lane) * 8);
    const uint4 a = __ldg(p), b = __ldg(p + 1);
    Fr f;
    f.l[0] = a.x; f.l[1] = a.y; f.l[2] = a.z; f.l[3] = a.w;
    f.l[4] = b.x; f.l[5] = b.y; f.l[6] = b.z; f.l[7] = b.w;
    return f;
}
__device__ __forceinline__ void stf(uint32_t* base, uint64_t row, uint32_t N, uint32_t lane, const Fr& f) {
    uint4* p = reinterpret_cast<uint4*>(base + (row * N + lane) * 8);
    p[0] = make_uint4(f.l[0], f.l[1], f.l[2], f.l[3]);
    p[1] = make_uint4(f.l[4], f.l[5], f.l[6], f.l[7]);
}
__device__ __forceinline__ Fr lds(const Fr* __restrict__ t, uint64_t i) {
    const uint4* p = reinterpret_cast<const uint4*>(t + i);
    const uint4 a = __ldg(p), b = __ldg(p + 1);
    Fr f;
    f.l[0] = a.x; f.l[1] = a.y; f.l[2] = a.z; f.l[3] = a.w;
    f.l[4] = b.x; f.l[5] = b.y; f.l[6] = b.z; f.l[7] = b.w;
    return f;
}
__device__ __forceinline__ void sts(Fr* t, uint64_t i, const Fr& f) {
    uint4* p = reinterpret_cast<uint4*>(t + i);
    p[0] = make_uint4(f.l[0], f.l[1], f.l[2], f.l[3]);
    p[1] = make_uint4(f.l[4], f.l[5], f.l[6], f.l[7]);
}

struct Tile {
    uint32_t q, rs;
    bool active;
};
__device__ __forceinline__ Tile tile(const GeoBn& g) {
    Tile t;
    t.q = blockIdx.y * g.tpr + threadIdx.x % g.tpr;  // lane
    t.rs = threadIdx.x / g.tpr;
    t.active = t.rs < g.rps;
    return t;
}

// Canonical total of component c of one lane; leaves its accumulators zeroed.
__device__ __noinline__ Fr take(const RedBn& red, uint32_t c, uint32_t N, uint32_t lane) {
    unsigned long long s[8];
    unsigned long long* p = &red.acc[((size_t)c * N + lane) * 8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        s[k] = __ldcg(p + k);
        p[k] = 0ull;
    }
    return redc_sums(s);
}

// C components per thread -> shared-memory sum over the CTA's row slices -> 64-bit
// atomic adds per limb -> the last CTA of the lane group finishes its lanes: one thread per
// (component, lane) total, then fin(c, lane, totals of the lane, tpr) per output value.
template <int C, class Fin>
__device__ __forceinline__ void reduce_bn(Fr (&acc)[C], const GeoBn& g, bool active, RedBn red, Fin fin) {
    extern __shared__ uint32_t smem[];
    const uint32_t tid = threadIdx.x, B = blockDim.x;
    uint32_t rows = g.rps;
    if (g.tpr < 32 && (g.tpr & (g.tpr - 1)) == 0) {
        // power-of-two tile below a warp (every thread active): first fold the warp's row
        // slices together with shuffles, leaving one row per warp
        for (uint32_t off = g.tpr; off < 32; off <<= 1)
#pragma unroll
            for (int c = 0; c < C; c++) {
                Fr o;
#pragma unroll
                for (int k = 0; k < 8; k++) o.l[k] = __shfl_xor_sync(0xffffffffu, acc[c].l[k], off);
                acc[c] = add(acc[c], o);
            }
        rows = B / 32;
        if ((tid & 31) < g.tpr)
#pragma unroll
            for (int c = 0; c < C; c++)
#pragma unroll
                for (int k = 0; k < 8; k++) smem[(c * 8 + k) * B + (tid >> 5) * g.tpr + (tid & 31)] = acc[c].l[k];
    } else {
#pragma unroll
        for (int c = 0; c < C; c++)
#pragma unroll
            for (int k = 0; k < 8; k++) smem[(c * 8 + k) * B + tid] = active ? acc[c].l[k] : 0u;
    }
    __syncthreads();
    for (uint32_t o = tid; o < (uint32_t)C * g.tpr; o += B) {
        const uint32_t c = o / g.tpr, q = o - c * g.tpr;
        Fr s = zero();
        for (uint32_t r = 0; r < rows; r++) {
            Fr x;
#pragma unroll
            for (int k = 0; k < 8; k++) x.l[k] = smem[(c * 8 + k) * B + r * g.tpr + q];
            s = add(s, x);
        }
        const uint32_t lane = blockIdx.y * g.tpr + q;
#pragma unroll
        for (int k = 0; k < 8; k++) atomicAdd(&red.acc[((size_t)c * g.N + lane) * 8 + k], (unsigned long long)s.l[k]);
    }
    __threadfence();
    __syncthreads();
    __shared__ unsigned int is_last;
    if (tid == 0) is_last = (atomicAdd(&red.ticket[blockIdx.y], 1u) == gridDim.x - 1) ? 1u : 0u;
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    // the last CTA: every (component, lane) total is reduced by its own thread, then each
    // output value is finished by its own thread (the finisher's chains run in parallel)
    Fr* tot = reinterpret_cast<Fr*>(smem);
    for (uint32_t o = tid; o < (uint32_t)C * g.tpr; o += B) {
        const uint32_t c = o / g.tpr, li = o - c * g.tpr;
        tot[o] = take(red, c, g.N, blockIdx.y * g.tpr + li);
    }
    __syncthreads();
    for (uint32_t o = tid; o < (uint32_t)C * g.tpr; o += B) {
        const uint32_t c = o / g.tpr, li = o - c * g.tpr;
        fin(c, blockIdx.y * g.tpr + li, tot + li, g.tpr);
    }
    if (tid == 0) red.ticket[blockIdx.y] = 0u;
    if (red.done) {
        __threadfence_system();
        __syncthreads();
        if (tid == 0) atomicAdd_system(red.done, 1u);
    }
}

// Output c of one lane from the canonical totals t[0], t[tpr], t[2 tpr] (components 0..2 of
// that lane): the evaluations at 0, 1 and 2 (6 p1 + 3 p0 - 2 p2raw).  Phase two multiplies
// by vx: a Montgomery product of a canonical value with vx's Montgomery form is the
// canonical product.
struct RoundFinBn {
    uint32_t* out;  // 3 x N x 8 limbs, canonical
    const uint32_t* vx;
    uint32_t N;
    uint32_t* dev = nullptr;  // device copy of out, or null
    __device__ __noinline__ void operator()(uint32_t c, uint32_t lane, const Fr* t, uint32_t tpr) const {
        Fr v;
        if (c < 2) {
            v = t[c * tpr];
        } else {
            const Fr p0 = t[0], p1 = t[tpr], p2r = t[2 * tpr];
            const Fr p1x2 = add(p1, p1);
            v = add(add(p1x2, p1x2), p1x2);       // 6 p1
            v = add(v, add(add(p0, p0), p0));    // + 3 p0
            v = sub(v, add(p2r, p2r));            // - 2 p2raw
        }
        if (vx) v = mul(v, ldf(vx, 0, N, lane));
        stf(out, c, N, lane, v);
        if (dev) stf(dev, c, N, lane, v);
    }
};

// Element of a host-written table read past the caches (each limb fetched again).
__device__ __forceinline__ Fr ldf_cv(const uint32_t* base, uint32_t N, uint32_t lane) {
    Fr f;
#pragma unroll
    for (int k = 0; k < 8; k++) f.l[k] = __ldcv(base + (size_t)lane * 8 + k);
    return f;
}

// The round's evaluations from two components per lane, p0 (t[0]) and p2raw (t[tpr]): p1 is
// the round's claim less p0 (an honest prover's round polynomial meets p0 + p1 = claim, the
// verifier's check in sumcheck.hpp:152).  The claim is `claim` (N x 8 words, host-written),
// or the previous round's polynomial at its challenge r (Montgomery form), degree_2_eval
// (sumcheck_verifier_utils.hpp:10-18) of its evaluations in `prev`.  Component 0 writes the
// evaluations at 0 and 1, component 1 the one at 2; with vx (phase two) the sums are
// multiplied by v(rx) first.  Canonical values times Montgomery forms give canonical values.
struct ClaimFinBn {
    uint32_t* out;          // 3 x N x 8 limbs, canonical
    uint32_t* dev;          // device copy of out, or null
    const uint32_t* claim;  // N x 8, or null
    const uint32_t* prev;   // 3 x N x 8, or null
    const uint32_t* vx;
    Fr r;
    uint32_t N;
    __device__ __noinline__ void operator()(uint32_t c, uint32_t lane, const Fr* t, uint32_t tpr) const {
        Fr cl;
        if (claim) {
            cl = ldf_cv(claim, N, lane);
        } else {
            const Fr v0 = ldf(prev, 0, N, lane), v1 = ldf(prev, 1, N, lane), v2 = ldf(prev, 2, N, lane);
            Fr inv2;
#pragma unroll
            for (int k = 0; k < 8; k++) inv2.l[k] = kInv2M[k];
            const Fr c2 = mul(add(sub(v2, add(v1, v1)), v0), inv2);
            const Fr c1 = sub(sub(v1, v0), c2);
            cl = add(v0, mul(add(mul(c2, r), c1), r));
        }
        Fr x = zero();
        if (vx) x = ldf(vx, 0, N, lane);
        Fr p0 = t[0];
        if (vx) p0 = mul(p0, x);
        const Fr p1 = sub(cl, p0);
        if (c == 0) {
            stf(out, 0, N, lane, p0);
            stf(out, 1, N, lane, p1);
            if (dev) {
                stf(dev, 0, N, lane, p0);
                stf(dev, 1, N, lane, p1);
            }
            return;
        }
        Fr p2r = t[tpr];
        if (vx) p2r = mul(p2r, x);
        const Fr p1x2 = add(p1, p1);
        Fr v = add(add(p1x2, p1x2), p1x2);    // 6 p1
        v = add(v, add(add(p0, p0), p0));     // + 3 p0
        v = sub(v, add(p2r, p2r));            // - 2 p2raw
        stf(out, 2, N, lane, v);
        if (dev) stf(dev, 2, N, lane, v);
    }
};

struct CopyFinBn {
    uint32_t* out;  // N x 8 limbs, canonical
    uint32_t N;
    __device__ void operator()(uint32_t, uint32_t lane, const Fr* t, uint32_t) const { stf(out, 0, N, lane, t[0]); }
};

__device__ __forceinline__ void accum(Fr (&acc)[3], const Fr& f0, const Fr& f1, const Fr& h0, const Fr& h1) {
    acc[0] = add(acc[0], mul(f0, h0));
    acc[1] = add(acc[1], mul(f1, h1));
    acc[2] = add(acc[2], mul(add(f0, f1), add(h0, h1)));
}
// p0 and p2raw only (the round's p1 comes from its claim: ClaimFinBn)
__device__ __forceinline__ void accum(Fr (&acc)[2], const Fr& f0, const Fr& f1, const Fr& h0, const Fr& h1) {
    acc[0] = add(acc[0], mul(f0, h0));
    acc[1] = add(acc[1], mul(add(f0, f1), add(h0, h1)));
}

// ---------------------------------------------------------------- kernels
// Input -> Montgomery table.  Canonical input (bad != null): an element >= r raises *bad
// and is stored as 0.  Otherwise every element is first reduced mod r (from_bytes of
// arbitrary 32-byte words: 2^256 < 6r, so at most five subtractions).
__global__ void k_load(const uint32_t* __restrict__ canon, uint32_t* __restrict__ mont, uint64_t n, unsigned int* bad) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        Fr x = lds(reinterpret_cast<const Fr*>(canon), i);
        uint32_t d[8];
        if (bad) {
            if (minus_r(x.l, d) == 0u) {  // no borrow: x >= r
                *reinterpret_cast<volatile unsigned int*>(bad) = 1u;  // every writer stores 1 (device or mapped flag)
                x = zero();
            }
        } else {
            for (int k = 0; k < 5 && minus_r(x.l, d) == 0u; k++)
#pragma unroll
                for (int q = 0; q < 8; q++) x.l[q] = d[q];
        }
        sts(reinterpret_cast<Fr*>(mont), i, to_mont(x));
    }
}

// Verifier gate sums (eval_sparse_circuit_connect_poly, one repetition): over the mul gates
// sum c eqz[o] eqx[i0] eqy[i1], or over the add gates sum c eqz[o] eqx[i0], walked by output
// (the evaluate CSR with Montgomery coefficients).  Thread sums -> warp shuffles -> shared
// memory -> 64-bit limb sums; the last block writes the canonical total (one REDC).
template <bool MUL>
__global__ void __launch_bounds__(256) k_gate_sums(uint64_t O, const uint32_t* __restrict__ off,
                                                   const uint32_t* __restrict__ gates, const Fr* __restrict__ coef,
                                                   const Fr* __restrict__ eqz, const Fr* __restrict__ eqx,
                                                   const Fr* __restrict__ eqy, unsigned long long* acc,
                                                   unsigned int* ticket, uint32_t* out) {
    Fr s = zero();
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t o = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; o < O; o += stride) {
        const uint32_t k0 = __ldg(off + o), k1 = __ldg(off + o + 1);
        if (k0 == k1) continue;
        const Fr ez = lds(eqz, o);
        for (uint32_t k = k0; k < k1; k++) {
            Fr t;
            if (MUL) {
                const uint4 g = __ldg(reinterpret_cast<const uint4*>(gates) + k);  // (i0, i1, c, 0)
                t = mul(mul(lds(eqx, g.x), lds(eqy, g.y)), lds(coef, k));
            } else {
                const uint2 g = __ldg(reinterpret_cast<const uint2*>(gates) + k);  // (i0, c)
                t = mul(lds(eqx, g.x), lds(coef, k));
            }
            s = add(s, mul(t, ez));
        }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        Fr o;
#pragma unroll
        for (int k = 0; k < 8; k++) o.l[k] = __shfl_xor_sync(0xffffffffu, s.l[k], d);
        s = add(s, o);
    }
    __shared__ Fr part[8];
    const uint32_t w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if ((threadIdx.x & 31) == 0) part[w] = s;
    __syncthreads();
    if (threadIdx.x < 8) {
        unsigned long long limb = 0;
        for (uint32_t q = 0; q < nw; q++) limb += part[q].l[threadIdx.x];
        atomicAdd(&acc[threadIdx.x], limb);
    }
    __threadfence();
    __syncthreads();
    __shared__ unsigned int is_last;
    if (threadIdx.x == 0) is_last = (atomicAdd(ticket, 1u) == gridDim.x - 1) ? 1u : 0u;
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    if (threadIdx.x == 0) {
        unsigned long long t[8];
#pragma unroll
        for (int k = 0; k < 8; k++) {
            t[k] = __ldcg(acc + k);
            acc[k] = 0ull;
        }
        const Fr r = redc_sums(t);
#pragma unroll
        for (int k = 0; k < 8; k++) out[k] = r.l[k];
        *ticket = 0u;
    }
}

// Montgomery -> canonical, in place.
__global__ void k_unload(uint32_t* v, uint64_t n) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    Fr* t = reinterpret_cast<Fr*>(v);
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint4* p = reinterpret_cast<const uint4*>(t + i);
        const uint4 a = p[0], b = p[1];
        Fr x;
        x.l[0] = a.x; x.l[1] = a.y; x.l[2] = a.z; x.l[3] = a.w;
        x.l[4] = b.x; x.l[5] = b.y; x.l[6] = b.z; x.l[7] = b.w;
        sts(t, i, from_mont(x));
    }
}

__global__ void __launch_bounds__(256) k_evaluate(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, uint64_t O,
                                                  const uint32_t* __restrict__ mo_off, const uint4* __restrict__ mo_g,
                                                  const Fr* __restrict__ mo_c, const uint32_t* __restrict__ ao_off,
                                                  const uint2* __restrict__ ao_g, const Fr* __restrict__ ao_c, GeoBn g) {
    const Tile t = tile(g);
    if (!t.active) return;
    for (uint64_t o = (uint64_t)blockIdx.x * g.rps + t.rs; o < O; o += (uint64_t)gridDim.x * g.rps) {
        Fr acc = zero();
        const uint32_t m0 = __ldg(mo_off + o), m1 = __ldg(mo_off + o + 1);
        for (uint32_t k = m0; k < m1; k++) {
            const uint4 gt = __ldg(mo_g + k);
            acc = add(acc, mul(mul(ldf(in, gt.x, g.N, t.q), ldf(in, gt.y, g.N, t.q)), lds(mo_c, k)));
        }
        const uint32_t a0 = __ldg(ao_off + o), a1 = __ldg(ao_off + o + 1);
        for (uint32_t k = a0; k < a1; k++) {
            const uint2 gt = __ldg(ao_g + k);
            acc = add(acc, mul(ldf(in, gt.x, g.N, t.q), lds(ao_c, k)));
        }
        stf(out, o, g.N, t.q, acc);
    }
}

// eq(r, z) * f = f * prod_t (bit t of z ? r_t : 1 - r_t) for z < 2^nvars (two tables summed
// when has_r2).  Split at bit h = min(nvars, 8): every CTA builds the 2^h-entry table of the
// low bits in shared memory by doubling, then each chunk of 2^h consecutive z shares one
// high-bit product, so an entry costs one multiplication (two with has_r2).
constexpr uint32_t kEqLowBits = 8;

__device__ __forceinline__ Fr eq_factor(const uint32_t (*r)[8], uint32_t t, bool bit) {
    Fr x;
#pragma unroll
    for (int k = 0; k < 8; k++) x.l[k] = r[t][k];
    return bit ? x : sub(one(), x);
}

__global__ void __launch_bounds__(256) k_eq(Fr* __restrict__ out, EqArgsBn a) {
    __shared__ Fr lo[2][1u << kEqLowBits];
    __shared__ Fr hi[2];
    const uint32_t h = a.nvars < kEqLowBits ? a.nvars : kEqLowBits;
    const uint32_t L = 1u << h;
    const uint32_t tabs = a.has_r2 ? 2u : 1u;
    if (threadIdx.x < tabs) lo[threadIdx.x][0] = one();
    __syncthreads();
    for (uint32_t t = 0; t < h; t++) {
        const uint32_t half = 1u << t;
        for (uint32_t x = threadIdx.x; x < half * tabs; x += blockDim.x) {
            const uint32_t k = x >> t, y = x & (half - 1);
            const uint32_t(*r)[8] = k ? a.r2 : a.r1;
            const Fr v = lo[k][y];
            lo[k][y + half] = mul(v, eq_factor(r, t, true));
            lo[k][y] = mul(v, eq_factor(r, t, false));
        }
        __syncthreads();
    }
    const uint64_t chunks = 1ull << (a.nvars - h);
    for (uint64_t c = blockIdx.x; c < chunks; c += gridDim.x) {
        if (threadIdx.x < tabs) {
            const uint32_t(*r)[8] = threadIdx.x ? a.r2 : a.r1;
            Fr e;
#pragma unroll
            for (int k = 0; k < 8; k++) e.l[k] = threadIdx.x ? a.f2[k] : a.f1[k];
            for (uint32_t t = h; t < a.nvars; t++) e = mul(e, eq_factor(r, t, (c >> (t - h)) & 1));
            hi[threadIdx.x] = e;
        }
        __syncthreads();
        for (uint32_t x = threadIdx.x; x < L; x += blockDim.x) {
            Fr e = mul(lo[0][x], hi[0]);
            if (a.has_r2) e = add(e, mul(lo[1][x], hi[1]));
            sts(out, (c << h) + x, e);
        }
        __syncthreads();
    }
}

__global__ void k_weights(uint64_t I, uint64_t Gm, const Fr* __restrict__ eqc, const uint4* __restrict__ mx_g,
                          const Fr* __restrict__ mx_c, const uint32_t* __restrict__ ax_off, const uint2* __restrict__ ax_g,
                          const Fr* __restrict__ ax_c, Fr* __restrict__ a_out, Fr* __restrict__ w_out) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t n = I > Gm ? I : Gm;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        if (i < Gm) sts(w_out, i, mul(lds(mx_c, i), lds(eqc, __ldg(&mx_g[i].y))));
        if (i < I) {
            Fr s = zero();
            const uint32_t k0 = __ldg(ax_off + i), k1 = __ldg(ax_off + i + 1);
            for (uint32_t k = k0; k < k1; k++) s = add(s, mul(lds(ax_c, k), lds(eqc, __ldg(&ax_g[k].x))));
            sts(a_out, i, s);
        }
    }
}

__global__ void __launch_bounds__(256) k_hg_round0(const uint32_t* __restrict__ v, uint64_t I,
                                                   const uint32_t* __restrict__ mx_off, const uint4* __restrict__ mx_g,
                                                   const Fr* __restrict__ a, const Fr* __restrict__ w, uint32_t* hg,
                                                   GeoBn g, RedBn red, const uint32_t* claim, uint32_t* evals_out) {
    const Tile t = tile(g);
    Fr acc[2] = {zero(), zero()};  // p0, p2raw
    if (t.active) {
        for (uint64_t i = (uint64_t)blockIdx.x * g.rps + t.rs; i < (I >> 1); i += (uint64_t)gridDim.x * g.rps) {
            Fr h0, h1;
            // not unrolled: each copy of the gate loop inlines a 256-bit product, and two of
            // them left this kernel waiting on instruction fetch (ncu: no_instruction stalls)
#pragma unroll 1
            for (int s = 0; s < 2; s++) {
                const uint64_t x = 2 * i + s;
                Fr h = lds(a, x);
                const uint32_t k0 = __ldg(mx_off + x), k1 = __ldg(mx_off + x + 1);
                for (uint32_t k = k0; k < k1; k++) h = add(h, mul(ldf(v, __ldg(&mx_g[k].x), g.N, t.q), lds(w, k)));
                stf(hg, x, g.N, t.q, h);
                if (s == 0) h0 = h;
                else h1 = h;
            }
            accum(acc, ldf(v, 2 * i, g.N, t.q), ldf(v, 2 * i + 1, g.N, t.q), h0, h1);
        }
    }
    reduce_bn<2>(acc, g, t.active, red, ClaimFinBn{evals_out, red.evals_dev, claim, nullptr, nullptr, zero(), g.N});
}

template <bool LANE_HG, bool FOLD>
__global__ void __launch_bounds__(256) k_round(RoundPtrsBn p, uint64_t npairs, const uint32_t* __restrict__ vx, GeoBn g,
                                               RedBn red, uint32_t* evals_out) {
    const Tile t = tile(g);
    Fr r;
#pragma unroll
    for (int k = 0; k < 8; k++) r.l[k] = p.r[k];
    // fold rounds sum p0 and p2raw (p1 from the claim), phase two's round 0 all three
    constexpr int C = FOLD ? 2 : 3;
    Fr acc[C];
#pragma unroll
    for (int c = 0; c < C; c++) acc[c] = zero();
    const Fr* hs = reinterpret_cast<const Fr*>(p.hsrc);
    Fr* hd = reinterpret_cast<Fr*>(p.hdst);
    // Phase two folds the lane-independent scalar table: with a power-of-two row tile of at
    // least 2, the threads of a row slice within a warp share it (two of them fold, the
    // others take the results by shuffle), so the loop runs warp-uniformly.
    const bool share = !LANE_HG && FOLD && g.tpr >= 2 && (g.tpr & (g.tpr - 1)) == 0;
    const uint32_t grp = g.tpr < 32 ? g.tpr : 32;
    const uint32_t gq = threadIdx.x & (grp - 1);
    const uint32_t q = threadIdx.x % g.tpr;
    const uint64_t stride = (uint64_t)gridDim.x * g.rps;
    for (uint64_t i = (uint64_t)blockIdx.x * g.rps + t.rs;; i += stride) {
        const bool valid = t.active && i < npairs;
        if (share) {
            if (!__any_sync(0xffffffffu, valid)) break;
        } else if (!valid) {
            break;
        }
        Fr f0 = zero(), f1 = zero(), h0, h1;
        if (FOLD) {
            if (valid) {
                f0 = fold(ldf(p.fsrc, 4 * i, g.N, t.q), ldf(p.fsrc, 4 * i + 1, g.N, t.q), r);
                f1 = fold(ldf(p.fsrc, 4 * i + 2, g.N, t.q), ldf(p.fsrc, 4 * i + 3, g.N, t.q), r);
                stf(p.fdst, 2 * i, g.N, t.q, f0);
                stf(p.fdst, 2 * i + 1, g.N, t.q, f1);
            }
            if (LANE_HG) {
                h0 = fold(ldf(p.hsrc, 4 * i, g.N, t.q), ldf(p.hsrc, 4 * i + 1, g.N, t.q), r);
                h1 = fold(ldf(p.hsrc, 4 * i + 2, g.N, t.q), ldf(p.hsrc, 4 * i + 3, g.N, t.q), r);
                stf(p.hdst, 2 * i, g.N, t.q, h0);
                stf(p.hdst, 2 * i + 1, g.N, t.q, h1);
            } else if (share) {
                Fr mine = zero();
                if (valid && gq < 2) mine = fold(lds(hs, 4 * i + 2 * gq), lds(hs, 4 * i + 2 * gq + 1), r);
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    h0.l[k] = __shfl_sync(0xffffffffu, mine.l[k], 0, grp);
                    h1.l[k] = __shfl_sync(0xffffffffu, mine.l[k], 1, grp);
                }
            } else {
                h0 = fold(lds(hs, 4 * i), lds(hs, 4 * i + 1), r);
                h1 = fold(lds(hs, 4 * i + 2), lds(hs, 4 * i + 3), r);
            }
            // the scalar table is shared by all lanes: the first thread of the row slice in
            // lane group 0 writes it
            if (!LANE_HG && valid && q == 0 && blockIdx.y == 0) {
                sts(hd, 2 * i, h0);
                sts(hd, 2 * i + 1, h1);
            }
        } else {
            f0 = ldf(p.fsrc, 2 * i, g.N, t.q);
            f1 = ldf(p.fsrc, 2 * i + 1, g.N, t.q);
            h0 = lds(hs, 2 * i);
            h1 = lds(hs, 2 * i + 1);
        }
        if (valid) accum(acc, f0, f1, h0, h1);
    }
    if constexpr (FOLD)
        reduce_bn<2>(acc, g, t.active, red,
                     ClaimFinBn{evals_out, red.evals_dev, nullptr, red.evals_prev, LANE_HG ? nullptr : vx, r, g.N});
    else
        reduce_bn<3>(acc, g, t.active, red, RoundFinBn{evals_out, LANE_HG ? nullptr : vx, g.N, red.evals_dev});
}

__global__ void k_s_build(uint64_t I, const uint32_t* __restrict__ my_off, const uint4* __restrict__ my_g,
                          const Fr* __restrict__ my_c, const Fr* __restrict__ eqc, const Fr* __restrict__ eqrx,
                          Fr* __restrict__ s_out) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t y = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; y < I; y += stride) {
        Fr s = zero();
        const uint32_t k0 = __ldg(my_off + y), k1 = __ldg(my_off + y + 1);
        for (uint32_t k = k0; k < k1; k++) {
            const uint4 gt = __ldg(my_g + k);  // (x, z, c, 0)
            s = add(s, mul(mul(lds(eqc, gt.y), lds(eqrx, gt.x)), lds(my_c, k)));
        }
        sts(s_out, y, s);
    }
}

__global__ void __launch_bounds__(256) k_wsum(const uint32_t* __restrict__ vals, uint64_t rows, const Fr* __restrict__ eq,
                                              GeoBn g, RedBn red, uint32_t* out) {
    const Tile t = tile(g);
    Fr acc[1] = {zero()};
    if (t.active)
        for (uint64_t z = (uint64_t)blockIdx.x * g.rps + t.rs; z < rows; z += (uint64_t)gridDim.x * g.rps)
            acc[0] = add(acc[0], mul(lds(eq, z), ldf(vals, z, g.N, t.q)));
    reduce_bn<1>(acc, g, t.active, red, CopyFinBn{out, g.N});
}

uint32_t grid1(uint64_t n) {
    uint64_t b = (n + 255) / 256;
    if (b < 1) b = 1;
    if (b > 152ull * 16) b = 152ull * 16;
    return (uint32_t)b;
}

dim3 grid_rows(const GeoBn& g, uint64_t rows, uint32_t ctas) {
    const uint32_t groups = g.N / g.tpr;
    uint64_t need = (rows + g.rps - 1) / g.rps;
    uint64_t cap = ctas / groups;
    if (cap < 1) cap = 1;
    if (need < 1) need = 1;
    return dim3((uint32_t)(need < cap ? need : cap), groups, 1);
}

}  // namespace

cudaError_t launch_load(const uint32_t* canon, uint32_t* mont, uint64_t n_elems, unsigned int* bad, cudaStream_t s) {
    k_load<<<grid1(n_elems), 256, 0, s>>>(canon, mont, n_elems, bad);
    return cudaGetLastError();
}

cudaError_t launch_gate_sums(bool mul_gates, uint64_t O, const uint32_t* off, const uint32_t* gates, const Fr* coef,
                             const Fr* eqz, const Fr* eqx, const Fr* eqy, unsigned long long* acc,
                             unsigned int* ticket, uint32_t* out, cudaStream_t s) {
    const uint32_t grid = grid1(O);
    if (mul_gates)
        k_gate_sums<true><<<grid, kBlock, 0, s>>>(O, off, gates, coef, eqz, eqx, eqy, acc, ticket, out);
    else
        k_gate_sums<false><<<grid, kBlock, 0, s>>>(O, off, gates, coef, eqz, eqx, eqy, acc, ticket, out);
    return cudaGetLastError();
}

cudaError_t launch_unload(uint32_t* v, uint64_t n_elems, cudaStream_t s) {
    k_unload<<<grid1(n_elems), 256, 0, s>>>(v, n_elems);
    return cudaGetLastError();
}

cudaError_t launch_evaluate(const uint32_t* in, uint32_t* out, uint64_t O, const uint32_t* mo_off, const uint4* mo_g,
                            const Fr* mo_c, const uint32_t* ao_off, const uint2* ao_g, const Fr* ao_c, const GeoBn& g,
                            uint32_t ctas, cudaStream_t s) {
    k_evaluate<<<grid_rows(g, O, ctas), 256, 0, s>>>(in, out, O, mo_off, mo_g, mo_c, ao_off, ao_g, ao_c, g);
    return cudaGetLastError();
}

cudaError_t launch_eq(Fr* out, const EqArgsBn& a, cudaStream_t s) {
    const uint64_t chunks = 1ull << (a.nvars > kEqLowBits ? a.nvars - kEqLowBits : 0);
    k_eq<<<(uint32_t)(chunks < 152ull * 4 ? chunks : 152ull * 4), 256, 0, s>>>(out, a);
    return cudaGetLastError();
}

cudaError_t launch_weights(uint64_t I, uint64_t Gm, const Fr* eqc, const uint4* mx_g, const Fr* mx_c,
                           const uint32_t* ax_off, const uint2* ax_g, const Fr* ax_c, Fr* a_out, Fr* w_out,
                           cudaStream_t s) {
    k_weights<<<grid1(I > Gm ? I : Gm), 256, 0, s>>>(I, Gm, eqc, mx_g, mx_c, ax_off, ax_g, ax_c, a_out, w_out);
    return cudaGetLastError();
}

cudaError_t launch_hg_round0(const uint32_t* v, uint64_t I, const uint32_t* mx_off, const uint4* mx_g, const Fr* a,
                             const Fr* w, uint32_t* hg, const GeoBn& g, uint32_t ctas, RedBn red, const uint32_t* claim,
                             uint32_t* evals_out, cudaStream_t s) {
    if (!claim) return cudaErrorInvalidValue;
    k_hg_round0<<<grid_rows(g, I / 2, ctas), 256, 3 * 8 * 256 * 4, s>>>(v, I, mx_off, mx_g, a, w, hg, g, red, claim,
                                                                       evals_out);
    return cudaGetLastError();
}

cudaError_t launch_round(bool lane_hg, bool fold_, const RoundPtrsBn& p, uint64_t npairs, const uint32_t* vx,
                         const GeoBn& g, uint32_t ctas, RedBn red, uint32_t* evals_out, cudaStream_t s) {
    const dim3 grid = grid_rows(g, npairs, ctas);
    const size_t smem = 3 * 8 * 256 * 4;
    if (fold_ && (!red.evals_prev || red.evals_prev == red.evals_dev)) return cudaErrorInvalidValue;
    if (lane_hg && fold_) k_round<true, true><<<grid, 256, smem, s>>>(p, npairs, vx, g, red, evals_out);
    else if (!lane_hg && fold_) k_round<false, true><<<grid, 256, smem, s>>>(p, npairs, vx, g, red, evals_out);
    else if (!lane_hg && !fold_) k_round<false, false><<<grid, 256, smem, s>>>(p, npairs, vx, g, red, evals_out);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

cudaError_t launch_s_build(uint64_t I, const uint32_t* my_off, const uint4* my_g, const Fr* my_c, const Fr* eqc,
                           const Fr* eqrx, Fr* s_out, cudaStream_t s) {
    k_s_build<<<grid1(I), 256, 0, s>>>(I, my_off, my_g, my_c, eqc, eqrx, s_out);
    return cudaGetLastError();
}

cudaError_t launch_wsum(const uint32_t* vals, uint64_t rows, const Fr* eq, const GeoBn& g, uint32_t ctas, RedBn red,
                        uint32_t* out, cudaStream_t s) {
    k_wsum<<<grid_rows(g, rows, ctas), 256, 8 * 256 * 4, s>>>(vals, rows, eq, g, red, out);
    return cudaGetLastError();
}

}  // namespace bn
}  // namespace gkrgpu
