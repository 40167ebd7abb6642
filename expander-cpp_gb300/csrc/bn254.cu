// BN254 scalar-field kernels (see bn254.cuh).  Same algorithms as the M31 kernels in
// kernels.cu, for one repetition (R = 1 for BN254, include/configuration/config.hpp:61-65),
// with 256-bit elements: one thread per element of a row, Montgomery multiplication on
// 8 x 32-bit limbs (CIOS, 64-bit multiply-accumulate chains).
#include "bn254.cuh"

namespace gkrgpu {
namespace bn {

namespace {

__constant__ uint32_t kR[8] = {0xf0000001u, 0x43e1f593u, 0x79b97091u, 0x2833e848u,
                               0x8181585du, 0xb85045b6u, 0xe131a029u, 0x30644e72u};
__constant__ uint32_t kOne[8] = {0x4ffffffbu, 0xac96341cu, 0x9f60cd29u, 0x36fc7695u,
                                 0x7879462eu, 0x666ea36fu, 0x9a07df2fu, 0x0e0a77c1u};  // 2^256 mod r
__constant__ uint32_t kR2[8] = {0xae216da7u, 0x1bb8e645u, 0xe35c59e3u, 0x53fe3ab1u,
                                0x53bb8085u, 0x8c49833du, 0x7f4e44a5u, 0x0216d0b1u};  // 2^512 mod r
constexpr uint32_t kNP = 0xefffffffu;  // -r^-1 mod 2^32

__device__ __forceinline__ bool geq_r(const uint32_t* t) {
#pragma unroll
    for (int i = 7; i >= 0; i--) {
        if (t[i] > kR[i]) return true;
        if (t[i] < kR[i]) return false;
    }
    return true;
}
__device__ __forceinline__ void sub_r(uint32_t* t) {
    uint64_t br = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const uint64_t d = (uint64_t)t[i] - kR[i] - br;
        t[i] = (uint32_t)d;
        br = (d >> 63) & 1;
    }
}
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
__device__ __forceinline__ Fr add(const Fr& a, const Fr& b) {
    Fr s;
    uint64_t c = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        c += (uint64_t)a.l[i] + b.l[i];
        s.l[i] = (uint32_t)c;
        c >>= 32;
    }
    if (geq_r(s.l)) sub_r(s.l);  // a + b < 2r < 2^255: no carry out of the top limb
    return s;
}
__device__ __forceinline__ Fr sub(const Fr& a, const Fr& b) {
    Fr d;
    uint64_t br = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const uint64_t x = (uint64_t)a.l[i] - b.l[i] - br;
        d.l[i] = (uint32_t)x;
        br = (x >> 63) & 1;
    }
    if (br) {
        uint64_t c = 0;
#pragma unroll
        for (int i = 0; i < 8; i++) {
            c += (uint64_t)d.l[i] + kR[i];
            d.l[i] = (uint32_t)c;
            c >>= 32;
        }
    }
    return d;
}
// Montgomery product a * b * 2^-256 mod r.
__device__ __forceinline__ Fr mul(const Fr& a, const Fr& b) {
    uint32_t t[10];
#pragma unroll
    for (int i = 0; i < 10; i++) t[i] = 0u;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        uint64_t c = 0;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            c += (uint64_t)a.l[j] * b.l[i] + t[j];
            t[j] = (uint32_t)c;
            c >>= 32;
        }
        c += t[8];
        t[8] = (uint32_t)c;
        t[9] = (uint32_t)(c >> 32);
        const uint32_t m = t[0] * kNP;
        c = ((uint64_t)m * kR[0] + t[0]) >> 32;
#pragma unroll
        for (int j = 1; j < 8; j++) {
            c += (uint64_t)m * kR[j] + t[j];
            t[j - 1] = (uint32_t)c;
            c >>= 32;
        }
        c += t[8];
        t[7] = (uint32_t)c;
        t[8] = t[9] + (uint32_t)(c >> 32);
    }
    Fr r;
#pragma unroll
    for (int i = 0; i < 8; i++) r.l[i] = t[i];
    if (t[8] || geq_r(r.l)) sub_r(r.l);
    return r;
}
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

// T = sum_k s[k] 2^(32k) (the 64-bit limb sums of many Montgomery values) reduced mod r:
// REDC(T) = T 2^-256, then a Montgomery product with 2^512 mod r gives T mod r.
__device__ Fr reduce_sums(const unsigned long long* s) {
    uint32_t t[16];
#pragma unroll
    for (int i = 0; i < 16; i++) t[i] = 0u;
    unsigned long long c = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const unsigned long long lo = c + (s[k] & 0xffffffffull);
        t[k] = (uint32_t)lo;
        c = (lo >> 32) + (s[k] >> 32);
    }
    t[8] = (uint32_t)c;
    t[9] = (uint32_t)(c >> 32);
    for (int i = 0; i < 8; i++) {
        const uint32_t m = t[i] * kNP;
        uint64_t cc = 0;
        for (int j = 0; j < 8; j++) {
            cc += (uint64_t)m * kR[j] + t[i + j];
            t[i + j] = (uint32_t)cc;
            cc >>= 32;
        }
        for (int j = i + 8; j < 16 && cc; j++) {
            cc += t[j];
            t[j] = (uint32_t)cc;
            cc >>= 32;
        }
    }
    Fr x;
#pragma unroll
    for (int i = 0; i < 8; i++) x.l[i] = t[8 + i];
    if (geq_r(x.l)) sub_r(x.l);
    Fr r2;
#pragma unroll
    for (int i = 0; i < 8; i++) r2.l[i] = kR2[i];
    return mul(x, r2);
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

// C components per thread -> shared-memory sum over the CTA's row slices -> 64-bit
// atomic adds per limb -> the last CTA of the lane group hands its lanes to fin(lane).
template <int C, class Fin>
__device__ __forceinline__ void reduce_bn(const Fr (&acc)[C], const GeoBn& g, bool active, RedBn red, Fin fin) {
    extern __shared__ uint32_t smem[];
    const uint32_t tid = threadIdx.x, B = blockDim.x;
#pragma unroll
    for (int c = 0; c < C; c++)
#pragma unroll
        for (int k = 0; k < 8; k++) smem[(c * 8 + k) * B + tid] = active ? acc[c].l[k] : 0u;
    __syncthreads();
    for (uint32_t o = tid; o < (uint32_t)C * g.tpr; o += B) {
        const uint32_t c = o / g.tpr, q = o - c * g.tpr;
        Fr s = zero();
        for (uint32_t r = 0; r < g.rps; r++) {
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
    for (uint32_t li = tid; li < g.tpr; li += B) fin(blockIdx.y * g.tpr + li);
    if (tid == 0) red.ticket[blockIdx.y] = 0u;
    if (red.done) {
        __threadfence_system();
        __syncthreads();
        if (tid == 0) atomicAdd_system(red.done, 1u);
    }
}

__device__ __forceinline__ Fr take(const RedBn& red, uint32_t c, uint32_t N, uint32_t lane) {
    unsigned long long s[8];
    unsigned long long* p = &red.acc[((size_t)c * N + lane) * 8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        s[k] = __ldcg(p + k);
        p[k] = 0ull;
    }
    return reduce_sums(s);
}

// Evaluations at 0, 1, 2 (canonical) of one lane; phase two multiplies by vx (Montgomery).
struct RoundFinBn {
    RedBn red;
    uint32_t* out;  // 3 x N x 8 limbs, canonical
    const uint32_t* vx;
    uint32_t N;
    __device__ void operator()(uint32_t lane) const {
        Fr p0 = take(red, 0, N, lane), p1 = take(red, 1, N, lane), p2r = take(red, 2, N, lane);
        const Fr p1x2 = add(p1, p1);
        Fr p2 = add(add(p1x2, p1x2), p1x2);             // 6 p1
        p2 = add(p2, add(add(p0, p0), p0));            // + 3 p0
        p2 = sub(p2, add(p2r, p2r));                    // - 2 p2raw
        if (vx) {
            const Fr x = ldf(vx, 0, N, lane);
            p0 = mul(p0, x);
            p1 = mul(p1, x);
            p2 = mul(p2, x);
        }
        stf(out, 0, N, lane, from_mont(p0));
        stf(out, 1, N, lane, from_mont(p1));
        stf(out, 2, N, lane, from_mont(p2));
    }
};

struct CopyFinBn {
    RedBn red;
    uint32_t* out;  // N x 8 limbs, canonical
    uint32_t N;
    __device__ void operator()(uint32_t lane) const { stf(out, 0, N, lane, from_mont(take(red, 0, N, lane))); }
};

__device__ __forceinline__ void accum(Fr (&acc)[3], const Fr& f0, const Fr& f1, const Fr& h0, const Fr& h1) {
    acc[0] = add(acc[0], mul(f0, h0));
    acc[1] = add(acc[1], mul(f1, h1));
    acc[2] = add(acc[2], mul(add(f0, f1), add(h0, h1)));
}

// ---------------------------------------------------------------- kernels
// Canonical input -> Montgomery table; an element >= r raises *bad (and is stored as 0).
__global__ void k_load(const uint32_t* __restrict__ canon, uint32_t* __restrict__ mont, uint64_t n, unsigned int* bad) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        Fr x = lds(reinterpret_cast<const Fr*>(canon), i);
        if (geq_r(x.l)) {
            atomicOr(bad, 1u);
            x = zero();
        }
        sts(reinterpret_cast<Fr*>(mont), i, to_mont(x));
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

__global__ void k_eq(Fr* __restrict__ out, EqArgsBn a) {
    const uint64_t size = 1ull << a.nvars;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t z = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; z < size; z += stride) {
        Fr e1, e2;
#pragma unroll
        for (int k = 0; k < 8; k++) { e1.l[k] = a.f1[k]; e2.l[k] = a.f2[k]; }
        for (uint32_t t = 0; t < a.nvars; t++) {
            Fr r1;
#pragma unroll
            for (int k = 0; k < 8; k++) r1.l[k] = a.r1[t][k];
            e1 = mul(e1, ((z >> t) & 1) ? r1 : sub(one(), r1));
            if (a.has_r2) {
                Fr r2;
#pragma unroll
                for (int k = 0; k < 8; k++) r2.l[k] = a.r2[t][k];
                e2 = mul(e2, ((z >> t) & 1) ? r2 : sub(one(), r2));
            }
        }
        sts(out, z, a.has_r2 ? add(e1, e2) : e1);
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
                                                   GeoBn g, RedBn red, uint32_t* evals_out) {
    const Tile t = tile(g);
    Fr acc[3] = {zero(), zero(), zero()};
    if (t.active) {
        for (uint64_t i = (uint64_t)blockIdx.x * g.rps + t.rs; i < (I >> 1); i += (uint64_t)gridDim.x * g.rps) {
            Fr h[2];
#pragma unroll
            for (int s = 0; s < 2; s++) {
                const uint64_t x = 2 * i + s;
                h[s] = lds(a, x);
                const uint32_t k0 = __ldg(mx_off + x), k1 = __ldg(mx_off + x + 1);
                for (uint32_t k = k0; k < k1; k++) h[s] = add(h[s], mul(ldf(v, __ldg(&mx_g[k].x), g.N, t.q), lds(w, k)));
                stf(hg, x, g.N, t.q, h[s]);
            }
            accum(acc, ldf(v, 2 * i, g.N, t.q), ldf(v, 2 * i + 1, g.N, t.q), h[0], h[1]);
        }
    }
    reduce_bn<3>(acc, g, t.active, red, RoundFinBn{red, evals_out, nullptr, g.N});
}

template <bool LANE_HG, bool FOLD>
__global__ void __launch_bounds__(256) k_round(RoundPtrsBn p, uint64_t npairs, const uint32_t* __restrict__ vx, GeoBn g,
                                               RedBn red, uint32_t* evals_out) {
    const Tile t = tile(g);
    Fr r;
#pragma unroll
    for (int k = 0; k < 8; k++) r.l[k] = p.r[k];
    Fr acc[3] = {zero(), zero(), zero()};
    const Fr* hs = reinterpret_cast<const Fr*>(p.hsrc);
    Fr* hd = reinterpret_cast<Fr*>(p.hdst);
    if (t.active) {
        for (uint64_t i = (uint64_t)blockIdx.x * g.rps + t.rs; i < npairs; i += (uint64_t)gridDim.x * g.rps) {
            Fr f0, f1, h0, h1;
            if (FOLD) {
                f0 = fold(ldf(p.fsrc, 4 * i, g.N, t.q), ldf(p.fsrc, 4 * i + 1, g.N, t.q), r);
                f1 = fold(ldf(p.fsrc, 4 * i + 2, g.N, t.q), ldf(p.fsrc, 4 * i + 3, g.N, t.q), r);
                stf(p.fdst, 2 * i, g.N, t.q, f0);
                stf(p.fdst, 2 * i + 1, g.N, t.q, f1);
                if (LANE_HG) {
                    h0 = fold(ldf(p.hsrc, 4 * i, g.N, t.q), ldf(p.hsrc, 4 * i + 1, g.N, t.q), r);
                    h1 = fold(ldf(p.hsrc, 4 * i + 2, g.N, t.q), ldf(p.hsrc, 4 * i + 3, g.N, t.q), r);
                    stf(p.hdst, 2 * i, g.N, t.q, h0);
                    stf(p.hdst, 2 * i + 1, g.N, t.q, h1);
                } else {
                    h0 = fold(lds(hs, 4 * i), lds(hs, 4 * i + 1), r);
                    h1 = fold(lds(hs, 4 * i + 2), lds(hs, 4 * i + 3), r);
                    // the scalar table is shared by all lanes: lane 0 of group 0 writes it
                    if (threadIdx.x % g.tpr == 0 && blockIdx.y == 0) {
                        sts(hd, 2 * i, h0);
                        sts(hd, 2 * i + 1, h1);
                    }
                }
            } else {
                f0 = ldf(p.fsrc, 2 * i, g.N, t.q);
                f1 = ldf(p.fsrc, 2 * i + 1, g.N, t.q);
                h0 = lds(hs, 2 * i);
                h1 = lds(hs, 2 * i + 1);
            }
            accum(acc, f0, f1, h0, h1);
        }
    }
    reduce_bn<3>(acc, g, t.active, red, RoundFinBn{red, evals_out, LANE_HG ? nullptr : vx, g.N});
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
    reduce_bn<1>(acc, g, t.active, red, CopyFinBn{red, out, g.N});
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
    k_eq<<<grid1(1ull << a.nvars), 256, 0, s>>>(out, a);
    return cudaGetLastError();
}

cudaError_t launch_weights(uint64_t I, uint64_t Gm, const Fr* eqc, const uint4* mx_g, const Fr* mx_c,
                           const uint32_t* ax_off, const uint2* ax_g, const Fr* ax_c, Fr* a_out, Fr* w_out,
                           cudaStream_t s) {
    k_weights<<<grid1(I > Gm ? I : Gm), 256, 0, s>>>(I, Gm, eqc, mx_g, mx_c, ax_off, ax_g, ax_c, a_out, w_out);
    return cudaGetLastError();
}

cudaError_t launch_hg_round0(const uint32_t* v, uint64_t I, const uint32_t* mx_off, const uint4* mx_g, const Fr* a,
                             const Fr* w, uint32_t* hg, const GeoBn& g, uint32_t ctas, RedBn red, uint32_t* evals_out,
                             cudaStream_t s) {
    k_hg_round0<<<grid_rows(g, I / 2, ctas), 256, 3 * 8 * 256 * 4, s>>>(v, I, mx_off, mx_g, a, w, hg, g, red, evals_out);
    return cudaGetLastError();
}

cudaError_t launch_round(bool lane_hg, bool fold_, const RoundPtrsBn& p, uint64_t npairs, const uint32_t* vx,
                         const GeoBn& g, uint32_t ctas, RedBn red, uint32_t* evals_out, cudaStream_t s) {
    const dim3 grid = grid_rows(g, npairs, ctas);
    const size_t smem = 3 * 8 * 256 * 4;
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
