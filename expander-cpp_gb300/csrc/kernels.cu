// Hand-written sm_103a kernels of the GKR prove path (M31).
//
// Data layout in HBM: every per-copy table is row-major rows x N u32 (row r, copy k at
// r*N + k), the byte layout of a proof vector (VectorizedM31::to_bytes, M31.hpp:420-426),
// so a warp's 16-byte loads along a row are fully coalesced.  Scalar tables that do not
// depend on the copy (eq tables, gate weights, the phase-two h(y) factor) are plain
// arrays of u32 read by broadcast.
//
// Reference counterparts:
//   k_evaluate       CircuitLayer::evaluate                     include/circuit/circuit.hpp:92-105
//   k_eq             _eq_evals_at                               include/LinearGKR/sumcheck_common.hpp:17-53
//   k_weights        the scalar factors of _prepare_g_x_vals    include/LinearGKR/sumcheck_helper.hpp:188-229
//   k_hg_round0      _prepare_g_x_vals + poly_eval_at(0)        sumcheck_helper.hpp:172-231, 68-102
//   k_hg_round1      hg rebuilt + receive_challenge + poly_eval_at(1)
//   k_round          receive_challenge + poly_eval_at(k)        sumcheck_helper.hpp:104-133, 68-102
//   k_s_build(4)     _prepare_h_y_vals (copy-independent part)  sumcheck_helper.hpp:233-261
//   k_p2_round01     phase-two poly_eval_at of rounds 0 and 1 from one pass (round 1's sums are
//                    quadratic in round 0's challenge); k_p2_round1_fin finishes round 1
//   k_p2_round2      phase-two round 2 refolding the layer input
//   k_wsum           eval_multilinear via an eq table           include/poly_commit/poly.hpp:88-104
//
// k_round gives each CTA one repetition j = blockIdx.x % R: the R CTAs of a row chunk are
// adjacent in launch order, run together and share their common source rows through L2,
// while each thread keeps only one repetition's state.  The kernels whose source is the
// layer input itself (k_hg_round0/1, k_p2_round01, k_p2_round2) keep all R repetitions in a
// thread, so each input row is read once.
#include <atomic>

#include "kernels.cuh"
#include "m31.cuh"

namespace gkrgpu {

const char* const kKernelNames[K_NUM_KERNELS] = {"check_canonical", "evaluate", "eq_table", "gate_weights",
                                                 "hg_build_round0", "round_fold_lane", "round_fold_scalar",
                                                 "phase2_s_build", "weighted_row_sum", "hg_rebuild_round1",
                                                 "verifier_gate_sums", "canonicalize", "phase2_round0", "stage_words", "round_tail",
                                                 "bn254_load",
                                                 "bn254_evaluate", "bn254_eq_table", "bn254_gate_weights",
                                                 "bn254_hg_build_round0", "bn254_round_fold_lane",
                                                 "bn254_round_fold_scalar", "bn254_phase2_s_build",
                                                 "bn254_weighted_row_sum", "bn254_unload"};

namespace {

using m31::add;
using m31::fold;
using m31::mul;
using m31::sub;

__device__ __forceinline__ uint4 ld4(const uint32_t* __restrict__ base, uint64_t row, uint32_t N, uint32_t lane0) {
    return __ldg(reinterpret_cast<const uint4*>(base + row * N + lane0));
}
__device__ __forceinline__ void st4(uint32_t* base, uint64_t row, uint32_t N, uint32_t lane0, uint4 v) {
    *reinterpret_cast<uint4*>(base + row * N + lane0) = v;
}
__device__ __forceinline__ uint32_t comp(const uint4& v, int l) { return l == 0 ? v.x : l == 1 ? v.y : l == 2 ? v.z : v.w; }
__device__ __forceinline__ uint4 mk4(const uint32_t (&a)[4]) { return make_uint4(a[0], a[1], a[2], a[3]); }

// Canonical residue of a sum of many canonical values (< 2^64 total).
__device__ __forceinline__ uint32_t reduce64(unsigned long long x) {
    x = (x & m31::P) + (x >> 31);
    x = (x & m31::P) + (x >> 31);
    uint32_t s = (uint32_t)x;
    return m31::umin(s, s - m31::P);
}

// Canonical total of component c at `lane`, re-zeroing the accumulator for the next launch.
__device__ __forceinline__ uint32_t take(const RedScratch& red, uint32_t c, uint32_t N, uint32_t lane) {
    unsigned long long* p = &red.acc[(size_t)c * N + lane];
    const uint32_t v = reduce64(__ldcg(p));
    *p = 0ull;
    return v;
}

// Reduction of C components x 4 lanes per thread: a shared-memory reduction over the CTA's
// row slices, one 64-bit atomic add per (component, lane) into red.acc at component
// comp_base + c, then the last CTA of this lane group (ticket blockIdx.y) hands every lane
// of the group to fin(lane), which collects the totals with take().
template <class Fin>
__device__ __forceinline__ void finish_group(const RedScratch& red, uint32_t base, uint32_t lanes, Fin& fin);

template <int C, class Fin>
__device__ __forceinline__ void reduce_group(const uint32_t (&acc)[C][4], const Geo& g, bool active, RedScratch red,
                                             uint32_t comp_base, Fin fin) {
    extern __shared__ uint32_t smem[];
    const uint32_t tid = threadIdx.x, B = blockDim.x;
#pragma unroll
    for (int c = 0; c < C; c++)
#pragma unroll
        for (int l = 0; l < 4; l++) smem[(c * 4 + l) * B + tid] = active ? acc[c][l] : 0u;
    __syncthreads();
    const uint32_t tpr = g.tpr, rps = g.rps;
    for (uint32_t o = tid; o < (uint32_t)C * 4 * tpr; o += B) {
        const uint32_t cl = o / tpr, q = o - cl * tpr;
        const uint32_t* col = smem + cl * B + q;
        unsigned long long s = 0;
        for (uint32_t r = 0; r < rps; r++) s += col[r * tpr];
        const uint32_t c = cl >> 2, l = cl & 3;
        const uint32_t lane = (blockIdx.y * tpr + q) * 4 + l;
        atomicAdd(&red.acc[(size_t)(comp_base + c) * g.N + lane], s);
    }
    finish_group(red, blockIdx.y * 4 * tpr, 4 * tpr, fin);
}

// After a CTA's atomic adds: the last CTA of lane group blockIdx.y (ticket) hands lanes
// base .. base + lanes - 1 to fin(lane), re-arms the ticket and, with red.done, publishes
// the group's results to the host (system-scope fence, then the completion counter).
template <class Fin>
__device__ __forceinline__ void finish_group(const RedScratch& red, uint32_t base, uint32_t lanes, Fin& fin) {
    const uint32_t tid = threadIdx.x, B = blockDim.x;
    __threadfence();
    __syncthreads();
    __shared__ unsigned int is_last;
    if (tid == 0) is_last = (atomicAdd(&red.ticket[blockIdx.y], 1u) == gridDim.x - 1) ? 1u : 0u;
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    for (uint32_t li = tid; li < lanes; li += B) fin(base + li);
    if (tid == 0) red.ticket[blockIdx.y] = 0u;
    if (red.done) {
        __threadfence_system();
        __syncthreads();
        if (tid == 0) atomicAdd_system(red.done, 1u);
    }
}

// reduce_group for kernels with one copy per thread: g.tpr threads (copies) per row slice,
// acc[c] the thread's canonical partial of component c for copy blockIdx.y * g.tpr + q.
template <int C, class Fin>
__device__ __forceinline__ void reduce_group1(const uint32_t (&acc)[C], const Geo& g, bool active, RedScratch red,
                                              Fin fin) {
    extern __shared__ uint32_t smem[];
    const uint32_t tid = threadIdx.x, B = blockDim.x, L = g.tpr, rps = g.rps;
#pragma unroll
    for (int c = 0; c < C; c++) smem[c * B + tid] = active ? acc[c] : 0u;
    __syncthreads();
    for (uint32_t o = tid; o < (uint32_t)C * L; o += B) {
        const uint32_t c = o / L, q = o - c * L;
        const uint32_t* col = smem + c * B + q;
        unsigned long long s = 0;
        for (uint32_t r = 0; r < rps; r++) s += col[r * L];
        atomicAdd(&red.acc[(size_t)c * g.N + blockIdx.y * L + q], s);
    }
    finish_group(red, blockIdx.y * L, L, fin);
}

struct TileIdx {
    uint32_t q, rs, lane0;
    bool active;
};
__device__ __forceinline__ TileIdx tile_idx(const Geo& g) {
    TileIdx t;
    t.q = threadIdx.x % g.tpr;
    t.rs = threadIdx.x / g.tpr;
    t.lane0 = (blockIdx.y * g.tpr + t.q) * 4;
    t.active = t.rs < g.rps;
    return t;
}

// Index of the i-th group a kernel works on: with a list, its i-th entry (the groups that
// have gates, in increasing order), otherwise i itself.
__device__ __forceinline__ uint64_t group_at(const uint32_t* __restrict__ list, uint64_t i) {
    return list ? (uint64_t)__ldg(list + i) : i;
}

// ---------------------------------------------------------------- input check
__global__ void k_check_canonical(const uint32_t* __restrict__ v, uint64_t n, unsigned int* flag) {
    uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    unsigned int bad = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n / 4; i += stride) {
        uint4 x = __ldg(reinterpret_cast<const uint4*>(v) + i);
        bad |= (x.x >= m31::P) | (x.y >= m31::P) | (x.z >= m31::P) | (x.w >= m31::P);
    }
    // every writer stores the same 1, so a plain store works for device and host-mapped flags
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) *reinterpret_cast<volatile unsigned int*>(flag) = 1u;
}

// ---------------------------------------------------------------- small transfers
// dst[k * n + i] = src_k[i] for i < n, k < nsrc: small tables moved between device memory and
// host-mapped memory by the SMs, so a proof's stream never waits behind a bulk copy of another
// proof on the copy engine.  With `done`, each CTA makes its writes visible to the host and
// then increments the counter (system scope).
__global__ void k_stage_words(uint32_t* dst, const uint32_t* s0, const uint32_t* s1, const uint32_t* s2, uint32_t nsrc,
                              uint64_t n, unsigned int* done) {
    const uint64_t total = n * nsrc, stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
        const uint64_t k = i / n, e = i - k * n;
        const uint32_t* src = k == 0 ? s0 : (k == 1 ? s1 : s2);
        dst[i] = src[e];
    }
    if (done) {
        __threadfence_system();
        __syncthreads();
        if (threadIdx.x == 0) atomicAdd_system(done, 1u);
    }
}

// In-place M31::from_bytes of u32 words (the verifier reads the commitment from proof bytes).
__global__ void k_canonicalize(uint32_t* v, uint64_t n) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) v[i] = m31::from_u32(v[i]);
}

// ---------------------------------------------------------------- verifier gate sums
// eval_sparse_circuit_connect_poly (include/LinearGKR/sumcheck_verifier_utils.hpp:22-56)
// for R points at once: mul sums c * eqz_j[o] * eqx_j[i0] * eqy_j[i1] over the mul gates
// (MUL), or add sums c * eqz_j[o] * eqx_j[i0] over the add gates, walked by output o (the
// evaluate CSR).  Block partials go to 64-bit accumulators; the last block writes the R
// canonical totals and re-zeroes the scratch.
template <bool MUL>
__global__ void __launch_bounds__(256) k_gate_sums(uint64_t O, uint64_t I, const uint32_t* __restrict__ off,
                                                   const uint32_t* __restrict__ gates, const uint32_t* __restrict__ eqz,
                                                   const uint32_t* __restrict__ eqx, const uint32_t* __restrict__ eqy,
                                                   uint32_t reps, unsigned long long* acc, unsigned int* ticket,
                                                   uint32_t* out) {
    uint32_t s[3] = {0u, 0u, 0u};
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t o = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; o < O; o += stride) {
        const uint32_t k0 = __ldg(off + o), k1 = __ldg(off + o + 1);
        for (uint32_t k = k0; k < k1; k++) {
            uint32_t i0, i1 = 0, c;
            if (MUL) {
                const uint4 g = __ldg(reinterpret_cast<const uint4*>(gates) + k);  // (i0, i1, c, 0)
                i0 = g.x; i1 = g.y; c = g.z;
            } else {
                const uint2 g = __ldg(reinterpret_cast<const uint2*>(gates) + k);  // (i0, c)
                i0 = g.x; c = g.y;
            }
            for (uint32_t j = 0; j < reps; j++) {
                uint32_t t = mul(mul(c, __ldg(eqz + (uint64_t)j * O + o)), __ldg(eqx + (uint64_t)j * I + i0));
                if (MUL) t = mul(t, __ldg(eqy + (uint64_t)j * I + i1));
                s[j] = add(s[j], t);
            }
        }
    }
    __shared__ unsigned long long part[3];
    if (threadIdx.x < 3) part[threadIdx.x] = 0ull;
    __syncthreads();
    for (uint32_t j = 0; j < reps; j++) {
        unsigned long long x = s[j];
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) x += __shfl_xor_sync(0xffffffffu, x, d);
        if ((threadIdx.x & 31) == 0) atomicAdd(&part[j], x);
    }
    __syncthreads();
    if (threadIdx.x < reps) atomicAdd(&acc[threadIdx.x], part[threadIdx.x]);
    __threadfence();
    __syncthreads();
    __shared__ unsigned int is_last;
    if (threadIdx.x == 0) is_last = (atomicAdd(ticket, 1u) == gridDim.x - 1) ? 1u : 0u;
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    if (threadIdx.x < reps) {
        out[threadIdx.x] = reduce64(__ldcg(&acc[threadIdx.x]));
        acc[threadIdx.x] = 0ull;
    }
    if (threadIdx.x == 0) *ticket = 0u;
}

// ---------------------------------------------------------------- layer evaluation
// out[o] = sum over mul gates (o, i0, i1, c) of in[i0]*in[i1]*c + sum over add gates
// (o, i0, c) of in[i0]*c, gates grouped by o (CSR), so every output row is written once.
__global__ void __launch_bounds__(256) k_evaluate(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, uint64_t O,
                                                  const uint32_t* __restrict__ mo_off, const uint4* __restrict__ mo_g,
                                                  const uint32_t* __restrict__ ao_off, const uint2* __restrict__ ao_g,
                                                  Geo g) {
    const TileIdx t = tile_idx(g);
    if (!t.active) return;
    for (uint64_t o = (uint64_t)blockIdx.x * g.rps + t.rs; o < O; o += (uint64_t)gridDim.x * g.rps) {
        uint32_t acc[4] = {0u, 0u, 0u, 0u};
        const uint32_t m0 = __ldg(mo_off + o), m1 = __ldg(mo_off + o + 1);
        for (uint32_t k = m0; k < m1; k++) {
            const uint4 gt = __ldg(mo_g + k);
            const uint4 a = ld4(in, gt.x, g.N, t.lane0), b = ld4(in, gt.y, g.N, t.lane0);
#pragma unroll
            for (int l = 0; l < 4; l++) acc[l] = add(acc[l], mul(mul(comp(a, l), comp(b, l)), gt.z));
        }
        const uint32_t a0 = __ldg(ao_off + o), a1 = __ldg(ao_off + o + 1);
        for (uint32_t k = a0; k < a1; k++) {
            const uint2 gt = __ldg(ao_g + k);
            const uint4 a = ld4(in, gt.x, g.N, t.lane0);
#pragma unroll
            for (int l = 0; l < 4; l++) acc[l] = add(acc[l], mul(comp(a, l), gt.y));
        }
        st4(out, o, g.N, t.lane0, mk4(acc));
    }
}

// ---------------------------------------------------------------- eq tables
// out[j][z] = f1 * eq(r1_j, z) + f2 * eq(r2_j, z), bit t of z paired with r[t]
// (little-endian, sumcheck_common.hpp:17-53); eq(r, 0) = 1 - r, eq(r, 1) = r.
__global__ void k_eq(uint32_t* __restrict__ out, EqArgs a) {
    const uint64_t size = 1ull << a.nvars;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t z = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; z < size; z += stride) {
        for (uint32_t j = 0; j < a.reps; j++) {
            uint32_t e1 = a.f1, e2 = a.f2;
            for (uint32_t t = 0; t < a.nvars; t++) {
                const bool bit = (z >> t) & 1;
                e1 = mul(e1, bit ? a.r1[j][t] : sub(1u, a.r1[j][t]));
                if (a.f2) e2 = mul(e2, bit ? a.r2[j][t] : sub(1u, a.r2[j][t]));
            }
            out[(uint64_t)j * size + z] = add(e1, a.f2 ? e2 : 0u);
        }
    }
}

// ---------------------------------------------------------------- phase-one scalar factors
// w[k].j = c_k * eqc_j[z_k] for every mul gate k (gates in CSR-by-x order) and
// a[x].j = sum over add gates (z, x, c) of c * eqc_j[z]: the copy-independent parts of
// hg(x) = sum_mul v(y) c eqc(z) + sum_add c eqc(z) (sumcheck_helper.hpp:203-229).
__global__ void k_weights(uint64_t I, uint64_t Gm, uint64_t O, const uint32_t* __restrict__ eqc,
                          const uint4* __restrict__ mx_g, const uint32_t* __restrict__ ax_off,
                          const uint2* __restrict__ ax_g, uint4* __restrict__ a_out, uint4* __restrict__ w_out,
                          uint32_t reps) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t n = I > Gm ? I : Gm;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        if (i < Gm) {
            const uint4 gt = __ldg(mx_g + i);  // (y, z, c, 0)
            uint32_t w[3] = {0u, 0u, 0u};
            for (uint32_t j = 0; j < reps; j++) w[j] = mul(gt.z, __ldg(eqc + (uint64_t)j * O + gt.y));
            w_out[i] = make_uint4(w[0], w[1], w[2], 0u);
        }
        if (i < I) {
            uint32_t s[3] = {0u, 0u, 0u};
            const uint32_t k0 = __ldg(ax_off + i), k1 = __ldg(ax_off + i + 1);
            for (uint32_t k = k0; k < k1; k++) {
                const uint2 gt = __ldg(ax_g + k);  // (z, c)
                for (uint32_t j = 0; j < reps; j++) s[j] = add(s[j], mul(gt.y, __ldg(eqc + (uint64_t)j * O + gt.x)));
            }
            a_out[i] = make_uint4(s[0], s[1], s[2], 0u);
        }
    }
}

// w_j[k] (1 - r_j) for the mul gates of even input rows x, w_j[k] r_j for odd x: the weights
// of k_hg_round1, whose sum over the gates of rows 2i and 2i+1 is then hg folded at r_j.
__global__ void k_scale_weights(uint64_t I, const uint32_t* __restrict__ mx_off, const uint4* __restrict__ w4,
                                uint4* __restrict__ w4r, uint4 r) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; x < I; x += stride) {
        const bool odd = x & 1;
        const uint32_t s0 = odd ? r.x : sub(1u, r.x), s1 = odd ? r.y : sub(1u, r.y), s2 = odd ? r.z : sub(1u, r.z);
        const uint32_t k0 = __ldg(mx_off + x), k1 = __ldg(mx_off + x + 1);
        for (uint32_t k = k0; k < k1; k++) {
            const uint4 w = __ldg(w4 + k);
            w4r[k] = make_uint4(mul(w.x, s0), mul(w.y, s1), mul(w.z, s2), 0u);
        }
    }
}

// ---------------------------------------------------------------- finishers
// Evaluations at 0, 1, 2 of every repetition's round polynomial for one lane; with vx the
// phase-two sums are multiplied by v(rx) (h = v(rx) * s).
struct RoundFin {
    RedScratch red;
    uint32_t* out;       // R x 3 x N
    const uint32_t* vx;  // R x N, or null
    uint32_t N, reps;
    __device__ void operator()(uint32_t lane) const {
        for (uint32_t j = 0; j < reps; j++) {
            uint32_t p0 = take(red, 3 * j, N, lane), p1 = take(red, 3 * j + 1, N, lane);
            uint32_t p2 = m31::eval_at_two(p0, p1, take(red, 3 * j + 2, N, lane));
            if (vx) {
                const uint32_t x = vx[(size_t)j * N + lane];
                p0 = mul(p0, x); p1 = mul(p1, x); p2 = mul(p2, x);
            }
            out[(size_t)(3 * j) * N + lane] = p0;
            out[(size_t)(3 * j + 1) * N + lane] = p1;
            out[(size_t)(3 * j + 2) * N + lane] = p2;
            if (red.evals_dev) {
                red.evals_dev[(size_t)(3 * j) * N + lane] = p0;
                red.evals_dev[(size_t)(3 * j + 1) * N + lane] = p1;
                red.evals_dev[(size_t)(3 * j + 2) * N + lane] = p2;
            }
        }
    }
};

// Round evaluations from two sums per repetition, p0 and p2raw: p1 is the round's claim less
// p0 (an honest prover's round polynomial meets p0 + p1 = claim, the verifier's check in
// sumcheck.hpp:152, so p1 is the same field element as its direct sum).  The claim is
// `claim` (R x N, written by the host before the launch), or without it the previous
// round's polynomial at its challenge r_j, eval_degree2 of the three evaluations in
// red.evals_dev, which this finisher then overwrites (each lane read before it is written).
// With vx (phase two) the sums are multiplied by v(rx) first; the claim is of the multiplied
// polynomial.
struct ClaimFin {
    RedScratch red;
    uint32_t* out;            // R x 3 x N
    const uint32_t* claim;    // R x N, or null
    uint32_t r[3];
    uint32_t N, reps;
    const uint32_t* vx = nullptr;  // R x N, or null
    __device__ void operator()(uint32_t lane) const {
        uint32_t* dev = red.evals_dev;
        for (uint32_t j = 0; j < reps; j++) {
            uint32_t cl;
            if (claim) {
                cl = __ldcv(claim + (size_t)j * N + lane);
            } else {
                const uint32_t rj = j == 0 ? r[0] : (j == 1 ? r[1] : r[2]);
                cl = m31::eval_degree2(dev[(size_t)(3 * j) * N + lane], dev[(size_t)(3 * j + 1) * N + lane],
                                       dev[(size_t)(3 * j + 2) * N + lane], rj);
            }
            uint32_t p0 = take(red, 2 * j, N, lane), p2raw = take(red, 2 * j + 1, N, lane);
            if (vx) {
                const uint32_t x = vx[(size_t)j * N + lane];
                p0 = mul(p0, x);
                p2raw = mul(p2raw, x);
            }
            const uint32_t p1 = sub(cl, p0), p2 = m31::eval_at_two(p0, p1, p2raw);
            out[(size_t)(3 * j) * N + lane] = p0;
            out[(size_t)(3 * j + 1) * N + lane] = p1;
            out[(size_t)(3 * j + 2) * N + lane] = p2;
            if (dev) {
                dev[(size_t)(3 * j) * N + lane] = p0;
                dev[(size_t)(3 * j + 1) * N + lane] = p1;
                dev[(size_t)(3 * j + 2) * N + lane] = p2;
            }
        }
    }
};

struct CopyFin {
    RedScratch red;
    uint32_t* out;  // reps x N
    uint32_t N, reps;
    __device__ void operator()(uint32_t lane) const {
        for (uint32_t j = 0; j < reps; j++) out[(size_t)j * N + lane] = take(red, j, N, lane);
    }
};

// p0 += f0 h0, p1 += f1 h1, p2raw += (f0 + f1)(h0 + h1) for four copies, each product added
// unreduced below 2^32 (mac_lazy): the reduction's 64-bit totals are reduced by the finisher.
__device__ __forceinline__ void accum_pair(uint32_t (&acc)[3][4], const uint32_t (&f0)[4], const uint32_t (&f1)[4],
                                           const uint32_t (&h0)[4], const uint32_t (&h1)[4]) {
#pragma unroll
    for (int l = 0; l < 4; l++) {
        acc[0][l] = m31::mac_lazy(acc[0][l], f0[l], h0[l]);
        acc[1][l] = m31::mac_lazy(acc[1][l], f1[l], h1[l]);
        acc[2][l] = m31::mac_lazy(acc[2][l], add(f0[l], f1[l]), add(h0[l], h1[l]));
    }
}

// p0 += f0 h0 and p2raw += (f0 + f1)(h0 + h1) for four copies (mac_lazy): the two sums of a
// round whose p1 comes from its claim (ClaimFin).
__device__ __forceinline__ void accum_pair2(uint32_t (&acc)[2][4], const uint32_t (&f0)[4], const uint32_t (&f1)[4],
                                            const uint32_t (&h0)[4], const uint32_t (&h1)[4]) {
#pragma unroll
    for (int l = 0; l < 4; l++) {
        acc[0][l] = m31::mac_lazy(acc[0][l], f0[l], h0[l]);
        acc[1][l] = m31::mac_lazy(acc[1][l], add(f0[l], f1[l]), add(h0[l], h1[l]));
    }
}

// ---------------------------------------------------------------- asynchronous row staging
// cp.async copies (global -> shared, no registers held while in flight) let a thread keep
// several iterations' rows in flight.  Each thread copies and later reads back only its
// own slots, so no barrier is needed between threads; a slot is refilled only after the
// values read from it have been used.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int K>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(K) : "memory");
}

// ---------------------------------------------------------------- gathered gate terms
// h_j += sum over mul gates k0 .. k1 - 1 of v[y_k] w_j[k] for the thread's four copies, each
// product added unreduced below 2^32 (mac_lazy).  U gates per step: their gathers (a gate
// index, then a row) are all in flight before the products (8 registers per extra gate).
template <int R, int U>
__device__ __forceinline__ void gate_terms(const uint32_t* __restrict__ v, const uint4* __restrict__ mx_g,
                                           const uint4* __restrict__ w4, uint32_t k0, uint32_t k1, uint32_t N,
                                           uint32_t lane0, uint32_t (&h)[R][4]) {
    uint32_t k = k0;
    for (; U > 1 && k + U <= k1; k += U) {
        uint32_t y[U];
        uint4 w[U], vy[U];
#pragma unroll
        for (int u = 0; u < U; u++) y[u] = __ldg(&mx_g[k + u].x);
#pragma unroll
        for (int u = 0; u < U; u++) w[u] = __ldg(w4 + k + u);
#pragma unroll
        for (int u = 0; u < U; u++) vy[u] = ld4(v, y[u], N, lane0);
#pragma unroll
        for (int u = 0; u < U; u++)
#pragma unroll
            for (int j = 0; j < R; j++)
#pragma unroll
                for (int l = 0; l < 4; l++) h[j][l] = m31::mac_lazy(h[j][l], comp(vy[u], l), comp(w[u], j));
    }
    for (; k < k1; k++) {
        const uint32_t y = __ldg(&mx_g[k].x);
        const uint4 w = __ldg(w4 + k);
        const uint4 vy = ld4(v, y, N, lane0);
#pragma unroll
        for (int j = 0; j < R; j++)
#pragma unroll
            for (int l = 0; l < 4; l++) h[j][l] = m31::mac_lazy(h[j][l], comp(vy, l), comp(w, j));
    }
}

// ---------------------------------------------------------------- phase one: hg build + round 0
// For each pair (x0, x1) = (2i, 2i+1): hg_j[x] = a_j[x] + sum over mul gates (x, y, k) of
// v[y] * w_j[k], then the round-0 sums of v(x) hg_j(x).  hg is not stored: round 1
// (k_hg_round1) rebuilds it, which costs the gathers again but saves writing and re-reading
// R full-width tables.  All repetitions in one thread: each gathered v[y] row serves the R
// weights.
// The round reads 4 bytes per copy and row and is bound by the integer multiply pipe, so it
// sums only p0 = sum f0 h0 and p2raw = sum (f0 + f1)(h0 + h1), each product added unreduced
// below 2^32 (mac_lazy); p1 is the layer's claim less p0 (ClaimFin).  A pair whose rows both
// lack mul gates (most pairs of a wide layer) has the scalar add weights as h and costs two
// products per copy and repetition: f0 a0 and (f0 + f1)(a0 + a1).  The pair's two input rows,
// their add-gate weights and CSR offsets are staged by cp.async kStages - 1 iterations ahead.
constexpr int kStages = 3;
constexpr int kStageFields = 5;  // v(2i), v(2i+1), a(2i), a(2i+1), (off(2i), off(2i+1), off(2i+2))
constexpr int kMaxStagedSmem = kStages * kStageFields * 16 * 256;
constexpr int kHg0Gates = 2, kHg1Gates = 2;  // gathers in flight per thread (gate_terms)

template <int R>
__global__ void __launch_bounds__(256, 2) k_hg_round0(const uint32_t* __restrict__ v, uint64_t npairs,
                                                      const uint32_t* __restrict__ pairs,
                                                      const uint32_t* __restrict__ mx_off,
                                                      const uint4* __restrict__ mx_g, const uint4* __restrict__ a4,
                                                      const uint4* __restrict__ w4, Geo g, RedScratch red,
                                                      const uint32_t* claim, uint32_t* evals_out) {
    extern __shared__ uint4 ring[];  // kStages x kStageFields x blockDim.x
    const TileIdx t = tile_idx(g);
    const uint32_t B = blockDim.x, tid = threadIdx.x;
    uint32_t acc[2 * R][4];  // 2j: p0, 2j + 1: p2raw
#pragma unroll
    for (int c = 0; c < 2 * R; c++)
#pragma unroll
        for (int l = 0; l < 4; l++) acc[c][l] = 0u;
    // adds the mul-gate terms of input row x (gates k0 .. k1) to h, canonical before and after
    auto gates = [&](uint32_t k0, uint32_t k1, uint32_t (&h)[R][4]) {
        if (k0 == k1) return;
        gate_terms<R, kHg0Gates>(v, mx_g, w4, k0, k1, g.N, t.lane0, h);
#pragma unroll
        for (int j = 0; j < R; j++)
#pragma unroll
            for (int l = 0; l < 4; l++) h[j][l] = m31::from_u32(h[j][l]);
    };
    if (t.active) {
        // iteration i works on pair q = group_at(pairs, i) (rows 2q, 2q+1); the list entry of
        // the iteration staged next is loaded one iteration ahead of its staging
        const uint64_t step = (uint64_t)gridDim.x * g.rps;
        const uint64_t i0 = (uint64_t)blockIdx.x * g.rps + t.rs;
        auto stage = [&](uint64_t i, uint64_t q, int slot) {
            if (i < npairs) {
                uint4* st = ring + (size_t)slot * kStageFields * B + tid;
                cp_async16(st, v + (2 * q) * g.N + t.lane0);
                cp_async16(st + B, v + (2 * q + 1) * g.N + t.lane0);
                cp_async16(st + 2 * B, a4 + 2 * q);
                cp_async16(st + 3 * B, a4 + 2 * q + 1);
                cp_async8(st + 4 * B, mx_off + 2 * q);
                cp_async4(reinterpret_cast<uint32_t*>(st + 4 * B) + 2, mx_off + 2 * q + 2);
            }
            cp_async_commit();  // one group per iteration, empty past the end
        };
#pragma unroll
        for (int s = 0; s < kStages - 1; s++) {
            const uint64_t i = i0 + s * step;
            stage(i, i < npairs ? group_at(pairs, i) : 0, s);
        }
        uint64_t next_q = i0 + (kStages - 1) * step < npairs ? group_at(pairs, i0 + (kStages - 1) * step) : 0;
        int slot = 0;
        for (uint64_t i = i0; i < npairs; i += step) {
            // refill the slot read in the previous iteration, then wait for this one
            const uint64_t is = i + (kStages - 1) * step, q = next_q;
            next_q = is + step < npairs ? group_at(pairs, is + step) : 0;
            stage(is, q, slot == 0 ? kStages - 1 : slot - 1);
            cp_async_wait<kStages - 1>();
            const uint4* st = ring + (size_t)slot * kStageFields * B + tid;
            const uint4 f0 = st[0], f1 = st[B], off = st[4 * B];
            uint32_t f01[4];
#pragma unroll
            for (int l = 0; l < 4; l++) f01[l] = add(comp(f0, l), comp(f1, l));
            if (off.x == off.z) {  // neither row has mul gates
#pragma unroll
                for (int j = 0; j < R; j++) {
                    const uint32_t a0 = reinterpret_cast<const uint32_t*>(st + 2 * B)[j];
                    const uint32_t a01 = add(a0, reinterpret_cast<const uint32_t*>(st + 3 * B)[j]);
#pragma unroll
                    for (int l = 0; l < 4; l++) {
                        acc[2 * j][l] = m31::mac_lazy(acc[2 * j][l], comp(f0, l), a0);
                        acc[2 * j + 1][l] = m31::mac_lazy(acc[2 * j + 1][l], f01[l], a01);
                    }
                }
            } else {
                // h = hg(2q), then hg(2q) + hg(2q+1): row 2q+1's add weights and gate terms are
                // added onto row 2q's hg
                uint32_t h[R][4];
                const uint4 a0 = st[2 * B], a1 = st[3 * B];
#pragma unroll
                for (int j = 0; j < R; j++)
#pragma unroll
                    for (int l = 0; l < 4; l++) h[j][l] = comp(a0, j);
                gates(off.x, off.y, h);
#pragma unroll
                for (int j = 0; j < R; j++)
#pragma unroll
                    for (int l = 0; l < 4; l++) {
                        acc[2 * j][l] = m31::mac_lazy(acc[2 * j][l], comp(f0, l), h[j][l]);
                        h[j][l] = add(h[j][l], comp(a1, j));
                    }
                gates(off.y, off.z, h);
#pragma unroll
                for (int j = 0; j < R; j++)
#pragma unroll
                    for (int l = 0; l < 4; l++) acc[2 * j + 1][l] = m31::mac_lazy(acc[2 * j + 1][l], f01[l], h[j][l]);
            }
            slot = slot + 1 == kStages ? 0 : slot + 1;
        }
        cp_async_wait<0>();
    }
    __syncthreads();  // the ring is reused as the reduction's scratch (sums below 2^32 are
                      // added as they are: the finisher reduces the 64-bit totals)
    reduce_group<2 * R>(acc, g, t.active, red, 0,
                        ClaimFin{red, evals_out, claim, {0u, 0u, 0u}, g.N, (uint32_t)R});
}

// ---------------------------------------------------------------- phase one, round 1
// Round 1 with hg rebuilt rather than read: for each output pair i the four source rows
// x = 4i..4i+3 get hg_j[x] = a_j[x] + sum over mul gates (x, y, k) of v[y] w_j[k] again,
// already folded (the fold is linear: the gate weights come scaled by 1 - r_j for even x and
// r_j for odd x, so one sum over both rows' gates is the folded hg),
// and hg_j and the layer input are folded at r_j into rows 2i, 2i+1 of hdst_j / fdst_j
// (what receive_challenge of round 0 would have left, sumcheck_helper.hpp:104-133), which
// are stored and summed into the round-1 evaluations.  All repetitions in one thread, as in
// k_hg_round0: each gathered v[y] row serves the R weights.  When neither source row of an
// output row has mul gates, its hg is the same for every copy: fold(a_j[x0], a_j[x1], r_j)
// is computed once.  The sums are those of k_hg_round0, p0 and p2raw with mac_lazy (p1 is
// the claim, round 0's polynomial at r_j, less p0); after the first row of a pair only its
// f and h are kept, for p2raw.
template <int R>
__global__ void __launch_bounds__(256) k_hg_round1(const uint32_t* __restrict__ v, uint64_t npairs,
                                                   const uint32_t* __restrict__ quads,
                                                   const uint32_t* __restrict__ mx_off, const uint4* __restrict__ mx_g,
                                                   const uint4* __restrict__ a4, const uint4* __restrict__ w4r,
                                                   RoundPtrs p, Geo g, RedScratch red, uint32_t* evals_out) {
    const TileIdx t = tile_idx(g);
    uint32_t acc[2 * R][4];  // 2j: p0, 2j + 1: p2raw
#pragma unroll
    for (int c = 0; c < 2 * R; c++)
#pragma unroll
        for (int l = 0; l < 4; l++) acc[c][l] = 0u;
    if (t.active) {
        // iteration ii works on output pair i = group_at(quads, ii) (source rows 4i .. 4i+3)
        const uint64_t step = (uint64_t)gridDim.x * g.rps;
        uint64_t ii = (uint64_t)blockIdx.x * g.rps + t.rs;
        uint64_t next_i = ii < npairs ? group_at(quads, ii) : 0;
        for (; ii < npairs; ii += step) {
            const uint64_t i = next_i;
            next_i = ii + step < npairs ? group_at(quads, ii + step) : 0;
            const uint4 o4 = __ldg(reinterpret_cast<const uint4*>(mx_off + 4 * i));  // off(4i .. 4i+3)
            const uint32_t o_end = __ldg(mx_off + 4 * i + 4);
            const uint32_t off[5] = {o4.x, o4.y, o4.z, o4.w, o_end};
            uint32_t fe[R][4], he[R][4];
#pragma unroll
            for (int s = 0; s < 2; s++) {
                const uint64_t x0 = 4 * i + 2 * s;
                const uint4 v0 = ld4(v, x0, g.N, t.lane0), v1 = ld4(v, x0 + 1, g.N, t.lane0);
                const uint4 a0 = __ldg(a4 + x0), a1 = __ldg(a4 + x0 + 1);
                // fold(hg(x0), hg(x1), r_j) = fold(a_j(x0), a_j(x1), r_j) plus the gate terms of
                // rows x0 and x1 (gates off(x0) .. off(x0 + 2), contiguous) with their weights
                // scaled by 1 - r_j and r_j (w4r, k_scale_weights)
                uint32_t h[R][4];
#pragma unroll
                for (int j = 0; j < R; j++) {
                    const uint32_t hs = fold(comp(a0, j), comp(a1, j), p.r[j]);
#pragma unroll
                    for (int l = 0; l < 4; l++) h[j][l] = hs;
                }
                if (off[2 * s] != off[2 * s + 2]) {
                    gate_terms<R, kHg1Gates>(v, mx_g, w4r, off[2 * s], off[2 * s + 2], g.N, t.lane0, h);
#pragma unroll
                    for (int j = 0; j < R; j++)
#pragma unroll
                        for (int l = 0; l < 4; l++) h[j][l] = m31::from_u32(h[j][l]);
                }
#pragma unroll
                for (int j = 0; j < R; j++) {
                    uint32_t f[4];
#pragma unroll
                    for (int l = 0; l < 4; l++) f[l] = fold(comp(v0, l), comp(v1, l), p.r[j]);
                    // null: round 2 refolds the layer input instead of reading stored copies
                    if (p.fdst[0]) st4(p.fdst[j], 2 * i + s, g.N, t.lane0, mk4(f));
                    // a copy-independent hg row is recomputed by round 2 (k_round with H1)
                    if (off[2 * s] != off[2 * s + 2]) st4(p.hdst[j], 2 * i + s, g.N, t.lane0, mk4(h[j]));
#pragma unroll
                    for (int l = 0; l < 4; l++) {
                        if (s == 0) {
                            acc[2 * j][l] = m31::mac_lazy(acc[2 * j][l], f[l], h[j][l]);
                            fe[j][l] = f[l];
                            he[j][l] = h[j][l];
                        } else {
                            acc[2 * j + 1][l] =
                                m31::mac_lazy(acc[2 * j + 1][l], add(fe[j][l], f[l]), add(he[j][l], h[j][l]));
                        }
                    }
                }
            }
        }
    }
    reduce_group<2 * R>(acc, g, t.active, red, 0,
                        ClaimFin{red, evals_out, nullptr, {p.r[0], p.r[1], p.r[2]}, g.N, (uint32_t)R});
}

// ---------------------------------------------------------------- persistent phase tail
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ uint32_t ld_acquire_sys(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.sys.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
// Loads that see this kernel's own earlier writes (L2, not the non-coherent read-only path).
__device__ __forceinline__ uint4 ld4cg(const uint32_t* base, uint64_t row, uint32_t N, uint32_t lane0) {
    return __ldcg(reinterpret_cast<const uint4*>(base + row * N + lane0));
}

// The fold and sums of a round are those of k_round<false, LANE_HG, true> (receive_challenge
// + poly_eval_at, sumcheck_helper.hpp:68-133) over this CTA's lane group and every row.
template <bool LANE_HG>
__global__ void __launch_bounds__(256) k_tail(TailArgs a) {
    extern __shared__ uint32_t tsm[];
    __shared__ uint32_t rch[3];
    __shared__ int stop;
    const Geo g = a.g;
    const TileIdx t = tile_idx(g);
    const uint32_t R = a.reps, tid = threadIdx.x, B = blockDim.x, tpr = g.tpr, rps = g.rps;
    const uint32_t S0 = 1u << (a.n - a.kt + 1);  // rows of the first round's source tables
    // shared memory: phase two's scalar tables (two buffers of R x S0), the reduction scratch
    // (12 x B), the totals (R x 12 x tpr)
    uint32_t* sbuf = tsm;
    uint32_t* red = tsm + (LANE_HG ? 0 : 2 * 3 * S0);
    uint32_t* tot = red + 12 * B;
    if (tid == 0) stop = 0;
    if (!LANE_HG) {
        // every CTA keeps its own copy of the scalar tables (the source of round kt)
        for (uint32_t j = 0; j < R; j++) {
            const uint32_t* src = (a.kt & 1) ? a.hB[j] : a.hA[j];
            for (uint32_t e = tid; e < S0; e += B) sbuf[j * S0 + e] = src[e];
        }
    }
    __syncthreads();
    for (uint32_t k = a.kt; k < a.n; k++) {
        if (k == a.kt) {
            if (tid < 3) rch[tid] = a.r_first[tid];
        } else if (tid == 0) {
            const uint32_t want = a.tag_base + (k - 1);
            const uint32_t* slot = a.mbox + 4 + 4 * (k - 1);
            const uint64_t t0 = global_ns();
            uint32_t ns = 32;
            int st = 0;
            while (ld_acquire_sys(slot) != want) {
                if (ld_acquire_sys(a.mbox) != 0) {
                    st = 1;
                    break;
                }
                if (global_ns() - t0 > a.wait_ns) {
                    st = 2;
                    break;
                }
                __nanosleep(ns);
                if (ns < 1024) ns *= 2;
            }
            if (st == 2) *reinterpret_cast<volatile unsigned int*>(a.err) = 1u;
            if (st == 0)
                for (int j = 0; j < 3; j++) rch[j] = reinterpret_cast<const volatile uint32_t*>(slot)[1 + j];
            stop = st;
        }
        __syncthreads();
        if (stop) return;
        const uint64_t npairs = 1ull << (a.n - k - 1);
        const bool odd = k & 1;
        // phase two: scalar tables ping-pong in shared memory (source of round kt in buffer 0)
        const uint32_t* ssrc = sbuf + ((k - a.kt) & 1) * 3 * S0;
        uint32_t* sdst = sbuf + (((k - a.kt) & 1) ^ 1) * 3 * S0;
        uint32_t acc[3][3][4];
#pragma unroll
        for (int j = 0; j < 3; j++)
#pragma unroll
            for (int c = 0; c < 3; c++)
#pragma unroll
                for (int l = 0; l < 4; l++) acc[j][c][l] = 0u;
        if (t.active) {
            for (uint64_t i = t.rs; i < npairs; i += rps) {
#pragma unroll
                for (int j = 0; j < 3; j++) {
                    if ((uint32_t)j >= R) break;
                    const uint32_t r = rch[j];
                    const uint32_t* fs = odd ? a.fB[j] : a.fA[j];
                    uint32_t* fd = odd ? a.fA[j] : a.fB[j];
                    uint32_t f0[4], f1[4], h0[4], h1[4];
                    uint4 x[4];
#pragma unroll
                    for (int q = 0; q < 4; q++) x[q] = ld4cg(fs, 4 * i + q, g.N, t.lane0);
                    if (LANE_HG) {
                        const uint32_t* hs = odd ? a.hB[j] : a.hA[j];
                        uint32_t* hd = odd ? a.hA[j] : a.hB[j];
                        uint4 y[4];
#pragma unroll
                        for (int q = 0; q < 4; q++) y[q] = ld4cg(hs, 4 * i + q, g.N, t.lane0);
#pragma unroll
                        for (int l = 0; l < 4; l++) {
                            h0[l] = fold(comp(y[0], l), comp(y[1], l), r);
                            h1[l] = fold(comp(y[2], l), comp(y[3], l), r);
                        }
                        st4(hd, 2 * i, g.N, t.lane0, mk4(h0));
                        st4(hd, 2 * i + 1, g.N, t.lane0, mk4(h1));
                    } else {
                        const uint32_t* sv = ssrc + j * S0 + 4 * i;
                        const uint32_t s0 = fold(sv[0], sv[1], r), s1 = fold(sv[2], sv[3], r);
                        if (t.q == 0) {
                            sdst[j * S0 + 2 * i] = s0;
                            sdst[j * S0 + 2 * i + 1] = s1;
                        }
#pragma unroll
                        for (int l = 0; l < 4; l++) {
                            h0[l] = s0;
                            h1[l] = s1;
                        }
                    }
#pragma unroll
                    for (int l = 0; l < 4; l++) {
                        f0[l] = fold(comp(x[0], l), comp(x[1], l), r);
                        f1[l] = fold(comp(x[2], l), comp(x[3], l), r);
                    }
                    st4(fd, 2 * i, g.N, t.lane0, mk4(f0));
                    st4(fd, 2 * i + 1, g.N, t.lane0, mk4(f1));
                    accum_pair(acc[j], f0, f1, h0, h1);
                }
            }
        }
        // totals per (repetition, component, lane) over the CTA's row slices
#pragma unroll
        for (int j = 0; j < 3; j++) {
            if ((uint32_t)j >= R) break;
            __syncthreads();
#pragma unroll
            for (int c = 0; c < 3; c++)
#pragma unroll
                for (int l = 0; l < 4; l++) red[(c * 4 + l) * B + tid] = t.active ? acc[j][c][l] : 0u;
            __syncthreads();
            for (uint32_t o = tid; o < 12 * tpr; o += B) {
                const uint32_t cl = o / tpr, q = o - cl * tpr;
                unsigned long long sum = 0;
                for (uint32_t rr = 0; rr < rps; rr++) sum += red[cl * B + rr * tpr + q];
                tot[(j * 12 + cl) * tpr + q] = reduce64(sum);
            }
        }
        __syncthreads();
        // evaluations at 0, 1, 2 of every repetition for this group's lanes (RoundFin)
        const uint32_t lanes = 4 * tpr, lane_base = blockIdx.y * lanes;
        for (uint32_t li = tid; li < lanes; li += B) {
            const uint32_t q = li >> 2, l = li & 3, lane = lane_base + li;
            for (uint32_t j = 0; j < R; j++) {
                uint32_t p0 = tot[(j * 12 + 0 * 4 + l) * tpr + q];
                uint32_t p1 = tot[(j * 12 + 1 * 4 + l) * tpr + q];
                const uint32_t c2 = tot[(j * 12 + 2 * 4 + l) * tpr + q];
                uint32_t p2 = m31::eval_at_two(p0, p1, c2);
                if (!LANE_HG) {
                    const uint32_t xv = a.vx[(size_t)j * g.N + lane];
                    p0 = mul(p0, xv);
                    p1 = mul(p1, xv);
                    p2 = mul(p2, xv);
                }
                a.evals_out[(size_t)(3 * j) * g.N + lane] = p0;
                a.evals_out[(size_t)(3 * j + 1) * g.N + lane] = p1;
                a.evals_out[(size_t)(3 * j + 2) * g.N + lane] = p2;
                if (k + 1 == a.n) {
                    const uint32_t* fd = odd ? a.fA[j] : a.fB[j];
                    a.rows_out[(size_t)(2 * j) * g.N + lane] = __ldcg(fd + lane);
                    a.rows_out[(size_t)(2 * j + 1) * g.N + lane] = __ldcg(fd + g.N + lane);
                }
            }
        }
        __threadfence_system();
        __syncthreads();
        if (tid == 0) atomicAdd_system(a.done, 1u);
    }
}

// ---------------------------------------------------------------- fold + reduce round
// FOLD: the inputs hold 4*npairs rows; rows (4i, 4i+1) and (4i+2, 4i+3) are folded at the
// previous round's challenge r_j into rows 2i and 2i+1 of the outputs, which are stored
// for the next round and summed into this round's evaluations.  Without FOLD the inputs
// hold 2*npairs rows and are summed directly (first round of phase two).
// SHARED: every repetition folds the same source table (the layer input at round 1).
// LANE_HG: hg is a per-copy table (phase one); otherwise it is a copy-independent scalar
// table s_j (phase two) and the finisher multiplies the sums by vx_j.
// HR (phase-one rounds 2 and 3, HR = round - 1): a source hg row q covers the 2^HR input
// rows q 2^HR .. (q+1) 2^HR - 1; where none of them has mul gates the previous round did
// not store it, and it is recomputed by folding their add weights a_j at the challenges of
// rounds 0 .. HR-1.  Round 2 (HR = 1) does not store its own output rows of that kind.
template <bool SHARED, bool LANE_HG, bool FOLD, int HR = 0>
__global__ void __launch_bounds__(256) k_round(RoundPtrs p, uint64_t npairs, const uint32_t* __restrict__ vx, Geo g,
                                               uint32_t reps, RedScratch red, uint32_t* evals_out) {
    const TileIdx t = tile_idx(g);
    const uint32_t j = blockIdx.x % reps, cx = blockIdx.x / reps, nx = gridDim.x / reps;
    // selects instead of p.x[j]: a dynamic index into kernel parameters would copy them to the stack
    const uint32_t* __restrict__ fs = (SHARED || j == 0) ? p.fsrc[0] : (j == 1 ? p.fsrc[1] : p.fsrc[2]);
    const uint32_t* __restrict__ hs = j == 0 ? p.hsrc[0] : (j == 1 ? p.hsrc[1] : p.hsrc[2]);
    uint32_t* __restrict__ fd = j == 0 ? p.fdst[0] : (j == 1 ? p.fdst[1] : p.fdst[2]);
    uint32_t* __restrict__ hd = j == 0 ? p.hdst[0] : (j == 1 ? p.hdst[1] : p.hdst[2]);
    const uint32_t r = j == 0 ? p.r[0] : (j == 1 ? p.r[1] : p.r[2]);
    uint32_t acc[2][4] = {};  // p0, p2raw
    if (t.active) {
        uint64_t i = (uint64_t)cx * g.rps + t.rs;
        const uint64_t step = (uint64_t)nx * g.rps;
        if (FOLD && !LANE_HG) {
            // scalar-h folds: two pairs per iteration, their eight row loads issued together
            auto fold_pair = [&](const uint4 (&a)[4], const uint4& sv, uint64_t ii) {
                const uint32_t s0 = fold(sv.x, sv.y, r), s1 = fold(sv.z, sv.w, r);
                if (t.q == 0 && blockIdx.y == 0) *reinterpret_cast<uint2*>(hd + 2 * ii) = make_uint2(s0, s1);
                uint32_t f0[4], f1[4], h0[4], h1[4];
#pragma unroll
                for (int l = 0; l < 4; l++) {
                    f0[l] = fold(comp(a[0], l), comp(a[1], l), r);
                    f1[l] = fold(comp(a[2], l), comp(a[3], l), r);
                    h0[l] = s0;
                    h1[l] = s1;
                }
                st4(fd, 2 * ii, g.N, t.lane0, mk4(f0));
                st4(fd, 2 * ii + 1, g.N, t.lane0, mk4(f1));
                accum_pair2(acc, f0, f1, h0, h1);
            };
            for (; i + step < npairs; i += 2 * step) {
                uint4 a[4], b[4];
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    a[k] = ld4(fs, 4 * i + k, g.N, t.lane0);
                    b[k] = ld4(fs, 4 * (i + step) + k, g.N, t.lane0);
                }
                const uint4 sa = __ldg(reinterpret_cast<const uint4*>(hs) + i);
                const uint4 sb = __ldg(reinterpret_cast<const uint4*>(hs) + i + step);
                fold_pair(a, sa, i);
                fold_pair(b, sb, i + step);
            }
        }
        for (; i < npairs; i += step) {
            uint32_t f0[4], f1[4], h0[4], h1[4];
            if (FOLD) {
                uint4 a[4];
#pragma unroll
                for (int k = 0; k < 4; k++) a[k] = ld4(fs, 4 * i + k, g.N, t.lane0);
                if (LANE_HG) {
                    uint4 b[4];
                    bool keep0 = true, keep1 = true;  // store output rows 2i, 2i+1
                    if (HR > 0) {
                        constexpr int SPAN = 1 << HR;  // input rows per source row
                        // offsets of input rows 4i SPAN .. 4(i+1) SPAN at the source rows' ends
                        uint32_t off[5];
                        const uint32_t* o = p.hoff + 4 * SPAN * i;
#pragma unroll
                        for (int k = 0; k <= 4; k++) off[k] = __ldg(o + k * SPAN);
                        const uint32_t r0 = j == 0 ? p.hr[0][0] : (j == 1 ? p.hr[0][1] : p.hr[0][2]);
                        const uint32_t r1 = j == 0 ? p.hr[1][0] : (j == 1 ? p.hr[1][1] : p.hr[1][2]);
#pragma unroll
                        for (int k = 0; k < 4; k++) {
                            if (off[k] == off[k + 1]) {
                                const uint32_t* a = reinterpret_cast<const uint32_t*>(p.ha + (4 * i + k) * SPAN) + j;
                                uint32_t hv = fold(__ldg(a), __ldg(a + 4), r0);
                                if (HR == 2) hv = fold(hv, fold(__ldg(a + 8), __ldg(a + 12), r0), r1);
                                b[k] = make_uint4(hv, hv, hv, hv);
                            } else {
                                b[k] = ld4(hs, 4 * i + k, g.N, t.lane0);
                            }
                        }
                        if (HR == 1) {
                            keep0 = off[0] != off[2];
                            keep1 = off[2] != off[4];
                        }
                    } else {
#pragma unroll
                        for (int k = 0; k < 4; k++) b[k] = ld4(hs, 4 * i + k, g.N, t.lane0);
                    }
#pragma unroll
                    for (int l = 0; l < 4; l++) {
                        h0[l] = fold(comp(b[0], l), comp(b[1], l), r);
                        h1[l] = fold(comp(b[2], l), comp(b[3], l), r);
                    }
                    if (keep0) st4(hd, 2 * i, g.N, t.lane0, mk4(h0));
                    if (keep1) st4(hd, 2 * i + 1, g.N, t.lane0, mk4(h1));
                } else {
                    const uint4 s = __ldg(reinterpret_cast<const uint4*>(hs) + i);
                    const uint32_t s0 = fold(s.x, s.y, r), s1 = fold(s.z, s.w, r);
                    if (t.q == 0 && blockIdx.y == 0) *reinterpret_cast<uint2*>(hd + 2 * i) = make_uint2(s0, s1);
#pragma unroll
                    for (int l = 0; l < 4; l++) { h0[l] = s0; h1[l] = s1; }
                }
#pragma unroll
                for (int l = 0; l < 4; l++) {
                    f0[l] = fold(comp(a[0], l), comp(a[1], l), r);
                    f1[l] = fold(comp(a[2], l), comp(a[3], l), r);
                }
                st4(fd, 2 * i, g.N, t.lane0, mk4(f0));
                st4(fd, 2 * i + 1, g.N, t.lane0, mk4(f1));
            } else {
                const uint4 a0 = ld4(fs, 2 * i, g.N, t.lane0), a1 = ld4(fs, 2 * i + 1, g.N, t.lane0);
#pragma unroll
                for (int l = 0; l < 4; l++) { f0[l] = comp(a0, l); f1[l] = comp(a1, l); }
                if (LANE_HG) {
                    const uint4 b0 = ld4(hs, 2 * i, g.N, t.lane0), b1 = ld4(hs, 2 * i + 1, g.N, t.lane0);
#pragma unroll
                    for (int l = 0; l < 4; l++) { h0[l] = comp(b0, l); h1[l] = comp(b1, l); }
                } else {
                    const uint2 s = __ldg(reinterpret_cast<const uint2*>(hs) + i);
#pragma unroll
                    for (int l = 0; l < 4; l++) { h0[l] = s.x; h1[l] = s.y; }
                }
            }
            accum_pair2(acc, f0, f1, h0, h1);
        }
    }
    reduce_group<2>(acc, g, t.active, red, 2 * j,
                    ClaimFin{red, evals_out, nullptr, {p.r[0], p.r[1], p.r[2]}, g.N, reps,
                             LANE_HG ? nullptr : vx});
}

// Phase-one round 2 after a round 1 that stored no folded copies of the layer input, with
// every repetition in one thread (each input row is loaded once for the R repetitions):
// output row 2i + s (s = 0, 1) of f folds input rows 8i + 4s .. 8i + 4s + 3 in pairs at the
// round-0 challenge r0_j (p.hr[0]) and then at the round-1 challenge r_j (p.r), and output
// row 2i + s of hg folds round 1's hg rows 4i + 2s, 4i + 2s + 1 at r_j, a row round 1 did not
// store (both its input rows without mul gates) being recomputed from the add weights at
// r0_j (receive_challenge twice, sumcheck_helper.hpp:104-133).  Output hg rows whose four
// input rows have no mul gates are not stored (round 3 recomputes them), as in
// k_round<.., HR = 1>.
template <int R>
__global__ void __launch_bounds__(256) k_p1_round2(RoundPtrs p, uint64_t npairs, Geo g, RedScratch red,
                                                   uint32_t* evals_out) {
    const TileIdx t = tile_idx(g);
    const uint32_t* __restrict__ v = p.fsrc[0];
    uint32_t acc[2 * R][4];  // 2j: p0, 2j + 1: p2raw
#pragma unroll
    for (int c = 0; c < 2 * R; c++)
#pragma unroll
        for (int l = 0; l < 4; l++) acc[c][l] = 0u;
    if (t.active) {
        for (uint64_t i = (uint64_t)blockIdx.x * g.rps + t.rs; i < npairs; i += (uint64_t)gridDim.x * g.rps) {
            // offsets of input rows 8i, 8i+2, .., 8i+8: round-1 hg row 4i + k covers input rows
            // 8i + 2k, 8i + 2k + 1
            uint32_t off[5];
#pragma unroll
            for (int k = 0; k <= 4; k++) off[k] = __ldg(p.hoff + 8 * i + 2 * k);
            uint32_t fe[R][4], he[R][4];
#pragma unroll
            for (int s = 0; s < 2; s++) {
                const uint64_t q = 8 * i + 4 * s;
                const uint4 x0 = ld4(v, q, g.N, t.lane0), x1 = ld4(v, q + 1, g.N, t.lane0);
                const uint4 x2 = ld4(v, q + 2, g.N, t.lane0), x3 = ld4(v, q + 3, g.N, t.lane0);
                const bool keep = off[2 * s] != off[2 * s + 2];
#pragma unroll
                for (int j = 0; j < R; j++) {
                    const uint32_t r0 = p.hr[0][j], r1 = p.r[j];
                    uint4 b[2];
#pragma unroll
                    for (int e = 0; e < 2; e++) {
                        const int k = 2 * s + e;
                        if (off[k] == off[k + 1]) {
                            const uint32_t* a = reinterpret_cast<const uint32_t*>(p.ha + (4 * i + k) * 2) + j;
                            const uint32_t hv = fold(__ldg(a), __ldg(a + 4), r0);
                            b[e] = make_uint4(hv, hv, hv, hv);
                        } else {
                            b[e] = ld4(p.hsrc[j], 4 * i + k, g.N, t.lane0);
                        }
                    }
                    uint32_t f[4], h[4];
#pragma unroll
                    for (int l = 0; l < 4; l++) {
                        f[l] = fold(fold(comp(x0, l), comp(x1, l), r0), fold(comp(x2, l), comp(x3, l), r0), r1);
                        h[l] = fold(comp(b[0], l), comp(b[1], l), r1);
                    }
                    st4(p.fdst[j], 2 * i + s, g.N, t.lane0, mk4(f));
                    if (keep) st4(p.hdst[j], 2 * i + s, g.N, t.lane0, mk4(h));
#pragma unroll
                    for (int l = 0; l < 4; l++) {
                        if (s == 0) {
                            acc[2 * j][l] = m31::mac_lazy(acc[2 * j][l], f[l], h[l]);
                            fe[j][l] = f[l];
                            he[j][l] = h[l];
                        } else {
                            acc[2 * j + 1][l] =
                                m31::mac_lazy(acc[2 * j + 1][l], add(fe[j][l], f[l]), add(he[j][l], h[l]));
                        }
                    }
                }
            }
        }
    }
    reduce_group<2 * R>(acc, g, t.active, red, 0,
                        ClaimFin{red, evals_out, nullptr, {p.r[0], p.r[1], p.r[2]}, g.N, (uint32_t)R});
}

// Shared-source rounds (phase-1 round 1, phase-2 rounds 0 and 1) with every repetition in
// one thread: the layer input rows are read once for all R repetitions instead of once per
// repetition-CTA.  Same semantics as k_round<true, LANE_HG, FOLD>.
template <int R, bool LANE_HG, bool FOLD>
__global__ void __launch_bounds__(256) k_round_shared(RoundPtrs p, uint64_t npairs, const uint32_t* __restrict__ vx,
                                                      Geo g, RedScratch red, uint32_t* evals_out) {
    const TileIdx t = tile_idx(g);
    const uint32_t* __restrict__ fs = p.fsrc[0];
    uint32_t acc[2 * R][4] = {};  // 2j: p0, 2j + 1: p2raw
    if (t.active) {
        for (uint64_t i = (uint64_t)blockIdx.x * g.rps + t.rs; i < npairs; i += (uint64_t)gridDim.x * g.rps) {
            uint4 a[4];
            if (FOLD) {
#pragma unroll
                for (int k = 0; k < 4; k++) a[k] = ld4(fs, 4 * i + k, g.N, t.lane0);
            } else {
                a[0] = ld4(fs, 2 * i, g.N, t.lane0);
                a[1] = ld4(fs, 2 * i + 1, g.N, t.lane0);
            }
#pragma unroll
            for (int j = 0; j < R; j++) {
                const uint32_t r = p.r[j];
                uint32_t f0[4], f1[4], h0[4], h1[4];
                if (FOLD) {
#pragma unroll
                    for (int l = 0; l < 4; l++) {
                        f0[l] = fold(comp(a[0], l), comp(a[1], l), r);
                        f1[l] = fold(comp(a[2], l), comp(a[3], l), r);
                    }
                    if (p.fdst[j]) {  // null: the next round refolds the source instead
                        st4(p.fdst[j], 2 * i, g.N, t.lane0, mk4(f0));
                        st4(p.fdst[j], 2 * i + 1, g.N, t.lane0, mk4(f1));
                    }
                } else {
#pragma unroll
                    for (int l = 0; l < 4; l++) { f0[l] = comp(a[0], l); f1[l] = comp(a[1], l); }
                }
                if (LANE_HG) {
                    uint4 b[4];
#pragma unroll
                    for (int k = 0; k < 4; k++) b[k] = ld4(p.hsrc[j], 4 * i + k, g.N, t.lane0);
#pragma unroll
                    for (int l = 0; l < 4; l++) {
                        h0[l] = fold(comp(b[0], l), comp(b[1], l), r);
                        h1[l] = fold(comp(b[2], l), comp(b[3], l), r);
                    }
                    st4(p.hdst[j], 2 * i, g.N, t.lane0, mk4(h0));
                    st4(p.hdst[j], 2 * i + 1, g.N, t.lane0, mk4(h1));
                } else if (FOLD) {
                    const uint4 s = __ldg(reinterpret_cast<const uint4*>(p.hsrc[j]) + i);
                    const uint32_t s0 = fold(s.x, s.y, r), s1 = fold(s.z, s.w, r);
                    if (t.q == 0 && blockIdx.y == 0) *reinterpret_cast<uint2*>(p.hdst[j] + 2 * i) = make_uint2(s0, s1);
#pragma unroll
                    for (int l = 0; l < 4; l++) { h0[l] = s0; h1[l] = s1; }
                } else {
                    const uint2 s = __ldg(reinterpret_cast<const uint2*>(p.hsrc[j]) + i);
#pragma unroll
                    for (int l = 0; l < 4; l++) { h0[l] = s.x; h1[l] = s.y; }
                }
#pragma unroll
                for (int l = 0; l < 4; l++) {
                    acc[2 * j][l] = add(acc[2 * j][l], mul(f0[l], h0[l]));
                    acc[2 * j + 1][l] = add(acc[2 * j + 1][l], mul(add(f0[l], f1[l]), add(h0[l], h1[l])));
                }
            }
        }
    }
    reduce_group<2 * R>(acc, g, t.active, red, 0,
                        ClaimFin{red, evals_out, nullptr, {p.r[0], p.r[1], p.r[2]}, g.N, (uint32_t)R,
                                 LANE_HG ? nullptr : vx});
}

// Phase-two round 2 from the layer input: round 1 stored only its folded scalar tables, not
// the folded copies f1_j(q) = fold(v(2q), v(2q+1), r0_j), which would be written once and
// read once; here each output pair i refolds the eight input rows 8i..8i+7 at r0_j (p.hr[0])
// and then at r1_j (p.r), stores rows 2i, 2i+1 of f2_j and the folded scalars, and sums the
// round-2 evaluations (receive_challenge + poly_eval_at, sumcheck_helper.hpp:68-133).  All
// repetitions in one thread: the eight rows are read once for the R tables.  The rows of the
// next kRowStages - 1 iterations are staged with cp.async while an iteration computes (each
// thread copies and reads back only its own slots).
constexpr int kRowStages = 3;
constexpr int kRowRingSmem = kRowStages * 8 * 16 * 256;

template <int R>
__global__ void __launch_bounds__(256) k_p2_round2(RoundPtrs p, uint64_t npairs, const uint32_t* __restrict__ vx,
                                                   Geo g, RedScratch red, uint32_t* evals_out) {
    extern __shared__ uint4 rows8[];  // kRowStages x 8 x blockDim.x
    const TileIdx t = tile_idx(g);
    const uint32_t B = blockDim.x, tid = threadIdx.x;
    const uint32_t* __restrict__ fs = p.fsrc[0];
    uint32_t acc[2 * R][4];  // 2j: p0, 2j + 1: p2raw
#pragma unroll
    for (int c = 0; c < 2 * R; c++)
#pragma unroll
        for (int l = 0; l < 4; l++) acc[c][l] = 0u;
    if (t.active) {
        const uint64_t step = (uint64_t)gridDim.x * g.rps;
        const uint64_t i0 = (uint64_t)blockIdx.x * g.rps + t.rs;
        auto stage = [&](uint64_t i, int slot) {
            if (i < npairs) {
                uint4* st = rows8 + (size_t)slot * 8 * B + tid;
#pragma unroll
                for (int k = 0; k < 8; k++) cp_async16(st + k * B, fs + (8 * i + k) * g.N + t.lane0);
            }
            cp_async_commit();  // one group per iteration, empty past the end
        };
#pragma unroll
        for (int q = 0; q < kRowStages - 1; q++) stage(i0 + q * step, q);
        int slot = 0;
        for (uint64_t i = i0; i < npairs; i += step) {
            // refill the slot read in the previous iteration, then wait for this one
            stage(i + (kRowStages - 1) * step, slot == 0 ? kRowStages - 1 : slot - 1);
            cp_async_wait<kRowStages - 1>();
            const uint4* st = rows8 + (size_t)slot * 8 * B + tid;
            uint4 a[8];
#pragma unroll
            for (int k = 0; k < 8; k++) a[k] = st[k * B];
            slot = slot + 1 == kRowStages ? 0 : slot + 1;
#pragma unroll
            for (int j = 0; j < R; j++) {
                const uint32_t r0 = p.hr[0][j], r1 = p.r[j];
                const uint4 sv = __ldg(reinterpret_cast<const uint4*>(p.hsrc[j]) + i);
                const uint32_t s0 = fold(sv.x, sv.y, r1), s1 = fold(sv.z, sv.w, r1);
                if (t.q == 0 && blockIdx.y == 0) *reinterpret_cast<uint2*>(p.hdst[j] + 2 * i) = make_uint2(s0, s1);
                uint32_t f0[4], f1[4], h0[4], h1[4];
#pragma unroll
                for (int l = 0; l < 4; l++) {
                    const uint32_t g0 = fold(comp(a[0], l), comp(a[1], l), r0), g1 = fold(comp(a[2], l), comp(a[3], l), r0);
                    const uint32_t g2 = fold(comp(a[4], l), comp(a[5], l), r0), g3 = fold(comp(a[6], l), comp(a[7], l), r0);
                    f0[l] = fold(g0, g1, r1);
                    f1[l] = fold(g2, g3, r1);
                    h0[l] = s0;
                    h1[l] = s1;
                }
                st4(p.fdst[j], 2 * i, g.N, t.lane0, mk4(f0));
                st4(p.fdst[j], 2 * i + 1, g.N, t.lane0, mk4(f1));
                // sums kept below 2^32 without reduction (mac_lazy), canonical at the end
                const uint32_t hs = add(s0, s1);
#pragma unroll
                for (int l = 0; l < 4; l++) {
                    acc[2 * j][l] = m31::mac_lazy(acc[2 * j][l], f0[l], h0[l]);
                    acc[2 * j + 1][l] = m31::mac_lazy(acc[2 * j + 1][l], add(f0[l], f1[l]), hs);
                }
            }
        }
        cp_async_wait<0>();
    }
#pragma unroll
    for (int c = 0; c < 2 * R; c++)
#pragma unroll
        for (int l = 0; l < 4; l++) acc[c][l] = m31::from_u32(acc[c][l]);
    __syncthreads();  // the ring is reused as the reduction's scratch
    reduce_group<2 * R>(acc, g, t.active, red, 0,
                        ClaimFin{red, evals_out, nullptr, {p.r[0], p.r[1], p.r[2]}, g.N, (uint32_t)R, vx});
}

// x == x mod p for any 64-bit x: x = hi 2^32 + lo and 2^32 == 2 (mod 2^31 - 1), so the result
// lo + 2 hi < 3 * 2^32.  Formed with a shift and an add with carry on the integer ALU (the
// multiply pipe is what the sum kernels saturate).  After it, four more products
// <= (p - 1)^2 keep a 64-bit sum below 3 * 2^32 + 2^64 - 2^35 + 16 < 2^64.
__device__ __forceinline__ uint64_t fold64(uint64_t x) {
    const uint32_t lo = (uint32_t)x, hi = (uint32_t)(x >> 32);
    uint32_t nl, nh;
    asm("{\n\t"
        ".reg .u32 t;\n\t"
        "shl.b32 t, %2, 1;\n\t"
        "add.cc.u32 %0, %3, t;\n\t"
        "shr.u32 t, %2, 31;\n\t"
        "addc.u32 %1, t, 0;\n\t"
        "}"
        : "=r"(nl), "=r"(nh)
        : "r"(hi), "r"(lo));
    return ((uint64_t)nh << 32) | nl;
}

// acc += a * b with one 32 x 32 -> 64-bit multiply-add.
__device__ __forceinline__ void mad64(uint64_t& acc, uint32_t a, uint32_t b) {
    asm("mad.wide.u32 %0, %1, %2, %0;" : "+l"(acc) : "r"(a), "r"(b));
}

// Phase-two round 0 (no fold): p0_j = sum f(2i) s_j(2i), p1_j = sum f(2i+1) s_j(2i+1),
// p2raw_j = sum (f(2i) + f(2i+1)) (s_j(2i) + s_j(2i+1)) over the layer input f = v, for
// all R repetitions in one thread so that each row read serves the R scalar tables.  With
// 4 bytes read per copy and row, the products are summed unreduced in 64-bit accumulators
// (one multiply-add each, every factor canonical) and folded every third pair.  The pair's
// two rows and the R scalar pairs are staged by cp.async kP2Stages - 1 iterations ahead.
// (SumcheckMultiLinearProdHelper::poly_eval_at on the first phase-two round,
// sumcheck_helper.hpp:68-102, with hg = v(rx) s: the finisher multiplies by vx.)
constexpr int kP2Stages = 6;
constexpr int kP2Fields = 4;  // v(2i), v(2i+1), (s_0, s_1) pairs, (s_2 pair, unused)
constexpr int kMaxP2Smem = kP2Stages * kP2Fields * 16 * 256;

struct P2Src {
    const uint32_t* f;     // the layer input, 2 npairs rows
    const uint32_t* s[3];  // the repetitions' scalar tables s_j
};

template <int R>
__global__ void __launch_bounds__(256, 2) k_p2_round0(P2Src src, uint64_t npairs, const uint32_t* __restrict__ vx,
                                                      Geo g, RedScratch red, uint32_t* evals_out) {
    extern __shared__ uint4 ring[];  // kP2Stages x kP2Fields x blockDim.x
    const TileIdx t = tile_idx(g);
    const uint32_t B = blockDim.x, tid = threadIdx.x;
    const uint32_t* __restrict__ fs = src.f;
    const uint32_t* hsrc[R];
#pragma unroll
    for (int j = 0; j < R; j++) hsrc[j] = src.s[j];
    uint64_t acc[3 * R][4];
#pragma unroll
    for (int c = 0; c < 3 * R; c++)
#pragma unroll
        for (int l = 0; l < 4; l++) acc[c][l] = 0ull;
    if (t.active) {
        const uint64_t step = (uint64_t)gridDim.x * g.rps;
        const uint64_t i0 = (uint64_t)blockIdx.x * g.rps + t.rs;
        auto stage = [&](uint64_t i, int slot) {
            if (i < npairs) {
                uint4* st = ring + (size_t)slot * kP2Fields * B + tid;
                cp_async16(st, fs + (2 * i) * g.N + t.lane0);
                cp_async16(st + B, fs + (2 * i + 1) * g.N + t.lane0);
#pragma unroll
                for (int j = 0; j < R; j++)
                    cp_async8(reinterpret_cast<uint2*>(st + (2 + j / 2) * B) + (j & 1), hsrc[j] + 2 * i);
            }
            cp_async_commit();  // one group per iteration, empty past the end
        };
#pragma unroll
        for (int s = 0; s < kP2Stages - 1; s++) stage(i0 + s * step, s);
        int slot = 0;
        uint32_t since_fold = 0;
        for (uint64_t i = i0; i < npairs; i += step) {
            stage(i + (kP2Stages - 1) * step, slot == 0 ? kP2Stages - 1 : slot - 1);
            cp_async_wait<kP2Stages - 1>();
            const uint4* st = ring + (size_t)slot * kP2Fields * B + tid;
            const uint4 f0 = st[0], f1 = st[B];
            uint32_t sa[R], sb[R], sab[R];
#pragma unroll
            for (int j = 0; j < R; j++) {
                const uint2 sj = reinterpret_cast<const uint2*>(st + (2 + j / 2) * B)[j & 1];
                sa[j] = sj.x;
                sb[j] = sj.y;
                sab[j] = add(sj.x, sj.y);
            }
#pragma unroll
            for (int l = 0; l < 4; l++) {
                const uint32_t a = comp(f0, l), b = comp(f1, l), ab = add(a, b);
#pragma unroll
                for (int j = 0; j < R; j++) {
                    acc[3 * j][l] += (uint64_t)a * sa[j];
                    acc[3 * j + 1][l] += (uint64_t)b * sb[j];
                    acc[3 * j + 2][l] += (uint64_t)ab * sab[j];
                }
            }
            if (++since_fold == 3) {
                since_fold = 0;
#pragma unroll
                for (int c = 0; c < 3 * R; c++)
#pragma unroll
                    for (int l = 0; l < 4; l++) acc[c][l] = fold64(acc[c][l]);
            }
            slot = slot + 1 == kP2Stages ? 0 : slot + 1;
        }
        cp_async_wait<0>();
    }
    uint32_t out[3 * R][4];
#pragma unroll
    for (int c = 0; c < 3 * R; c++)
#pragma unroll
        for (int l = 0; l < 4; l++) out[c][l] = reduce64(acc[c][l]);
    __syncthreads();  // the ring is reused as the reduction's scratch
    reduce_group<3 * R>(out, g, t.active, red, 0, RoundFin{red, evals_out, vx, g.N, (uint32_t)R});
}

// ---------------------------------------------------------------- phase two: rounds 0 and 1 in one pass
// Round 1 folds the layer input v and the scalar tables s_j at the round-0 challenge r
// (receive_challenge, sumcheck_helper.hpp:104-133), so its sums are quadratic in r.  Over a
// group of four input rows y = 4i..4i+3 (values v0..v3, scalars s0..s3), round 1's pair is
// f0 = (1-r) v0 + r v1, f1 = (1-r) v2 + r v3 (h0, h1 alike from s), and
//   p0_1    = sum f0 h0             = (1-r)^2 E00 + r(1-r) KE + r^2 E11,
//   p1_1    = sum f1 h1             = (1-r)^2 F22 + r(1-r) KF + r^2 F33,
//   p2raw_1 = sum (f0 + f1)(h0 + h1) = (1-r)^2 U00 + r(1-r) KU + r^2 U11,
// with E00 = sum v0 s0, E11 = sum v1 s1 and the cross sum KE = sum v0 s1 + v1 s0 = QE - E00 - E11,
// QE = sum (v0 + v1)(s0 + s1) (F.. and QF from rows 2, 3), and U.. the same over u0 = v0 + v2,
// u1 = v1 + v3 and t0 = s0 + s2, t1 = s1 + s3.  Round 0's sums (poly_eval_at over the pairs
// (4i, 4i+1), (4i+2, 4i+3), sumcheck_helper.hpp:68-102) are p0_0 = E00 + F22,
// p1_0 = E11 + F33 and p2raw_0 = QE + QF.  One pass over v therefore yields both rounds: the
// finisher writes round 0's evaluations (times v(rx), since h = v(rx) s) for the transcript
// and the 9R canonical sums to `sums`, and k_p2_round1_fin evaluates round 1 from them once r
// is known — round 1 never reads v.
// One copy per thread: nine products per repetition and group, summed unreduced in 64-bit
// sums that fold64 folds every fourth group (below 3 * 2^32 + 4 (p - 1)^2 < 2^64).  A warp
// covers 32 consecutive copies of one row group and stages it kP01Stages - 1 groups ahead
// with one 16-byte cp.async per thread (row wl / 8, copies 4 (wl % 8) ..), plus the group's
// scalars (s0..s3) and (t0, t1, s0 + s1, s2 + s3) of each repetition from lanes 0 .. 2R-1;
// after the wait a __syncwarp makes the whole slot visible and each thread reads its
// copy's four values transposed.
constexpr int kP01Stages = 8;
constexpr int kP01Sums = 9;       // E00, E11, QE, F22, F33, QF, U00, U11, QU
constexpr int kP01WarpSlot = 608;  // bytes per warp and stage: 4 rows x 32 copies x 4 B + 6 x 16 B scalars

struct P01Src {
    const uint32_t* v;     // the layer input, 4 ngroups rows
    const uint32_t* s[3];  // s_j: 4 ngroups scalars (s0..s3 of each group)
    const uint32_t* t[3];  // (t0, t1, s0 + s1, s2 + s3) of each group: 4 ngroups scalars
};

// Round 0's evaluations from the nine sums of each repetition, times v(rx); the sums are
// kept canonical in `sums` for round 1.
struct P01Fin {
    RedScratch red;
    uint32_t* out;       // R x 3 x N
    const uint32_t* vx;  // R x N
    uint32_t* sums;      // 9R x N
    uint32_t N, reps;
    __device__ void operator()(uint32_t lane) const {
        for (uint32_t j = 0; j < reps; j++) {
            uint32_t m[kP01Sums];
#pragma unroll
            for (int k = 0; k < kP01Sums; k++) {
                m[k] = take(red, kP01Sums * j + k, N, lane);
                sums[(size_t)(kP01Sums * j + k) * N + lane] = m[k];
            }
            const uint32_t p0 = add(m[0], m[3]), p1 = add(m[1], m[4]), p2raw = add(m[2], m[5]);
            const uint32_t x = vx[(size_t)j * N + lane];
            out[(size_t)(3 * j) * N + lane] = mul(p0, x);
            out[(size_t)(3 * j + 1) * N + lane] = mul(p1, x);
            out[(size_t)(3 * j + 2) * N + lane] = mul(m31::eval_at_two(p0, p1, p2raw), x);
        }
    }
};

template <int R>
__global__ void __launch_bounds__(256, 2) k_p2_round01(P01Src src, uint64_t ngroups, const uint32_t* __restrict__ quads,
                                                       const uint32_t* __restrict__ vx, Geo g, RedScratch red,
                                                       uint32_t* evals_out, uint32_t* sums_out) {
    extern __shared__ uint4 ring01[];  // kP01Stages x warps x kP01WarpSlot bytes
    const uint32_t tid = threadIdx.x, wl = tid & 31, w = tid >> 5, nw = blockDim.x >> 5;
    const uint32_t L = g.tpr, rs = tid / L;  // L: copies per row slice, a multiple of 32
    const bool active = rs < g.rps;          // uniform over a warp
    const uint64_t N = g.N;
    // this thread's global copy, and the 16 bytes it stages: row wl / 8 of the group, copies
    // 4 (wl % 8) .. of the warp's 32
    const uint64_t warp_lane0 = (uint64_t)blockIdx.y * L + (tid - rs * L - wl);
    const uint32_t* __restrict__ vst = src.v + (wl >> 3) * N + warp_lane0 + 4 * (wl & 7);
    const uint32_t* __restrict__ sst = nullptr;
    if (wl < 2 * R) {
        const uint32_t j = wl >> 1;
        sst = (wl & 1) ? (j == 0 ? src.t[0] : (j == 1 ? src.t[1] : src.t[2]))
                       : (j == 0 ? src.s[0] : (j == 1 ? src.s[1] : src.s[2]));
    }
    char* const ring = reinterpret_cast<char*>(ring01);
    uint64_t acc[R * kP01Sums];
#pragma unroll
    for (int c = 0; c < R * kP01Sums; c++) acc[c] = 0ull;
    if (active) {
        const uint64_t step = (uint64_t)gridDim.x * g.rps;
        const uint64_t i0 = (uint64_t)blockIdx.x * g.rps + rs;
        // iteration i works on row group q = group_at(quads, i) (rows 4q .. 4q+3); the list
        // entry of the iteration staged next is loaded one iteration ahead of its staging
        auto stage = [&](uint64_t i, uint64_t q, int slot) {
            if (i < ngroups) {
                char* st = ring + ((size_t)slot * nw + w) * kP01WarpSlot;
                cp_async16(st + 16 * wl, vst + 4 * q * N);
                if (sst) cp_async16(st + 512 + 16 * wl, sst + 4 * q);
            }
            cp_async_commit();  // one group per iteration, empty past the end
        };
#pragma unroll
        for (int s = 0; s < kP01Stages - 1; s++) {
            const uint64_t i = i0 + s * step;
            stage(i, i < ngroups ? group_at(quads, i) : 0, s);
        }
        uint64_t next_q = i0 + (kP01Stages - 1) * step < ngroups ? group_at(quads, i0 + (kP01Stages - 1) * step) : 0;
        int slot = 0;
        uint32_t it = 0;
        for (uint64_t i = i0; i < ngroups; i += step, it++) {
            __syncwarp();  // every lane has read the slot refilled next
            const uint64_t is = i + (kP01Stages - 1) * step, q = next_q;
            next_q = is + step < ngroups ? group_at(quads, is + step) : 0;
            stage(is, q, slot == 0 ? kP01Stages - 1 : slot - 1);
            cp_async_wait<kP01Stages - 1>();
            __syncwarp();  // the other lanes' copies of this slot are visible
            const char* st = ring + ((size_t)slot * nw + w) * kP01WarpSlot;
            const uint32_t* rows = reinterpret_cast<const uint32_t*>(st);
            const uint32_t x0 = rows[wl], x1 = rows[32 + wl], x2 = rows[64 + wl], x3 = rows[96 + wl];
            const uint4* sc = reinterpret_cast<const uint4*>(st + 512);
            const uint32_t u0 = add(x0, x2), u1 = add(x1, x3), w01 = add(x0, x1), w23 = add(x2, x3), wu = add(u0, u1);
#pragma unroll
            for (int j = 0; j < R; j++) {
                const uint4 sv = sc[2 * j], tv = sc[2 * j + 1];
                uint64_t* a = acc + kP01Sums * j;
                mad64(a[0], x0, sv.x);
                mad64(a[1], x1, sv.y);
                mad64(a[2], w01, tv.z);
                mad64(a[3], x2, sv.z);
                mad64(a[4], x3, sv.w);
                mad64(a[5], w23, tv.w);
                mad64(a[6], u0, tv.x);
                mad64(a[7], u1, tv.y);
                mad64(a[8], wu, add(tv.x, tv.y));
            }
            if ((it & 3) == 3) {
#pragma unroll
                for (int c = 0; c < R * kP01Sums; c++) acc[c] = fold64(acc[c]);
            }
            slot = slot + 1 == kP01Stages ? 0 : slot + 1;
        }
        cp_async_wait<0>();
    }
    uint32_t out[R * kP01Sums];
#pragma unroll
    for (int c = 0; c < R * kP01Sums; c++) out[c] = reduce64(acc[c]);
    __syncthreads();  // the ring is reused as the reduction's scratch
    reduce_group1<R * kP01Sums>(out, g, active, red, P01Fin{red, evals_out, vx, sums_out, g.N, (uint32_t)R});
}

// Round 1 of phase two at the round-0 challenges r_j from the sums of k_p2_round01: block 0
// evaluates every copy's p0_1, p1_1, p2_1 (times v(rx)) and publishes them like a round
// kernel's finisher; the other blocks fold the scalar tables at r_j for round 2,
// s'_j(2i) = fold(s_j(4i), s_j(4i+1), r_j), s'_j(2i+1) = fold(s_j(4i+2), s_j(4i+3), r_j).
struct P1Fold {
    const uint32_t* s[3];
    uint32_t* sd[3];
    uint32_t r[3];
};

__global__ void __launch_bounds__(256) k_p2_round1_fin(const uint32_t* __restrict__ sums, const uint32_t* __restrict__ vx,
                                                       P1Fold f, uint64_t ngroups, uint32_t N, uint32_t reps,
                                                       uint32_t* evals_out, uint32_t* evals_dev, unsigned int* done) {
    const uint32_t tid = threadIdx.x, B = blockDim.x;
    if (blockIdx.x == 0) {
        for (uint32_t j = 0; j < reps; j++) {
            const uint32_t r = j == 0 ? f.r[0] : (j == 1 ? f.r[1] : f.r[2]);
            const uint32_t omr = sub(1u, r);
            const uint32_t c0 = mul(omr, omr), c1 = mul(r, omr), c2 = mul(r, r);
            for (uint32_t lane = tid; lane < N; lane += B) {
                uint32_t m[kP01Sums];
#pragma unroll
                for (int k = 0; k < kP01Sums; k++) m[k] = __ldg(sums + (size_t)(kP01Sums * j + k) * N + lane);
                // the cross sums KE, KF, KU from QE, QF, QU
#pragma unroll
                for (int k = 2; k < kP01Sums; k += 3) m[k] = sub(sub(m[k], m[k - 2]), m[k - 1]);
                const uint32_t p0 = add(add(mul(c0, m[0]), mul(c1, m[2])), mul(c2, m[1]));
                const uint32_t p1 = add(add(mul(c0, m[3]), mul(c1, m[5])), mul(c2, m[4]));
                const uint32_t p2raw = add(add(mul(c0, m[6]), mul(c1, m[8])), mul(c2, m[7]));
                const uint32_t x = __ldg(vx + (size_t)j * N + lane);
                const uint32_t e0 = mul(p0, x), e1 = mul(p1, x), e2 = mul(m31::eval_at_two(p0, p1, p2raw), x);
                evals_out[(size_t)(3 * j) * N + lane] = e0;
                evals_out[(size_t)(3 * j + 1) * N + lane] = e1;
                evals_out[(size_t)(3 * j + 2) * N + lane] = e2;
                if (evals_dev) {
                    evals_dev[(size_t)(3 * j) * N + lane] = e0;
                    evals_dev[(size_t)(3 * j + 1) * N + lane] = e1;
                    evals_dev[(size_t)(3 * j + 2) * N + lane] = e2;
                }
            }
        }
        if (done) {
            __threadfence_system();
            __syncthreads();
            if (tid == 0) atomicAdd_system(done, 1u);
        }
        return;
    }
    const uint64_t total = (uint64_t)reps * ngroups, stride = (uint64_t)(gridDim.x - 1) * B;
    for (uint64_t idx = (uint64_t)(blockIdx.x - 1) * B + tid; idx < total; idx += stride) {
        const uint32_t j = (uint32_t)(idx / ngroups);
        const uint64_t i = idx - (uint64_t)j * ngroups;
        const uint32_t r = j == 0 ? f.r[0] : (j == 1 ? f.r[1] : f.r[2]);
        const uint32_t* sj = j == 0 ? f.s[0] : (j == 1 ? f.s[1] : f.s[2]);
        uint32_t* dj = j == 0 ? f.sd[0] : (j == 1 ? f.sd[1] : f.sd[2]);
        const uint4 sv = __ldg(reinterpret_cast<const uint4*>(sj) + i);
        reinterpret_cast<uint2*>(dj)[i] = make_uint2(fold(sv.x, sv.y, r), fold(sv.z, sv.w, r));
    }
}

// ---------------------------------------------------------------- phase two: s(y)
// s_j[y] = sum over mul gates (z, x, y, c) of eqc_j[z] * eq_rx_j[x] * c: the
// copy-independent factor of h(y) = v(rx) s(y) (sumcheck_helper.hpp:250-259).
__global__ void k_s_build(uint64_t I, uint64_t O, const uint32_t* __restrict__ my_off, const uint4* __restrict__ my_g,
                          const uint32_t* __restrict__ eqc, const uint32_t* __restrict__ eqrx, uint32_t* __restrict__ s_out,
                          uint64_t s_stride, uint32_t reps) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t y = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; y < I; y += stride) {
        uint32_t s[3] = {0u, 0u, 0u};
        const uint32_t k0 = __ldg(my_off + y), k1 = __ldg(my_off + y + 1);
        for (uint32_t k = k0; k < k1; k++) {
            const uint4 gt = __ldg(my_g + k);  // (x, z, c, 0)
            for (uint32_t j = 0; j < reps; j++) {
                const uint32_t e = mul(__ldg(eqc + (uint64_t)j * O + gt.y), __ldg(eqrx + (uint64_t)j * I + gt.x));
                s[j] = add(s[j], mul(e, gt.z));
            }
        }
        for (uint32_t j = 0; j < reps; j++) s_out[(uint64_t)j * s_stride + y] = s[j];
    }
}

// k_s_build over groups of four rows (I a multiple of 4), one thread per group, which also
// writes t_j(i) = (s_j(4i) + s_j(4i+2), s_j(4i+1) + s_j(4i+3), s_j(4i) + s_j(4i+1),
// s_j(4i+2) + s_j(4i+3)), the scalar pair sums that k_p2_round01 stages with each group.
__global__ void k_s_build4(uint64_t I, uint64_t O, const uint32_t* __restrict__ my_off, const uint4* __restrict__ my_g,
                           const uint32_t* __restrict__ eqc, const uint32_t* __restrict__ eqrx, uint32_t* __restrict__ s_out,
                           uint32_t* __restrict__ t_out, uint64_t s_stride, uint32_t reps) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x, ngroups = I / 4;
    for (uint64_t gi = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; gi < ngroups; gi += stride) {
        uint32_t s[3][4] = {};
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const uint64_t y = 4 * gi + k;
            const uint32_t k0 = __ldg(my_off + y), k1 = __ldg(my_off + y + 1);
            for (uint32_t e = k0; e < k1; e++) {
                const uint4 gt = __ldg(my_g + e);  // (x, z, c, 0)
                for (uint32_t j = 0; j < reps; j++) {
                    const uint32_t w = mul(__ldg(eqc + (uint64_t)j * O + gt.y), __ldg(eqrx + (uint64_t)j * I + gt.x));
                    s[j][k] = add(s[j][k], mul(w, gt.z));
                }
            }
        }
        for (uint32_t j = 0; j < reps; j++) {
            reinterpret_cast<uint4*>(s_out + (uint64_t)j * s_stride)[gi] = make_uint4(s[j][0], s[j][1], s[j][2], s[j][3]);
            reinterpret_cast<uint4*>(t_out + (uint64_t)j * s_stride)[gi] =
                make_uint4(add(s[j][0], s[j][2]), add(s[j][1], s[j][3]), add(s[j][0], s[j][1]), add(s[j][2], s[j][3]));
        }
    }
}

// ---------------------------------------------------------------- weighted row sums
// out[j] = sum_z eq_j[z] * vals[z]: eval_multilinear at r_j for each repetition.
template <int R>
__global__ void __launch_bounds__(256) k_wsum(const uint32_t* __restrict__ vals, uint64_t rows,
                                              const uint32_t* __restrict__ eq, Geo g, RedScratch red,
                                              uint32_t* out) {
    const TileIdx t = tile_idx(g);
    uint32_t acc[R][4];
#pragma unroll
    for (int c = 0; c < R; c++)
#pragma unroll
        for (int l = 0; l < 4; l++) acc[c][l] = 0u;
    if (t.active) {
        for (uint64_t z = (uint64_t)blockIdx.x * g.rps + t.rs; z < rows; z += (uint64_t)gridDim.x * g.rps) {
            const uint4 v = ld4(vals, z, g.N, t.lane0);
#pragma unroll
            for (int j = 0; j < R; j++) {
                const uint32_t w = __ldg(eq + (uint64_t)j * rows + z);
#pragma unroll
                for (int l = 0; l < 4; l++) acc[j][l] = add(acc[j][l], mul(comp(v, l), w));
            }
        }
    }
    reduce_group<R>(acc, g, t.active, red, 0, CopyFin{red, out, g.N, (uint32_t)R});
}

uint32_t grid_1d(uint64_t n, uint32_t block) {
    uint64_t b = (n + block - 1) / block;
    if (b < 1) b = 1;
    if (b > 152ull * 16) b = 152ull * 16;
    return (uint32_t)b;
}

// Row tile with repetition-split CTAs: gridDim.x = reps x row chunks.
LaunchShape rep_shape(const Geo& g, uint64_t rows, uint32_t block, uint32_t ctas_cap, uint32_t reps) {
    LaunchShape s = row_shape(g, rows, block, ctas_cap / reps, 2);
    s.grid.x *= reps;
    return s;
}

}  // namespace

// Row iterations a thread of a reducing kernel makes at least (when the table has that many
// rows): each CTA ends with a reduction epilogue (shared-memory sums, one 64-bit atomic per
// component and copy, the last-CTA finisher), which small grids pay less often.
constexpr uint32_t kMinRowIters = 4;

LaunchShape row_shape(const Geo& g, uint64_t rows, uint32_t block, uint32_t ctas_cap, uint32_t smem_components) {
    LaunchShape s;
    const uint32_t groups = g.N / (4 * g.tpr);
    uint64_t need = (rows + (uint64_t)g.rps * kMinRowIters - 1) / ((uint64_t)g.rps * kMinRowIters);
    uint64_t cap = ctas_cap / groups;
    if (cap < 1) cap = 1;
    if (need < 1) need = 1;
    s.grid = dim3((uint32_t)(need < cap ? need : cap), groups, 1);
    s.block = dim3(block, 1, 1);
    s.smem = (size_t)smem_components * 4 * block * sizeof(uint32_t);
    return s;
}

cudaError_t launch_check_canonical(const uint32_t* v, uint64_t n, unsigned int* flag, cudaStream_t s) {
    k_check_canonical<<<grid_1d(n / 4, 256), 256, 0, s>>>(v, n, flag);
    return cudaGetLastError();
}

cudaError_t launch_evaluate(const uint32_t* in, uint32_t* out, uint64_t O, const uint32_t* mo_off, const uint4* mo_g,
                            const uint32_t* ao_off, const uint2* ao_g, const Geo& g, uint32_t block, uint32_t ctas,
                            cudaStream_t s) {
    LaunchShape sh = row_shape(g, O, block, ctas, 0);
    k_evaluate<<<sh.grid, sh.block, 0, s>>>(in, out, O, mo_off, mo_g, ao_off, ao_g, g);
    return cudaGetLastError();
}

cudaError_t launch_canonicalize(uint32_t* v, uint64_t n, cudaStream_t s) {
    k_canonicalize<<<grid_1d(n, 256), 256, 0, s>>>(v, n);
    return cudaGetLastError();
}
cudaError_t launch_gate_sums(bool mul_gates, uint64_t O, uint64_t I, const uint32_t* off, const uint32_t* gates,
                             const uint32_t* eqz, const uint32_t* eqx, const uint32_t* eqy, uint32_t reps,
                             unsigned long long* acc, unsigned int* ticket, uint32_t* out, cudaStream_t s) {
    if (reps < 1 || reps > 3) return cudaErrorInvalidValue;
    const uint32_t grid = grid_1d(O, 256);
    if (mul_gates)
        k_gate_sums<true><<<grid, 256, 0, s>>>(O, I, off, gates, eqz, eqx, eqy, reps, acc, ticket, out);
    else
        k_gate_sums<false><<<grid, 256, 0, s>>>(O, I, off, gates, eqz, eqx, eqy, reps, acc, ticket, out);
    return cudaGetLastError();
}
cudaError_t launch_eq(uint32_t* out, const EqArgs& a, cudaStream_t s) {
    k_eq<<<grid_1d(1ull << a.nvars, 256), 256, 0, s>>>(out, a);
    return cudaGetLastError();
}

cudaError_t launch_scale_weights(uint64_t I, const uint32_t* mx_off, const uint4* w4, uint4* w4r, const uint32_t r[3],
                                 int reps, cudaStream_t s) {
    if (reps < 1 || reps > 3) return cudaErrorInvalidValue;
    const uint4 rr = make_uint4(r[0], reps > 1 ? r[1] : 0u, reps > 2 ? r[2] : 0u, 0u);
    k_scale_weights<<<grid_1d(I, 256), 256, 0, s>>>(I, mx_off, w4, w4r, rr);
    return cudaGetLastError();
}

cudaError_t launch_weights(uint64_t I, uint64_t Gm, uint64_t O, const uint32_t* eqc, const uint4* mx_g,
                           const uint32_t* ax_off, const uint2* ax_g, uint4* a_out, uint4* w_out, uint32_t reps,
                           cudaStream_t s) {
    k_weights<<<grid_1d(I > Gm ? I : Gm, 256), 256, 0, s>>>(I, Gm, O, eqc, mx_g, ax_off, ax_g, a_out, w_out, reps);
    return cudaGetLastError();
}

// Dynamic shared memory of the staged kernels: the cp.async ring, or the reduction's
// scratch where that is larger (they share the allocation).
// Dynamic shared memory of k_hg_round0: the cp.async ring, or the reduction's scratch where
// that is larger (they share the allocation).  Above 48 KiB less the kernel's static shared
// memory a launch needs the opt-in, which is set once per device and instantiation to the
// largest size any launch asks for (block <= 256).
template <int R>
static size_t hg0_smem(size_t ring_bytes, size_t red_bytes) {
    static std::atomic<uint64_t> opted{0};  // one bit per device
    int dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = 1ull << (dev & 63);
    if (!(opted.load(std::memory_order_relaxed) & bit)) {
        cudaFuncSetAttribute(k_hg_round0<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxStagedSmem);
        opted.fetch_or(bit);
    }
    return ring_bytes > red_bytes ? ring_bytes : red_bytes;
}

// Dynamic shared memory of a kernel with a row ring (kRowRingSmem at most): the opt-in above
// 48 KiB is set once per device and kernel (one instance of this function per kernel).
template <auto Kernel>
static size_t ring_smem(size_t bytes) {
    static std::atomic<uint64_t> opted{0};  // one bit per device
    int dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = 1ull << (dev & 63);
    if (!(opted.load(std::memory_order_relaxed) & bit)) {
        cudaFuncSetAttribute(Kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kRowRingSmem);
        opted.fetch_or(bit);
    }
    return bytes;
}

Geo tail_geo(uint32_t N) {
    Geo g;
    g.N = N;
    const uint32_t Q = N / 4;
    uint32_t tpr = Q < 32 ? Q : 32;
    while (tpr > 1 && Q % tpr) tpr--;
    g.tpr = tpr;
    g.rps = 256 / tpr;
    return g;
}

uint32_t tail_max_rows(uint32_t N, int reps, bool lane_hg) {
    // about 256 KiB of table rows per CTA and round, and at most 1024 rows (the scalar tables
    // of phase two sit in shared memory)
    const Geo g = tail_geo(N);
    const uint64_t per_row = (uint64_t)4 * g.tpr * 4 * (lane_hg ? 2 * reps : reps);
    uint64_t rows = (256ull << 10) / per_row;
    if (rows > 1024) rows = 1024;
    uint32_t p = 1;
    while ((uint64_t)p * 2 <= rows) p *= 2;
    return p;
}

cudaError_t launch_tail(bool lane_hg, const TailArgs& a, cudaStream_t s) {
    if (a.reps < 1 || a.reps > 3 || a.kt < 1 || a.kt >= a.n || a.n - a.kt > kMboxRounds - 1)
        return cudaErrorInvalidValue;
    const uint32_t S0 = 1u << (a.n - a.kt + 1);
    if (S0 > 1024 || a.g.tpr < 1 || a.g.tpr > 32 || a.g.rps < 1 || a.g.tpr * a.g.rps > 256 || a.g.N % (4 * a.g.tpr))
        return cudaErrorInvalidValue;
    const dim3 grid(1, a.g.N / (4 * a.g.tpr), 1);
    const size_t smem = 4 * ((lane_hg ? 0 : 2 * 3 * (size_t)S0) + 12 * 256 + 3 * 12 * (size_t)a.g.tpr);
    if (lane_hg)
        k_tail<true><<<grid, 256, smem, s>>>(a);
    else
        k_tail<false><<<grid, 256, smem, s>>>(a);
    return cudaGetLastError();
}

uint32_t launch_stage_words(uint32_t* dst, const uint32_t* const* srcs, uint32_t nsrc, uint64_t n, unsigned int* done,
                            cudaStream_t s, cudaError_t* err) {
    const uint64_t total = n * nsrc;
    uint64_t ctas = (total + 256 * 16 - 1) / (256 * 16);
    if (ctas < 1) ctas = 1;
    if (ctas > 64) ctas = 64;
    k_stage_words<<<(uint32_t)ctas, 256, 0, s>>>(dst, srcs[0], nsrc > 1 ? srcs[1] : nullptr,
                                                 nsrc > 2 ? srcs[2] : nullptr, nsrc, n, done);
    *err = cudaGetLastError();
    return (uint32_t)ctas;
}

cudaError_t launch_hg_round0(int reps, const uint32_t* v, uint64_t npairs, const uint32_t* pairs,
                             const uint32_t* mx_off, const uint4* mx_g, const uint4* a4, const uint4* w4, const Geo& g,
                             uint32_t block, uint32_t ctas, RedScratch red, const uint32_t* claim,
                             uint32_t* evals_out, cudaStream_t s) {
    if (!claim) return cudaErrorInvalidValue;
    // the kernel's launch bound is 256 threads: wider tiles are narrowed to it
    Geo gb = g;
    if (block > 256) block = 256;
    while (gb.tpr > block && gb.tpr % 2 == 0) gb.tpr /= 2;
    if (gb.tpr > block) return cudaErrorInvalidValue;
    gb.rps = block / gb.tpr;
    LaunchShape sh = row_shape(gb, npairs, block, ctas, 2 * reps);
    const size_t ring = (size_t)kStages * kStageFields * sizeof(uint4) * block;
#define GKR_HG0(RR)                                                                                                \
    k_hg_round0<RR><<<sh.grid, sh.block, hg0_smem<RR>(ring, sh.smem), s>>>(v, npairs, pairs, mx_off, mx_g, a4, w4, \
                                                                          gb, red, claim, evals_out)
    switch (reps) {
        case 1: GKR_HG0(1); break;
        case 2: GKR_HG0(2); break;
        case 3: GKR_HG0(3); break;
        default: return cudaErrorInvalidValue;
    }
#undef GKR_HG0
    return cudaGetLastError();
}

cudaError_t launch_hg_round1(int reps, const uint32_t* v, uint64_t npairs, const uint32_t* quads,
                             const uint32_t* mx_off, const uint4* mx_g, const uint4* a4, const uint4* w4r,
                             const RoundPtrs& p, const Geo& g, uint32_t block, uint32_t ctas, RedScratch red,
                             uint32_t* evals_out, cudaStream_t s) {
    if (quads && p.fdst[0]) return cudaErrorInvalidValue;  // stored folded copies need every pair
    if (!red.evals_dev) return cudaErrorInvalidValue;       // the claim is round 0's polynomial
    LaunchShape sh = row_shape(g, npairs, block, ctas, 2 * reps);
#define GKR_HG1(RR) \
    k_hg_round1<RR><<<sh.grid, sh.block, sh.smem, s>>>(v, npairs, quads, mx_off, mx_g, a4, w4r, p, g, red, evals_out)
    switch (reps) {
        case 1: GKR_HG1(1); break;
        case 2: GKR_HG1(2); break;
        case 3: GKR_HG1(3); break;
        default: return cudaErrorInvalidValue;
    }
#undef GKR_HG1
    return cudaGetLastError();
}

// Shared-memory opt-in of k_p2_round0 (as hg0_smem): once per device and instantiation.
template <int R>
static size_t p2_smem(size_t bytes) {
    static std::atomic<uint64_t> opted{0};
    int dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = 1ull << (dev & 63);
    if (!(opted.load(std::memory_order_relaxed) & bit)) {
        cudaFuncSetAttribute(k_p2_round0<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxP2Smem);
        opted.fetch_or(bit);
    }
    return bytes;
}

cudaError_t launch_round(int reps, bool shared_src, bool lane_hg, bool fold_, const RoundPtrs& p, uint64_t npairs,
                         const uint32_t* vx, const Geo& g, uint32_t block, uint32_t ctas, RedScratch red,
                         uint32_t* evals_out, cudaStream_t s) {
    if (reps < 1 || reps > 3) return cudaErrorInvalidValue;
    if (lane_hg && !fold_) return cudaErrorInvalidValue;  // phase-one round 0 lives in k_hg_round0
    if (!fold_ && !shared_src) return cudaErrorInvalidValue;
    if (!fold_) {
        // phase-two round 0 (k_p2_round0): launch bound 256 threads, wider tiles narrowed
        Geo gb = g;
        uint32_t b = block > 256 ? 256 : block;
        while (gb.tpr > b && gb.tpr % 2 == 0) gb.tpr /= 2;
        if (gb.tpr > b) return cudaErrorInvalidValue;
        gb.rps = b / gb.tpr;
        const LaunchShape sh = row_shape(gb, npairs, b, ctas, 3 * reps);
        const size_t ring = (size_t)kP2Stages * kP2Fields * sizeof(uint4) * b;
        const size_t smem = ring > sh.smem ? ring : sh.smem;
        const P2Src src{p.fsrc[0], {p.hsrc[0], p.hsrc[1], p.hsrc[2]}};
        switch (reps) {
            case 1: k_p2_round0<1><<<sh.grid, sh.block, p2_smem<1>(smem), s>>>(src, npairs, vx, gb, red, evals_out); break;
            case 2: k_p2_round0<2><<<sh.grid, sh.block, p2_smem<2>(smem), s>>>(src, npairs, vx, gb, red, evals_out); break;
            default: k_p2_round0<3><<<sh.grid, sh.block, p2_smem<3>(smem), s>>>(src, npairs, vx, gb, red, evals_out); break;
        }
        return cudaGetLastError();
    }
    if (!red.evals_dev) return cudaErrorInvalidValue;  // fold rounds take their claim from it
    if (shared_src) {
        // one read of the shared layer input for all repetitions
        LaunchShape sh = row_shape(g, npairs, block, ctas, 2 * reps);
#define GKR_SHARED(RR, LH, FO) k_round_shared<RR, LH, FO><<<sh.grid, sh.block, sh.smem, s>>>(p, npairs, vx, g, red, evals_out)
#define GKR_SHARED_R(RR)                                  \
    if (lane_hg) GKR_SHARED(RR, true, true);              \
    else GKR_SHARED(RR, false, true);
        switch (reps) {
            case 1: GKR_SHARED_R(1) break;
            case 2: GKR_SHARED_R(2) break;
            default: GKR_SHARED_R(3) break;
        }
#undef GKR_SHARED_R
#undef GKR_SHARED
        return cudaGetLastError();
    }
    LaunchShape sh = rep_shape(g, npairs, block, ctas, reps);
#define GKR_ROUND(SH, LH, FO) k_round<SH, LH, FO><<<sh.grid, sh.block, sh.smem, s>>>(p, npairs, vx, g, reps, red, evals_out)
    if (lane_hg) {
        if (shared_src) GKR_ROUND(true, true, true);
        else GKR_ROUND(false, true, true);
    } else {
        if (shared_src) GKR_ROUND(true, false, true);
        else GKR_ROUND(false, false, true);
    }
#undef GKR_ROUND
    return cudaGetLastError();
}

cudaError_t launch_round_hr(int round, int reps, const RoundPtrs& p, uint64_t npairs, const Geo& g, uint32_t block,
                            uint32_t ctas, RedScratch red, uint32_t* evals_out, cudaStream_t s) {
    if (reps < 1 || reps > 3 || !p.hoff || !p.ha || (round != 2 && round != 3) || !red.evals_dev)
        return cudaErrorInvalidValue;
    LaunchShape sh = rep_shape(g, npairs, block, ctas, reps);
    if (round == 2)
        k_round<false, true, true, 1><<<sh.grid, sh.block, sh.smem, s>>>(p, npairs, nullptr, g, reps, red, evals_out);
    else
        k_round<false, true, true, 2><<<sh.grid, sh.block, sh.smem, s>>>(p, npairs, nullptr, g, reps, red, evals_out);
    return cudaGetLastError();
}

cudaError_t launch_p1_round2(int reps, const RoundPtrs& p, uint64_t npairs, const Geo& g, uint32_t block,
                             uint32_t ctas, RedScratch red, uint32_t* evals_out, cudaStream_t s) {
    if (!p.hoff || !p.ha || !red.evals_dev) return cudaErrorInvalidValue;
    LaunchShape sh = row_shape(g, npairs, block, ctas, 2 * reps);
    switch (reps) {
        case 1: k_p1_round2<1><<<sh.grid, sh.block, sh.smem, s>>>(p, npairs, g, red, evals_out); break;
        case 2: k_p1_round2<2><<<sh.grid, sh.block, sh.smem, s>>>(p, npairs, g, red, evals_out); break;
        case 3: k_p1_round2<3><<<sh.grid, sh.block, sh.smem, s>>>(p, npairs, g, red, evals_out); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_p2_round2(int reps, const RoundPtrs& p, uint64_t npairs, const uint32_t* vx, const Geo& g,
                             uint32_t block, uint32_t ctas, RedScratch red, uint32_t* evals_out, cudaStream_t s) {
    if (!red.evals_dev || block > 256) return cudaErrorInvalidValue;
    LaunchShape sh = row_shape(g, npairs, block, ctas, 2 * reps);
    const size_t ring = (size_t)kRowStages * 8 * sizeof(uint4) * block;
    const size_t smem = ring > sh.smem ? ring : sh.smem;
    switch (reps) {
        case 1: k_p2_round2<1><<<sh.grid, sh.block, ring_smem<k_p2_round2<1>>(smem), s>>>(p, npairs, vx, g, red, evals_out); break;
        case 2: k_p2_round2<2><<<sh.grid, sh.block, ring_smem<k_p2_round2<2>>(smem), s>>>(p, npairs, vx, g, red, evals_out); break;
        case 3: k_p2_round2<3><<<sh.grid, sh.block, ring_smem<k_p2_round2<3>>(smem), s>>>(p, npairs, vx, g, red, evals_out); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// Lanes per row slice of the one-copy-per-thread kernels: the largest divisor of N up to 256.
static uint32_t one_copy_slice(uint32_t N) {
    uint32_t L = N < 256 ? N : 256;
    while (L > 1 && N % L) L--;
    return L;
}

uint32_t p2_round01_groups(uint32_t N) {
    const uint32_t L = N ? one_copy_slice(N) : 1;
    return L % 32 ? 0 : N / L;
}

cudaError_t launch_p2_round01(int reps, const uint32_t* v, const uint32_t* const* s, const uint32_t* const* t,
                              uint64_t ngroups, const uint32_t* quads, const uint32_t* vx, uint32_t N, uint32_t ctas,
                              RedScratch red, uint32_t* evals_out, uint32_t* sums_out, cudaStream_t st) {
    if (reps < 1 || reps > 3 || p2_round01_groups(N) == 0) return cudaErrorInvalidValue;
    if ((reinterpret_cast<uintptr_t>(v) & 15) != 0) return cudaErrorInvalidValue;  // 16-byte cp.async
    Geo g;
    g.N = N;
    g.tpr = one_copy_slice(N);
    g.rps = 256 / g.tpr;
    const uint32_t groups = N / g.tpr;
    uint64_t need = (ngroups + (uint64_t)g.rps * kMinRowIters - 1) / ((uint64_t)g.rps * kMinRowIters), cap = ctas / groups;
    if (cap < 1) cap = 1;
    if (need < 1) need = 1;
    const dim3 grid((uint32_t)(need < cap ? need : cap), groups, 1);
    const size_t ring = (size_t)kP01Stages * 8 * kP01WarpSlot, red_b = (size_t)3 * kP01Sums * 4 * 256;
    const size_t smem = ring > red_b ? ring : red_b;
    P01Src src;
    src.v = v;
    for (int j = 0; j < 3; j++) {
        src.s[j] = j < reps ? s[j] : nullptr;
        src.t[j] = j < reps ? t[j] : nullptr;
    }
    switch (reps) {
        case 1: k_p2_round01<1><<<grid, 256, smem, st>>>(src, ngroups, quads, vx, g, red, evals_out, sums_out); break;
        case 2: k_p2_round01<2><<<grid, 256, smem, st>>>(src, ngroups, quads, vx, g, red, evals_out, sums_out); break;
        default: k_p2_round01<3><<<grid, 256, smem, st>>>(src, ngroups, quads, vx, g, red, evals_out, sums_out); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_p2_round1_fin(int reps, const uint32_t* sums, const uint32_t* vx, const uint32_t* const* s,
                                 uint32_t* const* sd, const uint32_t* r, uint64_t ngroups, uint32_t N,
                                 uint32_t* evals_out, uint32_t* evals_dev, unsigned int* done, cudaStream_t st) {
    if (reps < 1 || reps > 3) return cudaErrorInvalidValue;
    P1Fold f;
    for (int j = 0; j < 3; j++) {
        f.s[j] = j < reps ? s[j] : nullptr;
        f.sd[j] = j < reps ? sd[j] : nullptr;
        f.r[j] = j < reps ? r[j] : 0u;
    }
    const uint32_t fold_blocks = grid_1d((uint64_t)reps * ngroups, 256);
    k_p2_round1_fin<<<1 + fold_blocks, 256, 0, st>>>(sums, vx, f, ngroups, N, (uint32_t)reps, evals_out, evals_dev,
                                                      done);
    return cudaGetLastError();
}

cudaError_t launch_s_build4(uint64_t I, uint64_t O, const uint32_t* my_off, const uint4* my_g, const uint32_t* eqc,
                            const uint32_t* eqrx, uint32_t* s_out, uint32_t* t_out, uint64_t s_stride, uint32_t reps,
                            cudaStream_t s) {
    if (I % 4 || (s_stride % 4)) return cudaErrorInvalidValue;
    k_s_build4<<<grid_1d(I / 4, 256), 256, 0, s>>>(I, O, my_off, my_g, eqc, eqrx, s_out, t_out, s_stride, reps);
    return cudaGetLastError();
}

cudaError_t launch_s_build(uint64_t I, uint64_t O, const uint32_t* my_off, const uint4* my_g, const uint32_t* eqc,
                           const uint32_t* eqrx, uint32_t* s_out, uint64_t s_stride, uint32_t reps, cudaStream_t s) {
    k_s_build<<<grid_1d(I, 256), 256, 0, s>>>(I, O, my_off, my_g, eqc, eqrx, s_out, s_stride, reps);
    return cudaGetLastError();
}

cudaError_t launch_wsum(int reps, const uint32_t* vals, uint64_t rows, const uint32_t* eq, const Geo& g,
                        uint32_t block, uint32_t ctas, RedScratch red, uint32_t* out, cudaStream_t s) {
    LaunchShape sh = row_shape(g, rows, block, ctas, reps);
    switch (reps) {
        case 1: k_wsum<1><<<sh.grid, sh.block, sh.smem, s>>>(vals, rows, eq, g, red, out); break;
        case 2: k_wsum<2><<<sh.grid, sh.block, sh.smem, s>>>(vals, rows, eq, g, red, out); break;
        case 3: k_wsum<3><<<sh.grid, sh.block, sh.smem, s>>>(vals, rows, eq, g, red, out); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace gkrgpu
