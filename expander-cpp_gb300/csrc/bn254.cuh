// BN254 scalar field kernels of the GKR prove path (Config::field_type = BN254, R = 1).
//
// Element encoding (the reference declares BN254 but ships no implementation, so this is
// the project's definition): a canonical integer in [0, r) serialised as 32 little-endian
// bytes; a 32-byte string (e.g. a SHA-256 digest) is read little-endian and reduced mod r.
// On the device every table holds Montgomery forms (x * 2^256 mod r) as 8 little-endian
// 32-bit limbs; conversion happens when the input is loaded and when results leave.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.cuh"

namespace gkrgpu {
namespace bn {

struct Fr {
    uint32_t l[8];
};

// Threads per CTA of every row-tiled BN254 kernel.
constexpr uint32_t kBlock = 256;

// Row tile: one thread per element (lane) of a row; tpr threads per row slice.
struct GeoBn {
    uint32_t N, tpr, rps;
};

// Reduction scratch: per (component, lane, limb) 64-bit limb sums, one ticket per lane
// group, optional completion counter in host-mapped memory (see RedScratch).
struct RedBn {
    unsigned long long* acc;  // comps x N x 8
    unsigned int* ticket;
    unsigned int* done = nullptr;
    // Device copies of the published round evaluations (3 x N x 8 words each, canonical):
    // the round kernels write theirs to evals_dev, and a round that takes p1 from its claim
    // reads the previous round's from evals_prev (a different buffer).
    const uint32_t* evals_prev = nullptr;
    uint32_t* evals_dev = nullptr;
};

struct EqArgsBn {
    uint32_t r1[32][8];
    uint32_t r2[32][8];
    uint32_t f1[8], f2[8];
    uint32_t nvars, has_r2;
};

struct RoundPtrsBn {
    const uint32_t* fsrc;
    uint32_t* fdst;
    const uint32_t* hsrc;  // per-lane hg table (phase one) or scalar s table (phase two)
    uint32_t* hdst;
    uint32_t r[8];  // challenge of the previous round, Montgomery form
};

// Input -> Montgomery table; with bad a non-canonical element raises *bad, without it every
// element is reduced mod r first (the verifier's from_bytes).
cudaError_t launch_load(const uint32_t* canon, uint32_t* mont, uint64_t n_elems, unsigned int* bad, cudaStream_t s);
// Verifier gate sums of one layer (one repetition): mul or add gates of the evaluate CSR with
// their Montgomery coefficients; acc (8 x u64) and ticket zero before and after; out receives
// the canonical total (8 words).
cudaError_t launch_gate_sums(bool mul_gates, uint64_t O, const uint32_t* off, const uint32_t* gates, const Fr* coef,
                             const Fr* eqz, const Fr* eqx, const Fr* eqy, unsigned long long* acc,
                             unsigned int* ticket, uint32_t* out, cudaStream_t s);
cudaError_t launch_unload(uint32_t* v, uint64_t n_elems, cudaStream_t s);
cudaError_t launch_evaluate(const uint32_t* in, uint32_t* out, uint64_t O, const uint32_t* mo_off, const uint4* mo_g,
                            const Fr* mo_c, const uint32_t* ao_off, const uint2* ao_g, const Fr* ao_c, const GeoBn& g,
                            uint32_t ctas, cudaStream_t s);
cudaError_t launch_eq(Fr* out, const EqArgsBn& a, cudaStream_t s);
cudaError_t launch_weights(uint64_t I, uint64_t Gm, const Fr* eqc, const uint4* mx_g, const Fr* mx_c,
                           const uint32_t* ax_off, const uint2* ax_g, const Fr* ax_c, Fr* a_out, Fr* w_out,
                           cudaStream_t s);
// Phase-one hg table and round 0: `claim` (N x 8 words, canonical, device-readable,
// required) is alpha v(rz1) + beta v(rz2) per copy; the evaluations at 1 are the claim less
// those at 0.
cudaError_t launch_hg_round0(const uint32_t* v, uint64_t I, const uint32_t* mx_off, const uint4* mx_g, const Fr* a,
                             const Fr* w, uint32_t* hg, const GeoBn& g, uint32_t ctas, RedBn red, const uint32_t* claim,
                             uint32_t* evals_out, cudaStream_t s);
// A sumcheck round.  With fold (every round after a phase's first) the round's claim is the
// previous round's polynomial at p.r, from red.evals_prev (required), and the evaluations at
// 1 are that claim less those at 0; phase two's round 0 (no fold) sums all three.
cudaError_t launch_round(bool lane_hg, bool fold, const RoundPtrsBn& p, uint64_t npairs, const uint32_t* vx,
                         const GeoBn& g, uint32_t ctas, RedBn red, uint32_t* evals_out, cudaStream_t s);
cudaError_t launch_s_build(uint64_t I, const uint32_t* my_off, const uint4* my_g, const Fr* my_c, const Fr* eqc,
                           const Fr* eqrx, Fr* s_out, cudaStream_t s);
cudaError_t launch_wsum(const uint32_t* vals, uint64_t rows, const Fr* eq, const GeoBn& g, uint32_t ctas, RedBn red,
                        uint32_t* out, cudaStream_t s);

}  // namespace bn
}  // namespace gkrgpu
