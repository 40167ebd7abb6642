// Device kernels of the GKR prove path and their host-side launch wrappers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gkrgpu {

// Thread tile for a table of rows x N lanes stored row-major (row r, lane k at r*N + k).
// Each thread owns 4 consecutive lanes (one 16-byte load); tpr threads cover a slice of
// 4*tpr lanes of one row, rps such slices (rows) share a CTA, and gridDim.y = N/(4*tpr)
// lane groups cover the whole row.
struct Geo {
    uint32_t N;    // lanes (data-parallel circuit copies), multiple of 4
    uint32_t tpr;  // threads per row slice
    uint32_t rps;  // row slices per CTA (blockDim.x / tpr)
};

// Scratch of the reducing kernels: per-(component, lane) 64-bit accumulators and the
// arrival ticket of the last-CTA finisher.  Both are left zeroed by every launch.
struct RedScratch {
    unsigned long long* acc;  // components x N
    unsigned int* ticket;
    // Optional completion counter in host-mapped memory: each lane group's finishing CTA
    // increments it (system scope) after its results are visible to the host.
    unsigned int* done = nullptr;
    // Optional device copy of the published round evaluations (R x 3 x N): the round kernels
    // that take p1 from their claim read the previous round's evaluations here.
    uint32_t* evals_dev = nullptr;
};

struct EqArgs {
    uint32_t r1[3][32];
    uint32_t r2[3][32];
    uint32_t f1, f2;  // factors alpha (table 1) and beta (table 2; 0 = no second table)
    uint32_t nvars;
    uint32_t reps;
};

struct RoundPtrs {
    const uint32_t* fsrc[3];
    uint32_t* fdst[3];
    const uint32_t* hsrc[3];
    uint32_t* hdst[3];
    uint32_t r[3];
    // Phase-one rounds 2 and 3: the stored hg rows of the previous round whose input rows
    // (2 or 4 of them) have no mul gates were not stored; they are the folds of the add
    // weights a_j of those rows at the earlier challenges, from the layer's CSR offsets by
    // input row (hoff), add weights (ha) and the challenges of rounds 0 and 1 (hr[round][j]).
    const uint32_t* hoff;
    const uint4* ha;
    uint32_t hr[2][3];
};

// Persistent tail of a sumcheck phase (k_tail): rounds kt .. n-1 in one launch, one CTA per
// lane group.  Round k folds its source tables at the challenges of round k-1 into its
// destination tables (round k reads B and writes A when k is odd, the other way round when
// k is even), publishes the round's evaluations to evals_out and bumps `done` once per CTA;
// the last round also publishes rows 0..1 of each repetition's folded f table to rows_out.
// The challenges of round k-1 > kt-1 come from the host through the mailbox (host-mapped
// words: [0] abort, [4 + 4k] tag of round k's challenges = tag_base + k, [5 + 4k + j] r_k[j]).
// Each wait is bounded by wait_ns: when it expires the kernel sets *err and returns; a
// nonzero abort word makes it return at once.
constexpr uint32_t kMboxRounds = 40;
constexpr uint32_t kMboxWords = 4 + 4 * kMboxRounds;
struct TailArgs {
    uint32_t *fA[3], *fB[3];  // per-copy f tables
    uint32_t *hA[3], *hB[3];  // per-copy hg tables (phase one) or scalar s tables (phase two)
    const uint32_t* vx;       // phase two: R x N claims the sums are multiplied by; null in phase one
    uint32_t r_first[3];      // challenges of round kt - 1
    uint32_t kt, n, reps;
    uint32_t tag_base;
    const uint32_t* mbox;
    uint32_t* evals_out;      // R x 3 x N
    uint32_t* rows_out;       // R x 2 x N
    unsigned int* done;
    unsigned int* err;
    unsigned long long wait_ns;
    Geo g;
};

struct LaunchShape {
    dim3 grid, block;
    size_t smem;
};

// Kernel identifiers for launch accounting.
enum KernelId {
    K_CHECK = 0,
    K_EVALUATE,
    K_EQ,
    K_WEIGHTS,
    K_HG_ROUND0,
    K_ROUND_LANE,
    K_ROUND_SCALAR,
    K_S_BUILD,
    K_WSUM,
    K_HG_ROUND1,
    K_GATE_SUMS,   // verifier
    K_CANONICAL,   // verifier
    K_P2_ROUND0,
    K_STAGE,  // small transfers between device and host-mapped memory
    K_TAIL,   // a phase's last rounds in one persistent launch (k_tail)
    // BN254 kernels (bn254.cuh)
    K_BN_LOAD,
    K_BN_EVALUATE,
    K_BN_EQ,
    K_BN_WEIGHTS,
    K_BN_HG_ROUND0,
    K_BN_ROUND_LANE,
    K_BN_ROUND_SCALAR,
    K_BN_S_BUILD,
    K_BN_WSUM,
    K_BN_UNLOAD,
    K_NUM_KERNELS
};
extern const char* const kKernelNames[K_NUM_KERNELS];

// Shape of a row-tiled launch over `rows` rows; ctas_cap bounds gridDim.x * gridDim.y.
LaunchShape row_shape(const Geo& g, uint64_t rows, uint32_t block, uint32_t ctas_cap, uint32_t smem_components);

// Launch wrappers (all asynchronous on `s`).
cudaError_t launch_check_canonical(const uint32_t* v, uint64_t n, unsigned int* flag, cudaStream_t s);
// v[i] = v[i] mod p in place (M31::from_bytes of raw proof words).
cudaError_t launch_canonicalize(uint32_t* v, uint64_t n, cudaStream_t s);
// Verifier gate sums for `reps` points: over the mul gates (CSR by output: off, (i0, i1, c, 0)
// gates) sum c eqz_j[o] eqx_j[i0] eqy_j[i1], or over the add gates ((i0, c) gates) sum
// c eqz_j[o] eqx_j[i0]; eq tables are reps x O / reps x I.  acc (3 x u64) and ticket must be
// zero and are left zero; out receives reps canonical totals.
cudaError_t launch_gate_sums(bool mul_gates, uint64_t O, uint64_t I, const uint32_t* off, const uint32_t* gates,
                             const uint32_t* eqz, const uint32_t* eqx, const uint32_t* eqy, uint32_t reps,
                             unsigned long long* acc, unsigned int* ticket, uint32_t* out, cudaStream_t s);
cudaError_t launch_evaluate(const uint32_t* in, uint32_t* out, uint64_t O, const uint32_t* mo_off, const uint4* mo_g,
                            const uint32_t* ao_off, const uint2* ao_g, const Geo& g, uint32_t block, uint32_t ctas,
                            cudaStream_t s);
cudaError_t launch_eq(uint32_t* out, const EqArgs& a, cudaStream_t s);
// dst[k * n + i] = srcs[k][i] (nsrc <= 3 tables of n words) by a small kernel instead of the
// copy engine, for transfers between device and host-mapped memory; with `done`, every CTA
// increments it after its writes are visible to the host.  Returns the CTA count (the
// number of increments); *err receives the launch status.
uint32_t launch_stage_words(uint32_t* dst, const uint32_t* const* srcs, uint32_t nsrc, uint64_t n, unsigned int* done,
                            cudaStream_t s, cudaError_t* err);
// w4r[k].j = w4[k].j (1 - r_j) for the mul gates of even input rows, w4[k].j r_j for odd
// rows (CSR-by-x offsets mx_off over I rows): the weights of launch_hg_round1.
cudaError_t launch_scale_weights(uint64_t I, const uint32_t* mx_off, const uint4* w4, uint4* w4r, const uint32_t r[3],
                                 int reps, cudaStream_t s);
cudaError_t launch_weights(uint64_t I, uint64_t Gm, uint64_t O, const uint32_t* eqc, const uint4* mx_g,
                           const uint32_t* ax_off, const uint2* ax_g, uint4* a_out, uint4* w_out, uint32_t reps,
                           cudaStream_t s);
// Phase-one hg (not stored) and the round-0 evaluations over `npairs` pairs of input rows:
// pair i is (2q, 2q+1) with q = pairs[i], or q = i without a list (pairs = null).  Pairs
// left out of the list must have no gate whose first input is in them (their hg is zero).
// `claim` (R x N, device-readable, required) is the round's claim alpha v(rz1) + beta v(rz2)
// per repetition and copy: the evaluations at 1 are the claim less those at 0.
cudaError_t launch_hg_round0(int reps, const uint32_t* v, uint64_t npairs, const uint32_t* pairs,
                             const uint32_t* mx_off, const uint4* mx_g, const uint4* a4, const uint4* w4, const Geo& g,
                             uint32_t block, uint32_t ctas, RedScratch red, const uint32_t* claim,
                             uint32_t* evals_out, cudaStream_t s);
// Phase-one round 1 rebuilding hg from the gate weights (no stored hg table): outputs
// p.fdst[j] / p.hdst[j] (I/2 rows each; p.fdst[0] null: the folded copies are not stored),
// challenges p.r[j]; npairs output pairs, pair i folding input rows 4q .. 4q+3 with
// q = quads[i] (q = i without a list).  A list, which may leave out only groups of four rows
// with no gate whose first input is in them, needs p.fdst[0] null.  red.evals_dev (required)
// must hold round 0's evaluations: the round's claim is round 0's polynomial at p.r[j], and
// the evaluations at 1 are that claim less those at 0.  w4r: the gate weights scaled at p.r
// (launch_scale_weights).
cudaError_t launch_hg_round1(int reps, const uint32_t* v, uint64_t npairs, const uint32_t* quads,
                             const uint32_t* mx_off, const uint4* mx_g, const uint4* a4, const uint4* w4r,
                             const RoundPtrs& p, const Geo& g, uint32_t block, uint32_t ctas, RedScratch red,
                             uint32_t* evals_out, cudaStream_t s);
// The fold rounds below (launch_round_hr, launch_p1_round2, launch_p2_round2 and
// launch_round with fold) sum p0 and p2raw only: red.evals_dev (required) must hold the
// previous round's evaluations in the same phase, whose polynomial at p.r[j] is the round's
// claim, and the evaluations at 1 are that claim less those at 0.  Every round kernel writes
// its evaluations to red.evals_dev as well as to evals_out when red.evals_dev is given.
// Phase-one round 2 or 3 (k = round, a k_round with per-copy hg and fold) reading the
// previous round's stored hg rows and recomputing the copy-independent ones (p.hoff, p.ha,
// p.hr); round 2 in turn does not store its copy-independent output rows.
cudaError_t launch_round_hr(int round, int reps, const RoundPtrs& p, uint64_t npairs, const Geo& g, uint32_t block,
                            uint32_t ctas, RedScratch red, uint32_t* evals_out, cudaStream_t s);
// Phase-one round 2 refolding the layer input p.fsrc[0] at the round-0 challenges p.hr[0][j]
// and p.r[j], all repetitions per thread (round 1 stored no folded copies); hg rows as
// launch_round_hr(2, ..) (p.hsrc, p.hoff, p.ha); npairs = I/8.
cudaError_t launch_p1_round2(int reps, const RoundPtrs& p, uint64_t npairs, const Geo& g, uint32_t block,
                             uint32_t ctas, RedScratch red, uint32_t* evals_out, cudaStream_t s);
// Phase-two round 2 refolding the layer input p.fsrc[0] at the round-0 challenges p.hr[0]
// (round 1 stored only its scalar tables) and at p.r; outputs p.fdst / p.hdst as k_round.
cudaError_t launch_p2_round2(int reps, const RoundPtrs& p, uint64_t npairs, const uint32_t* vx, const Geo& g,
                             uint32_t block, uint32_t ctas, RedScratch red, uint32_t* evals_out, cudaStream_t s);
cudaError_t launch_round(int reps, bool shared_src, bool lane_hg, bool fold, const RoundPtrs& p, uint64_t npairs,
                         const uint32_t* vx, const Geo& g, uint32_t block, uint32_t ctas, RedScratch red,
                         uint32_t* evals_out, cudaStream_t s);
// Phase-two rounds 0 and 1 in one pass over the layer input v (4 ngroups rows, ngroups >= 2):
// round 0's evaluations (times vx) are published to evals_out as by the round kernels, and
// 9 * reps canonical sums per copy go to sums_out (9 reps x N) for launch_p2_round1_fin.
// s[j] are the scalar tables (16-byte aligned), t[j] their pair sums (launch_s_build4);
// red.acc needs 9 * reps x N accumulators.  Publishes p2_round01_groups(N) lane groups;
// p2_round01_groups(N) is 0 where the kernel does not apply (its row slices of up to 256
// copies must be a multiple of 32 copies).
// Groups i < ngroups are rows 4q .. 4q+3 with q = quads[i] (q = i without a list); a list
// may leave out only groups with no mul gate whose second input is in them (s_j zero there).
cudaError_t launch_p2_round01(int reps, const uint32_t* v, const uint32_t* const* s, const uint32_t* const* t,
                              uint64_t ngroups, const uint32_t* quads, const uint32_t* vx, uint32_t N, uint32_t ctas,
                              RedScratch red, uint32_t* evals_out, uint32_t* sums_out, cudaStream_t st);
uint32_t p2_round01_groups(uint32_t N);
// Phase-two round 1 from those sums at the round-0 challenges r[j]: evaluations to evals_out
// and evals_dev (when given; one completion count on done), and the scalar tables s[j]
// folded into sd[j] (2 ngroups entries each) for round 2.
cudaError_t launch_p2_round1_fin(int reps, const uint32_t* sums, const uint32_t* vx, const uint32_t* const* s,
                                 uint32_t* const* sd, const uint32_t* r, uint64_t ngroups, uint32_t N,
                                 uint32_t* evals_out, uint32_t* evals_dev, unsigned int* done, cudaStream_t st);
// launch_s_build plus the pair sums t_j(i) = (s_j(4i) + s_j(4i+2), s_j(4i+1) + s_j(4i+3),
// s_j(4i) + s_j(4i+1), s_j(4i+2) + s_j(4i+3)) into t_out (4 I/4 entries, stride s_stride);
// I and s_stride multiples of 4.
cudaError_t launch_s_build4(uint64_t I, uint64_t O, const uint32_t* my_off, const uint4* my_g, const uint32_t* eqc,
                            const uint32_t* eqrx, uint32_t* s_out, uint32_t* t_out, uint64_t s_stride, uint32_t reps,
                            cudaStream_t s);
cudaError_t launch_s_build(uint64_t I, uint64_t O, const uint32_t* my_off, const uint4* my_g, const uint32_t* eqc,
                           const uint32_t* eqrx, uint32_t* s_out, uint64_t s_stride, uint32_t reps, cudaStream_t s);
// Rows of a tail round's source tables above which a phase keeps its per-round kernels
// (the tail's CTA reads all its rows alone), and the tile of the tail kernel.
uint32_t tail_max_rows(uint32_t N, int reps, bool lane_hg);
Geo tail_geo(uint32_t N);
cudaError_t launch_tail(bool lane_hg, const TailArgs& a, cudaStream_t s);
cudaError_t launch_wsum(int reps, const uint32_t* vals, uint64_t rows, const uint32_t* eq, const Geo& g,
                        uint32_t block, uint32_t ctas, RedScratch red, uint32_t* out, cudaStream_t s);

}  // namespace gkrgpu
