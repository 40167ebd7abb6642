/* Test infrastructure only: CPU oracle for the GKR prove path (see gkr_oracle.h).
 *
 * Every function restates one piece of the reference (PolyhedraZK/Expander-cpp) and
 * cites it.  The loops follow the reference's order and its gate_exists bookkeeping so
 * that a reader can check them line by line; the field is exact, so the bytes do not
 * depend on summation order anyway.  Parity of this file with the reference is pinned
 * by tests/test_oracle.py (against oracle/_ref) and tests/golden/golden.json.
 */
#include "gkr_oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define P 2147483647u

/* ---------------------------------------------------------------- M31 field
 * include/field/M31.hpp:64-93 (scalar) and include/field/M31_avx.tcc:97-176 (packed);
 * both return canonical values in [0, p) for canonical inputs. */
/* Branch-free forms (a conditional subtraction as a minimum of two candidates) so that gcc
 * vectorises the per-lane loops with portable flags; the values are the same.  The hot lane
 * loops carry `ivdep`: lane k of a row depends only on lane k of its sources (an in-place
 * fold reads and writes the same lane), so gcc may skip its run-time overlap checks. */
static inline uint32_t m_umin(uint32_t a, uint32_t b) { return a < b ? a : b; }
/* a + b < 2^32: r - p wraps above r exactly when r < p */
static inline uint32_t m_add(uint32_t a, uint32_t b) { uint32_t r = a + b; return m_umin(r, r - P); }
/* a - b wraps above p exactly when a < b, and then d + p (mod 2^32) is the result */
static inline uint32_t m_sub(uint32_t a, uint32_t b) { uint32_t d = a - b; return m_umin(d, d + P); }
/* a b < 2^62: (x & p) + (x >> 31) < 2p for canonical inputs, then one subtraction */
static inline uint32_t m_mul(uint32_t a, uint32_t b) {
    uint64_t x = (uint64_t)a * b;
    uint32_t s = ((uint32_t)x & P) + (uint32_t)(x >> 31);
    return m_umin(s, s - P);
}
/* M31::from_bytes / PackedM31::from_bytes: M31.hpp:111-116, M31_avx.tcc:62-67 */
static inline uint32_t m_reduce(uint32_t x) { x = (x & P) + (x >> 31); return m_umin(x, x - P); }

/* ---------------------------------------------------------------- SHA-256 (FIPS 180-4)
 * The reference hashes with Bitcoin Core's CSHA256 (lib/btc_sha256/crypto/sha256.cpp),
 * i.e. standard SHA-256; this is an independent plain implementation of the standard. */
static const uint32_t K256[64] = {
    0x428a2f98, 0x71374491, 0xb5c0fbcf, 0xe9b5dba5, 0x3956c25b, 0x59f111f1, 0x923f82a4, 0xab1c5ed5,
    0xd807aa98, 0x12835b01, 0x243185be, 0x550c7dc3, 0x72be5d74, 0x80deb1fe, 0x9bdc06a7, 0xc19bf174,
    0xe49b69c1, 0xefbe4786, 0x0fc19dc6, 0x240ca1cc, 0x2de92c6f, 0x4a7484aa, 0x5cb0a9dc, 0x76f988da,
    0x983e5152, 0xa831c66d, 0xb00327c8, 0xbf597fc7, 0xc6e00bf3, 0xd5a79147, 0x06ca6351, 0x14292967,
    0x27b70a85, 0x2e1b2138, 0x4d2c6dfc, 0x53380d13, 0x650a7354, 0x766a0abb, 0x81c2c92e, 0x92722c85,
    0xa2bfe8a1, 0xa81a664b, 0xc24b8b70, 0xc76c51a3, 0xd192e819, 0xd6990624, 0xf40e3585, 0x106aa070,
    0x19a4c116, 0x1e376c08, 0x2748774c, 0x34b0bcb5, 0x391c0cb3, 0x4ed8aa4a, 0x5b9cca4f, 0x682e6ff3,
    0x748f82ee, 0x78a5636f, 0x84c87814, 0x8cc70208, 0x90befffa, 0xa4506ceb, 0xbef9a3f7, 0xc67178f2};

#define ROR(x, n) (((x) >> (n)) | ((x) << (32 - (n))))

static void sha_block(uint32_t st[8], const uint8_t* p) {
    uint32_t w[64];
    for (int i = 0; i < 16; i++)
        w[i] = ((uint32_t)p[4 * i] << 24) | ((uint32_t)p[4 * i + 1] << 16) | ((uint32_t)p[4 * i + 2] << 8) | p[4 * i + 3];
    for (int i = 16; i < 64; i++) {
        uint32_t s0 = ROR(w[i - 15], 7) ^ ROR(w[i - 15], 18) ^ (w[i - 15] >> 3);
        uint32_t s1 = ROR(w[i - 2], 17) ^ ROR(w[i - 2], 19) ^ (w[i - 2] >> 10);
        w[i] = w[i - 16] + s0 + w[i - 7] + s1;
    }
    uint32_t a = st[0], b = st[1], c = st[2], d = st[3], e = st[4], f = st[5], g = st[6], h = st[7];
    for (int i = 0; i < 64; i++) {
        uint32_t t1 = h + (ROR(e, 6) ^ ROR(e, 11) ^ ROR(e, 25)) + ((e & f) ^ (~e & g)) + K256[i] + w[i];
        uint32_t t2 = (ROR(a, 2) ^ ROR(a, 13) ^ ROR(a, 22)) + ((a & b) ^ (a & c) ^ (b & c));
        h = g; g = f; f = e; e = d + t1; d = c; c = b; b = a; a = t1 + t2;
    }
    st[0] += a; st[1] += b; st[2] += c; st[3] += d; st[4] += e; st[5] += f; st[6] += g; st[7] += h;
}

void oracle_sha256(const uint8_t* in, uint64_t len, uint8_t out[32]) {
    uint32_t st[8] = {0x6a09e667, 0xbb67ae85, 0x3c6ef372, 0xa54ff53a, 0x510e527f, 0x9b05688c, 0x1f83d9ab, 0x5be0cd19};
    uint64_t full = len / 64;
    for (uint64_t b = 0; b < full; b++) sha_block(st, in + 64 * b);
    uint8_t tail[128];
    uint64_t rem = len - 64 * full;
    memset(tail, 0, sizeof(tail));
    if (rem) memcpy(tail, in + 64 * full, rem);
    tail[rem] = 0x80;
    uint64_t tl = (rem + 9 <= 64) ? 64 : 128;
    uint64_t bits = len * 8;
    for (int i = 0; i < 8; i++) tail[tl - 1 - i] = (uint8_t)(bits >> (8 * i));
    sha_block(st, tail);
    if (tl == 128) sha_block(st, tail + 64);
    for (int i = 0; i < 8; i++) {
        out[4 * i] = (uint8_t)(st[i] >> 24); out[4 * i + 1] = (uint8_t)(st[i] >> 16);
        out[4 * i + 2] = (uint8_t)(st[i] >> 8); out[4 * i + 3] = (uint8_t)st[i];
    }
}

/* ---------------------------------------------------------------- transcript
 * include/fiat_shamir/transcript.hpp:87-175.  A challenge hashes the bytes appended since
 * the previous challenge, or the previous digest when nothing was appended (:91-103); the
 * digest starts as 32 zero bytes (:118-125). */
typedef struct {
    uint8_t* bytes;
    uint64_t len, cap, hash_start;
    uint8_t digest[32];
    int overflow;
} transcript;

static void tr_init(transcript* t, uint8_t* buf, uint64_t cap) {
    t->bytes = buf; t->len = 0; t->cap = cap; t->hash_start = 0; t->overflow = 0;
    memset(t->digest, 0, 32);
}
static void tr_append(transcript* t, const void* p, uint64_t n) {
    if (t->len + n > t->cap) { t->overflow = 1; t->len += n; return; }
    memcpy(t->bytes + t->len, p, n);
    t->len += n;
}
static void tr_hash_to_digest(transcript* t) {
    if (t->len > t->hash_start) {
        oracle_fs_hash(t->bytes + t->hash_start, t->len - t->hash_start, t->digest);
        t->hash_start = t->len;
    } else {
        oracle_fs_hash(t->digest, 32, t->digest);
    }
}
/* Transcript::challenge_f, :139-147: M31::from_bytes of the digest's first 4 bytes. */
static uint32_t tr_challenge(transcript* t) {
    tr_hash_to_digest(t);
    uint32_t x;
    memcpy(&x, t->digest, 4);
    return m_reduce(x);
}

/* grind, include/LinearGKR/LinearGKR.hpp:13-32: challenge_fs(256/31 = 8) laid out at
 * 4-byte offsets, 2^grinding_bits in-place SHA-256 rounds, then appended. */
static void grind(transcript* t, int grinding_bits) {
    uint8_t h[32];
    memset(h, 0, 32);
    for (int i = 0; i < 256 / 31; i++) {
        uint32_t c = tr_challenge(t);
        memcpy(h + 4 * i, &c, 4);
    }
    for (long i = 0; i < (1L << grinding_bits); i++) oracle_fs_hash(h, 32, h);
    tr_append(t, h, 32);
}

int oracle_num_repetitions(int grinding_bits) {
    /* include/configuration/config.hpp:61-65 with security_bits = 100, field_size = 31 */
    int s = 100 - grinding_bits;
    return s / 31 + (s % 31 != 0);
}

/* ---------------------------------------------------------------- eq tables
 * include/LinearGKR/sumcheck_common.hpp:9-53.  _eq(x, y) = 2xy - x - y + 1. */
static inline uint32_t eq_(uint32_t x, uint32_t y) {
    return m_add(m_sub(m_sub(m_mul(m_mul(x, y), 2), x), y), 1);
}
static void eq_evals_primitive(const uint32_t* r, uint32_t nr, uint32_t factor, uint32_t* out) {
    out[0] = factor;
    uint64_t cur = 1;
    for (uint32_t i = 0; i < nr; i++) {
        uint32_t e0 = eq_(r[i], 0), e1 = eq_(r[i], 1);
        for (uint64_t j = 0; j < cur; j++) {
            out[j + cur] = m_mul(out[j], e1);
            out[j] = m_mul(out[j], e0);
        }
        cur <<= 1;
    }
}
static void eq_evals_at(const uint32_t* r, uint32_t nr, uint32_t factor, uint32_t* out, uint32_t* first, uint32_t* second) {
    uint32_t fh = nr / 2;
    uint64_t mask = (1ull << fh) - 1;
    eq_evals_primitive(r, fh, factor, first);
    eq_evals_primitive(r + fh, nr - fh, 1, second);
    for (uint64_t i = 0; i < (1ull << nr); i++) out[i] = m_mul(first[i & mask], second[i >> fh]);
}

/* ---------------------------------------------------------------- circuit
 * Circuit::evaluate / CircuitLayer::evaluate, include/circuit/circuit.hpp:92-105,273-280. */
static int check_layers(const oracle_layer* L, int nl, uint32_t N) {
    if (nl <= 0 || N == 0) return -1;
    for (int l = 0; l < nl; l++) {
        if (L[l].nb_input_vars > 30 || L[l].nb_output_vars > 30) return -1;
        if (l + 1 < nl && L[l].nb_output_vars != L[l + 1].nb_input_vars) return -1;
        uint64_t I = 1ull << L[l].nb_input_vars, O = 1ull << L[l].nb_output_vars;
        for (uint64_t g = 0; g < L[l].n_mul; g++) {
            const uint32_t* s = L[l].mul + 4 * g;
            if (s[0] >= O || s[1] >= I || s[2] >= I || s[3] >= P) return -1;
        }
        for (uint64_t g = 0; g < L[l].n_add; g++) {
            const uint32_t* s = L[l].add + 3 * g;
            if (s[0] >= O || s[1] >= I || s[2] >= P) return -1;
        }
    }
    return 0;
}

static void layer_eval(const oracle_layer* L, uint32_t N, const uint32_t* in, uint32_t* out) {
    uint64_t O = 1ull << L->nb_output_vars;
    memset(out, 0, O * N * 4);
    for (uint64_t g = 0; g < L->n_mul; g++) {
        const uint32_t* s = L->mul + 4 * g;
        uint32_t* o = out + (uint64_t)s[0] * N;
        const uint32_t *a = in + (uint64_t)s[1] * N, *b = in + (uint64_t)s[2] * N;
        #pragma GCC ivdep
        for (uint32_t k = 0; k < N; k++) o[k] = m_add(o[k], m_mul(m_mul(a[k], b[k]), s[3]));
    }
    for (uint64_t g = 0; g < L->n_add; g++) {
        const uint32_t* s = L->add + 3 * g;
        uint32_t* o = out + (uint64_t)s[0] * N;
        const uint32_t* a = in + (uint64_t)s[1] * N;
        #pragma GCC ivdep
        for (uint32_t k = 0; k < N; k++) o[k] = m_add(o[k], m_mul(a[k], s[2]));
    }
}

static uint64_t values_rows(const oracle_layer* L, int nl) {
    uint64_t rows = 0;
    for (int l = 0; l < nl; l++) rows += 1ull << L[l].nb_input_vars;
    return rows + (1ull << L[nl - 1].nb_output_vars);
}

/* Fills vals[l] (input of layer l) and vals[nl] (output of the last layer). */
static void eval_all(const oracle_layer* L, int nl, uint32_t N, const uint32_t* input, uint32_t* buf, uint32_t** vals) {
    uint64_t off = 0;
    for (int l = 0; l <= nl; l++) {
        vals[l] = buf + off;
        off += (l < nl ? (1ull << L[l].nb_input_vars) : (1ull << L[nl - 1].nb_output_vars)) * N;
    }
    uint64_t I0 = 1ull << L[0].nb_input_vars;
    for (uint64_t i = 0; i < I0 * N; i++) vals[0][i] = m_reduce(input[i]);
    for (int l = 0; l < nl; l++) layer_eval(&L[l], N, vals[l], vals[l + 1]);
}

int oracle_evaluate(const oracle_layer* layers, int nlayers, uint32_t N, const uint32_t* input, uint32_t* out) {
    if (check_layers(layers, nlayers, N)) return -1;
    uint32_t** vals = (uint32_t**)malloc(sizeof(uint32_t*) * (nlayers + 1));
    eval_all(layers, nlayers, N, input, out, vals);
    free(vals);
    return 0;
}

/* eval_multilinear, include/poly_commit/poly.hpp:88-104 */
void oracle_eval_multilinear(const uint32_t* evals, uint32_t nb_vars, uint32_t N, const uint32_t* r, uint32_t* out) {
    uint64_t n = 1ull << nb_vars;
    uint32_t* s = (uint32_t*)malloc(n * N * 4);
    memcpy(s, evals, n * N * 4);
    uint64_t cur = n >> 1;
    for (uint32_t v = 0; v < nb_vars; v++) {
        for (uint64_t i = 0; i < cur; i++) {
            uint32_t *d = s + i * N, *a = s + 2 * i * N, *b = s + (2 * i + 1) * N;
            #pragma GCC ivdep
            for (uint32_t k = 0; k < N; k++) d[k] = m_add(a[k], m_mul(m_sub(b[k], a[k]), r[v]));
        }
        cur >>= 1;
    }
    memcpy(out, s, N * 4);
    free(s);
}

/* ---------------------------------------------------------------- sumcheck prover
 * GKRScratchPad (include/LinearGKR/scratch_pad.hpp:8-65): one per repetition. */
typedef struct {
    uint32_t *v_evals, *hg_evals, *eq_rx, *eq_rz1, *eq_rz2, *eq_first, *eq_second;
    uint8_t* gate_exists;
} scratch_pad;

static int pad_alloc(scratch_pad* p, uint32_t max_in_vars, uint32_t max_out_vars, uint32_t N) {
    uint64_t I = 1ull << max_in_vars, O = 1ull << max_out_vars;
    uint64_t half = 1ull << ((max_in_vars > max_out_vars ? max_in_vars : max_out_vars) / 2 + 1);
    p->v_evals = (uint32_t*)malloc(I * N * 4);
    p->hg_evals = (uint32_t*)malloc(I * N * 4);
    p->eq_rx = (uint32_t*)malloc(I * 4);
    p->eq_rz1 = (uint32_t*)malloc(O * 4);
    p->eq_rz2 = (uint32_t*)malloc(O * 4);
    p->eq_first = (uint32_t*)malloc(half * 4);
    p->eq_second = (uint32_t*)malloc(half * 4);
    p->gate_exists = (uint8_t*)malloc(I);
    return (p->v_evals && p->hg_evals && p->eq_rx && p->eq_rz1 && p->eq_rz2 && p->eq_first && p->eq_second && p->gate_exists) ? 0 : -1;
}
static void pad_free(scratch_pad* p) {
    free(p->v_evals); free(p->hg_evals); free(p->eq_rx); free(p->eq_rz1); free(p->eq_rz2);
    free(p->eq_first); free(p->eq_second); free(p->gate_exists);
}

/* SumcheckMultiLinearProdHelper, include/LinearGKR/sumcheck_helper.hpp:47-135 */
typedef struct {
    uint32_t nb_vars, var_idx;
    uint64_t cur_eval_size;
    uint32_t *bk_f, *bk_hg;
    const uint32_t* initial_v;
} prod_helper;

static void ph_prepare(prod_helper* h, uint32_t nb_vars, uint32_t* f, uint32_t* hg, const uint32_t* v) {
    h->nb_vars = nb_vars; h->var_idx = 0; h->cur_eval_size = 1ull << nb_vars;
    h->bk_f = f; h->bk_hg = hg; h->initial_v = v;
}

/* poly_eval_at, :68-102: evaluations at 0, 1, 2 of the round polynomial. */
static void ph_poly_eval_at(const prod_helper* h, uint32_t var_idx, const uint8_t* gate_exists, uint32_t N, uint32_t* out) {
    uint32_t *p0 = out, *p1 = out + N, *p2 = out + 2 * N;
    memset(out, 0, 3 * N * 4);
    const uint32_t* src = var_idx == 0 ? h->initial_v : h->bk_f;
    uint64_t n = 1ull << (h->nb_vars - var_idx - 1);
    for (uint64_t i = 0; i < n; i++) {
        if (!gate_exists[2 * i] && !gate_exists[2 * i + 1]) continue;
        const uint32_t *f0 = src + 2 * i * N, *f1 = f0 + N, *g0 = h->bk_hg + 2 * i * N, *g1 = g0 + N;
        #pragma GCC ivdep
        for (uint32_t k = 0; k < N; k++) {
            p0[k] = m_add(p0[k], m_mul(f0[k], g0[k]));
            p1[k] = m_add(p1[k], m_mul(f1[k], g1[k]));
            p2[k] = m_add(p2[k], m_mul(m_add(f0[k], f1[k]), m_add(g0[k], g1[k])));
        }
    }
    for (uint32_t k = 0; k < N; k++)
        p2[k] = m_sub(m_add(m_mul(p1[k], 6), m_mul(p0[k], 3)), m_mul(p2[k], 2));
}

/* receive_challenge, :104-133: in-place fold of f and hg at r. */
static void ph_receive_challenge(prod_helper* h, uint32_t r, uint8_t* gate_exists, uint32_t N) {
    const uint32_t* src = h->var_idx == 0 ? h->initial_v : h->bk_f;
    for (uint64_t i = 0; i < (h->cur_eval_size >> 1); i++) {
        uint32_t* f = h->bk_f + i * N;
        const uint32_t *a = src + 2 * i * N, *b = a + N;
        uint32_t* g = h->bk_hg + i * N;
        const uint32_t *ga = h->bk_hg + 2 * i * N, *gb = ga + N;
        if (!gate_exists[2 * i] && !gate_exists[2 * i + 1]) {
            gate_exists[i] = 0;
            #pragma GCC ivdep
            for (uint32_t k = 0; k < N; k++) f[k] = m_add(a[k], m_mul(m_sub(b[k], a[k]), r));
            memset(g, 0, N * 4);
        } else {
            gate_exists[i] = 1;
            #pragma GCC ivdep
            for (uint32_t k = 0; k < N; k++) {
                f[k] = m_add(a[k], m_mul(m_sub(b[k], a[k]), r));
                g[k] = m_add(ga[k], m_mul(m_sub(gb[k], ga[k]), r));
            }
        }
    }
    h->cur_eval_size >>= 1;
    h->var_idx++;
}

/* SumcheckGKRHelper, :150-342 */
typedef struct {
    const uint32_t *rz1, *rz2;
    uint32_t alpha, beta;
    const oracle_layer* layer;
    const uint32_t* layer_input;
    scratch_pad* pad;
    uint32_t rx[32], ry[32];
    uint32_t nrx, nry;
    prod_helper xh, yh;
    uint32_t nb_in, nb_out, N;
} gkr_helper;

/* _prepare_g_x_vals, :172-231 */
static void prepare_g_x(gkr_helper* h) {
    scratch_pad* pad = h->pad;
    uint32_t N = h->N;
    uint64_t I = 1ull << h->nb_in, O = 1ull << h->nb_out;
    memset(pad->hg_evals, 0, I * N * 4);
    memset(pad->gate_exists, 0, I);
    eq_evals_at(h->rz1, h->nb_out, h->alpha, pad->eq_rz1, pad->eq_first, pad->eq_second);
    eq_evals_at(h->rz2, h->nb_out, h->beta, pad->eq_rz2, pad->eq_first, pad->eq_second);
    for (uint64_t i = 0; i < O; i++) pad->eq_rz1[i] = m_add(pad->eq_rz1[i], pad->eq_rz2[i]);
    const oracle_layer* L = h->layer;
    for (uint64_t g = 0; g < L->n_mul; g++) {
        const uint32_t* s = L->mul + 4 * g;
        uint32_t x = s[1], y = s[2], z = s[0];
        uint32_t w = m_mul(s[3], pad->eq_rz1[z]);
        uint32_t* hg = pad->hg_evals + (uint64_t)x * N;
        const uint32_t* vy = h->layer_input + (uint64_t)y * N;
        #pragma GCC ivdep
        for (uint32_t k = 0; k < N; k++) hg[k] = m_add(hg[k], m_mul(vy[k], w));
        pad->gate_exists[x] = 1;
    }
    for (uint64_t g = 0; g < L->n_add; g++) {
        const uint32_t* s = L->add + 3 * g;
        uint32_t x = s[1], z = s[0];
        uint32_t w = m_mul(s[2], pad->eq_rz1[z]);
        uint32_t* hg = pad->hg_evals + (uint64_t)x * N;
        #pragma GCC ivdep
        for (uint32_t k = 0; k < N; k++) hg[k] = m_add(hg[k], w);
        pad->gate_exists[x] = 1;
    }
}

/* _prepare_h_y_vals, :233-261, with v_rx = vx_claim */
static void prepare_h_y(gkr_helper* h, const uint32_t* v_rx) {
    scratch_pad* pad = h->pad;
    uint32_t N = h->N;
    uint64_t I = 1ull << h->nb_in;
    memset(pad->hg_evals, 0, I * N * 4);
    memset(pad->gate_exists, 0, I);
    eq_evals_at(h->rx, h->nrx, 1, pad->eq_rx, pad->eq_first, pad->eq_second);
    const oracle_layer* L = h->layer;
    for (uint64_t g = 0; g < L->n_mul; g++) {
        const uint32_t* s = L->mul + 4 * g;
        uint32_t x = s[1], y = s[2], z = s[0];
        uint32_t w = m_mul(m_mul(pad->eq_rz1[z], pad->eq_rx[x]), s[3]);
        uint32_t* hg = pad->hg_evals + (uint64_t)y * N;
        #pragma GCC ivdep
        for (uint32_t k = 0; k < N; k++) hg[k] = m_add(hg[k], m_mul(v_rx[k], w));
        pad->gate_exists[y] = 1;
    }
}

static void gh_prepare(gkr_helper* h, const oracle_layer* L, const uint32_t* layer_input, const uint32_t* rz1,
                       const uint32_t* rz2, uint32_t alpha, uint32_t beta, scratch_pad* pad, uint32_t N) {
    h->nb_in = L->nb_input_vars; h->nb_out = L->nb_output_vars; h->N = N;
    h->rz1 = rz1; h->rz2 = rz2; h->alpha = alpha; h->beta = beta;
    h->layer = L; h->layer_input = layer_input; h->pad = pad; h->nrx = h->nry = 0;
    prepare_g_x(h);
    ph_prepare(&h->xh, h->nb_in, pad->v_evals, pad->hg_evals, layer_input);
}

/* poly_evals_at, :302-317 (phase two is prepared lazily at var_idx == nb_input_vars) */
static void gh_poly_evals_at(gkr_helper* h, uint32_t var_idx, uint32_t* out) {
    if (var_idx < h->nb_in) {
        ph_poly_eval_at(&h->xh, var_idx, h->pad->gate_exists, h->N, out);
    } else {
        if (var_idx == h->nb_in) {
            /* _prepare_phase_two, :263-272: vx_claim() is v_evals[0] */
            uint32_t* vx = (uint32_t*)malloc(h->N * 4);
            memcpy(vx, h->pad->v_evals, h->N * 4);
            prepare_h_y(h, vx);
            free(vx);
            ph_prepare(&h->yh, h->nb_in, h->pad->v_evals, h->pad->hg_evals, h->layer_input);
        }
        ph_poly_eval_at(&h->yh, var_idx - h->nb_in, h->pad->gate_exists, h->N, out);
    }
}

static void gh_receive_challenge(gkr_helper* h, uint32_t var_idx, uint32_t r) {
    if (var_idx < h->nb_in) {
        ph_receive_challenge(&h->xh, r, h->pad->gate_exists, h->N);
        h->rx[h->nrx++] = r;
    } else {
        ph_receive_challenge(&h->yh, r, h->pad->gate_exists, h->N);
        h->ry[h->nry++] = r;
    }
}

/* sumcheck_prove_gkr_layer, include/LinearGKR/sumcheck.hpp:52-111 */
static void sumcheck_prove_layer(const oracle_layer* L, const uint32_t* layer_input, uint32_t (*rz1)[32],
                                 uint32_t (*rz2)[32], uint32_t alpha, uint32_t beta, transcript* t, scratch_pad* pads,
                                 int R, uint32_t N, gkr_helper* helpers, uint32_t* evals_buf) {
    for (int j = 0; j < R; j++) gh_prepare(&helpers[j], L, layer_input, rz1[j], rz2[j], alpha, beta, &pads[j], N);
    uint32_t n = L->nb_input_vars;
    for (uint32_t i_var = 0; i_var < 2 * n; i_var++) {
        for (int j = 0; j < R; j++) {
            gh_poly_evals_at(&helpers[j], i_var, evals_buf);
            tr_append(t, evals_buf, 3ull * N * 4);
            uint32_t r = tr_challenge(t);
            gh_receive_challenge(&helpers[j], i_var, r);
            if (i_var == n - 1) tr_append(t, pads[j].v_evals, (uint64_t)N * 4); /* vx_claim */
        }
    }
    for (int j = 0; j < R; j++) tr_append(t, pads[j].v_evals, (uint64_t)N * 4); /* vy_claim */
}

uint64_t oracle_proof_size(const oracle_layer* L, int nl, uint32_t N, int R) {
    uint64_t rows = 0;
    for (int l = 0; l < nl; l++) rows += (uint64_t)R * (6ull * L[l].nb_input_vars + 2);
    return (1ull << L[0].nb_input_vars) * N * 4 + 32 + rows * N * 4;
}

/* Prover::prove, include/LinearGKR/LinearGKR.hpp:58-90, and gkr_prove, include/LinearGKR/gkr.hpp:24-73 */
int oracle_prove(const oracle_layer* L, int nl, uint32_t N, const uint32_t* input, int grinding_bits,
                 uint8_t* proof_out, uint64_t proof_cap, uint64_t* proof_len, uint32_t* claimed_v) {
    if (check_layers(L, nl, N)) return -1;
    for (int l = 0; l < nl; l++) if (L[l].nb_input_vars == 0) return -1;
    int R = oracle_num_repetitions(grinding_bits);
    if (R > 8) return -1;
    uint64_t need = oracle_proof_size(L, nl, N, R);
    *proof_len = need;
    if (need > proof_cap) return 2;

    uint32_t** vals = (uint32_t**)malloc(sizeof(uint32_t*) * (nl + 1));
    uint32_t* vbuf = (uint32_t*)malloc(values_rows(L, nl) * N * 4);
    eval_all(L, nl, N, input, vbuf, vals);

    uint32_t max_in = 0, max_out = 0;
    for (int l = 0; l < nl; l++) {
        if (L[l].nb_input_vars > max_in) max_in = L[l].nb_input_vars;
        if (L[l].nb_output_vars > max_out) max_out = L[l].nb_output_vars;
    }
    scratch_pad* pads = (scratch_pad*)calloc(R, sizeof(scratch_pad));
    gkr_helper* helpers = (gkr_helper*)calloc(R, sizeof(gkr_helper));
    for (int j = 0; j < R; j++) pad_alloc(&pads[j], max_in, max_out, N);
    uint32_t* evals_buf = (uint32_t*)malloc(3ull * N * 4);

    transcript t;
    tr_init(&t, proof_out, proof_cap);
    /* RawPC::commit + RawCommitment::to_bytes: the input layer verbatim (raw.hpp:19-27,61-71) */
    tr_append(&t, vals[0], (1ull << L[0].nb_input_vars) * N * 4);
    grind(&t, grinding_bits);

    /* gkr_prove */
    uint32_t rz1[8][32], rz2[8][32];
    uint32_t nz = L[nl - 1].nb_output_vars;
    for (uint32_t i = 0; i < nz; i++)
        for (int j = 0; j < R; j++) { rz1[j][i] = tr_challenge(&t); rz2[j][i] = 0; }
    uint32_t alpha = 1, beta = 0;
    for (int j = 0; j < R; j++) oracle_eval_multilinear(vals[nl], nz, N, rz1[j], claimed_v + (uint64_t)j * N);
    for (int i = nl - 1; i >= 0; i--) {
        sumcheck_prove_layer(&L[i], vals[i], rz1, rz2, alpha, beta, &t, pads, R, N, helpers, evals_buf);
        alpha = tr_challenge(&t);
        beta = tr_challenge(&t);
        for (int j = 0; j < R; j++) {
            memcpy(rz1[j], helpers[j].rx, sizeof(uint32_t) * helpers[j].nrx);
            memcpy(rz2[j], helpers[j].ry, sizeof(uint32_t) * helpers[j].nry);
        }
    }
    /* RawPC::open: empty openings, LinearGKR.hpp:77-86 */

    for (int j = 0; j < R; j++) pad_free(&pads[j]);
    free(pads); free(helpers); free(evals_buf); free(vbuf); free(vals);
    return t.overflow ? 2 : 0;
}

/* ---------------------------------------------------------------- verifier
 * degree_2_eval, include/LinearGKR/sumcheck_verifier_utils.hpp:10-18 (INV_2 = 2^30) */
static void degree_2_eval(const uint32_t* e, uint32_t x, uint32_t N, uint32_t* out) {
    for (uint32_t k = 0; k < N; k++) {
        uint32_t c0 = e[k], v1 = e[N + k], v2 = e[2 * N + k];
        uint32_t c2 = m_mul(1u << 30, m_add(m_sub(v2, m_mul(v1, 2)), c0));
        uint32_t c1 = m_sub(m_sub(v1, c0), c2);
        out[k] = m_add(c0, m_mul(m_add(m_mul(c2, x), c1), x));
    }
}

/* eval_sparse_circuit_connect_poly, :22-56.  ris = 1 (add) or 2 (mul) points. */
static uint32_t eval_sparse(const oracle_layer* L, int is_mul, const uint32_t* rz1, const uint32_t* rz2, uint32_t nz,
                            uint32_t alpha, uint32_t beta, const uint32_t* rx, const uint32_t* ry, uint32_t nx) {
    uint64_t O = 1ull << nz, I = 1ull << nx;
    uint32_t *e1 = (uint32_t*)malloc(O * 4), *e2 = (uint32_t*)malloc(O * 4);
    uint32_t *ex = (uint32_t*)malloc(I * 4), *ey = (uint32_t*)malloc(I * 4);
    eq_evals_primitive(rz1, nz, alpha, e1);
    eq_evals_primitive(rz2, nz, beta, e2);
    eq_evals_primitive(rx, nx, 1, ex);
    if (is_mul) eq_evals_primitive(ry, nx, 1, ey);
    uint32_t v = 0;
    if (is_mul) {
        for (uint64_t g = 0; g < L->n_mul; g++) {
            const uint32_t* s = L->mul + 4 * g;
            uint32_t prod = m_add(e1[s[0]], e2[s[0]]);
            prod = m_mul(prod, ex[s[1]]);
            prod = m_mul(prod, ey[s[2]]);
            v = m_add(v, m_mul(prod, s[3]));
        }
    } else {
        for (uint64_t g = 0; g < L->n_add; g++) {
            const uint32_t* s = L->add + 3 * g;
            uint32_t prod = m_mul(m_add(e1[s[0]], e2[s[0]]), ex[s[1]]);
            v = m_add(v, m_mul(prod, s[2]));
        }
    }
    free(e1); free(e2); free(ex); free(ey);
    return v;
}

static int vec_eq(const uint32_t* a, const uint32_t* b, uint32_t N) { return memcmp(a, b, (size_t)N * 4) == 0; }

typedef struct { const uint8_t* bytes; uint64_t idx, len; int bad; } proof_reader;

/* Proof::get_next_and_step, include/fiat_shamir/transcript.hpp:46-52 */
static void pr_next(proof_reader* p, uint32_t N, uint32_t* out) {
    if (p->idx + (uint64_t)N * 4 > p->len) { p->bad = 1; memset(out, 0, (size_t)N * 4); return; }
    memcpy(out, p->bytes + p->idx, (size_t)N * 4);
    for (uint32_t k = 0; k < N; k++) out[k] = m_reduce(out[k]);
    p->idx += (uint64_t)N * 4;
}

/* Verifier::verify (LinearGKR.hpp:105-149), gkr_verify (gkr.hpp:75-122),
 * sumcheck_verify_gkr_layer (sumcheck.hpp:113-176), RawPC::verify (raw.hpp:75-78) */
int oracle_verify(const oracle_layer* L, int nl, uint32_t N, const uint32_t* input, int grinding_bits,
                  const uint8_t* proof, uint64_t proof_len, const uint32_t* claimed_v) {
    (void)input;
    if (check_layers(L, nl, N)) return -1;
    int R = oracle_num_repetitions(grinding_bits);
    if (R > 8) return -1;
    uint64_t I0 = 1ull << L[0].nb_input_vars;
    uint64_t com_bytes = I0 * N * 4;
    if (proof_len < com_bytes + 32) return 0;
    uint32_t* commitment = (uint32_t*)malloc(com_bytes);
    memcpy(commitment, proof, com_bytes);
    for (uint64_t i = 0; i < I0 * N; i++) commitment[i] = m_reduce(commitment[i]);

    uint64_t tcap = proof_len + 64;
    uint8_t* tbuf = (uint8_t*)malloc(tcap);
    transcript t;
    tr_init(&t, tbuf, tcap);
    tr_append(&t, proof, com_bytes);
    grind(&t, grinding_bits);
    proof_reader pr = {proof, com_bytes + 32, proof_len, 0};

    uint32_t rz1[8][32], rz2[8][32], rx[8][32], ry[8][32];
    uint32_t nz = L[nl - 1].nb_output_vars;
    for (uint32_t i = 0; i < nz; i++)
        for (int j = 0; j < R; j++) { rz1[j][i] = tr_challenge(&t); rz2[j][i] = 0; }
    uint32_t alpha = 1, beta = 0;
    uint32_t* cv1 = (uint32_t*)malloc((size_t)R * N * 4);
    uint32_t* cv2 = (uint32_t*)calloc((size_t)R * N, 4);
    memcpy(cv1, claimed_v, (size_t)R * N * 4);
    for (uint64_t i = 0; i < (uint64_t)R * N; i++) cv1[i] = m_reduce(cv1[i]);
    uint32_t* sum = (uint32_t*)malloc((size_t)R * N * 4);
    uint32_t* vx = (uint32_t*)malloc((size_t)R * N * 4);
    uint32_t* vy = (uint32_t*)malloc((size_t)R * N * 4);
    uint32_t* ev = (uint32_t*)malloc(3ull * N * 4);
    int verified = 1;

    for (int li = nl - 1; li >= 0; li--) {
        const oracle_layer* Ly = &L[li];
        uint32_t n = Ly->nb_input_vars;
        for (int j = 0; j < R; j++)
            for (uint32_t k = 0; k < N; k++)
                sum[j * N + k] = m_add(m_mul(cv1[j * N + k], alpha), m_mul(cv2[j * N + k], beta));
        for (uint32_t i_var = 0; i_var < 2 * n; i_var++) {
            for (int j = 0; j < R; j++) {
                pr_next(&pr, N, ev); pr_next(&pr, N, ev + N); pr_next(&pr, N, ev + 2 * N);
                tr_append(&t, ev, 3ull * N * 4);
                uint32_t r = tr_challenge(&t);
                if (i_var < n) rx[j][i_var] = r; else ry[j][i_var - n] = r;
                for (uint32_t k = 0; k < N; k++)
                    if (m_add(ev[k], ev[N + k]) != sum[j * N + k]) verified = 0;
                degree_2_eval(ev, r, N, sum + j * N);
                if (i_var == n - 1) {
                    pr_next(&pr, N, vx + j * N);
                    uint32_t a = eval_sparse(Ly, 0, rz1[j], rz2[j], Ly->nb_output_vars, alpha, beta, rx[j], NULL, n);
                    for (uint32_t k = 0; k < N; k++) sum[j * N + k] = m_sub(sum[j * N + k], m_mul(vx[j * N + k], a));
                    tr_append(&t, vx + j * N, (uint64_t)N * 4);
                }
            }
        }
        for (int j = 0; j < R; j++) {
            pr_next(&pr, N, vy + j * N);
            uint32_t m = eval_sparse(Ly, 1, rz1[j], rz2[j], Ly->nb_output_vars, alpha, beta, rx[j], ry[j], n);
            for (uint32_t k = 0; k < N; k++)
                if (sum[j * N + k] != m_mul(m_mul(vx[j * N + k], vy[j * N + k]), m)) verified = 0;
            tr_append(&t, vy + j * N, (uint64_t)N * 4);
        }
        alpha = tr_challenge(&t);
        beta = tr_challenge(&t);
        for (int j = 0; j < R; j++) {
            memcpy(rz1[j], rx[j], 4 * n);
            memcpy(rz2[j], ry[j], 4 * n);
        }
        memcpy(cv1, vx, (size_t)R * N * 4);
        memcpy(cv2, vy, (size_t)R * N * 4);
    }
    /* RawPC::verify at rz1 and rz2 with the last layer's claims (openings are empty). */
    uint32_t n0 = L[0].nb_input_vars;
    uint32_t* e = (uint32_t*)malloc((size_t)N * 4);
    for (int j = 0; j < R; j++) {
        oracle_eval_multilinear(commitment, n0, N, rz1[j], e);
        if (!vec_eq(e, cv1 + j * N, N)) verified = 0;
        oracle_eval_multilinear(commitment, n0, N, rz2[j], e);
        if (!vec_eq(e, cv2 + j * N, N)) verified = 0;
    }
    if (pr.bad) verified = 0;
    free(e); free(commitment); free(tbuf); free(cv1); free(cv2); free(sum); free(vx); free(vy); free(ev);
    return verified;
}

/* ---------------------------------------------------------------- throughput harness */
typedef struct {
    const oracle_layer* L;
    int nl;
    uint32_t N;
    const uint32_t* input;
    int grinding_bits, reps;
    int rc;
} bench_arg;

static void* bench_thread(void* p) {
    bench_arg* a = (bench_arg*)p;
    int R = oracle_num_repetitions(a->grinding_bits);
    uint64_t need = oracle_proof_size(a->L, a->nl, a->N, R);
    uint8_t* proof = (uint8_t*)malloc(need);
    uint32_t* cv = (uint32_t*)malloc((size_t)R * a->N * 4);
    uint64_t len;
    a->rc = 0;
    for (int i = 0; i < a->reps; i++)
        if (oracle_prove(a->L, a->nl, a->N, a->input, a->grinding_bits, proof, need, &len, cv)) a->rc = -1;
    free(proof); free(cv);
    return NULL;
}

double oracle_bench(const oracle_layer* L, int nl, uint32_t N, const uint32_t* input, int grinding_bits,
                    int n_threads, int proofs_per_thread) {
    if (n_threads < 1 || n_threads > 1024) return -1;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * n_threads);
    bench_arg* args = (bench_arg*)malloc(sizeof(bench_arg) * n_threads);
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    for (int i = 0; i < n_threads; i++) {
        args[i] = (bench_arg){L, nl, N, input, grinding_bits, proofs_per_thread, 0};
        pthread_create(&th[i], NULL, bench_thread, &args[i]);
    }
    int rc = 0;
    for (int i = 0; i < n_threads; i++) { pthread_join(th[i], NULL); rc |= args[i].rc; }
    clock_gettime(CLOCK_MONOTONIC, &t1);
    free(th); free(args);
    if (rc) return -1;
    return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}
