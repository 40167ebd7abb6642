/* Test infrastructure only: BN254 restatement of the reference prover and verifier
 * (Config::field_type = BN254, include/configuration/config.hpp:12-16,53-65: one repetition).
 *
 * The same protocol as gkr_oracle.c (which cites the reference lines it follows) over the
 * BN254 scalar field of bn254.h.  Inside this file every value is held in Montgomery form
 * (x * 2^256 mod r); bytes entering the transcript are canonical (32 little-endian bytes per
 * element), and a 32-byte digest becomes a challenge by from_bytes (reduce mod r).  Pinned
 * against the reference templates instantiated over the same field (oracle/ref_driver.cpp)
 * and against tests/golden/.  Only tests and bench.py's CPU-baseline arm load it.
 */
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "bn254.h"
#include "gkr_oracle.h"

typedef bn_t fe;

static fe fe_r2(void) {
    fe r;
    memcpy(r.v, BN_R2, 32);
    return r;
}
static inline fe to_m(fe a) { return bn_mont(a, fe_r2()); }
static inline fe from_m(fe a) {
    fe one = {{1, 0, 0, 0}};
    return bn_mont(a, one);
}
static inline fe fm(fe a, fe b) { return bn_mont(a, b); }
static inline fe fa(fe a, fe b) { return bn_add(a, b); }
static inline fe fs(fe a, fe b) { return bn_sub(a, b); }
static inline fe small(uint32_t x) { return to_m(bn_from_u32(x)); }
static inline fe fe_zero(void) {
    fe z = {{0, 0, 0, 0}};
    return z;
}
static inline int fe_eq(fe a, fe b) { return bn_eq(a, b); }

/* ---------------------------------------------------------------- transcript
 * As in gkr_oracle.c (transcript.hpp:87-175); rows are serialised canonically. */
typedef struct {
    uint8_t* bytes;
    uint64_t len, cap, hash_start;
    uint8_t digest[32];
    int overflow;
} tr_t;

static void tr_init(tr_t* t, uint8_t* buf, uint64_t cap) {
    t->bytes = buf;
    t->len = 0;
    t->cap = cap;
    t->hash_start = 0;
    t->overflow = 0;
    memset(t->digest, 0, 32);
}
static void tr_append(tr_t* t, const void* p, uint64_t n) {
    if (t->len + n > t->cap) {
        t->overflow = 1;
        t->len += n;
        return;
    }
    memcpy(t->bytes + t->len, p, n);
    t->len += n;
}
/* Appends a row of N Montgomery values as their canonical bytes. */
static void tr_append_row(tr_t* t, const fe* row, uint32_t N) {
    for (uint32_t k = 0; k < N; k++) {
        uint8_t b[32];
        bn_to_bytes(from_m(row[k]), b);
        tr_append(t, b, 32);
    }
}
static void tr_hash_to_digest(tr_t* t) {
    if (t->len > t->hash_start) {
        oracle_fs_hash(t->bytes + t->hash_start, t->len - t->hash_start, t->digest);
        t->hash_start = t->len;
    } else {
        oracle_fs_hash(t->digest, 32, t->digest);
    }
}
/* challenge_f: the digest read little-endian, reduced mod r (canonical). */
static fe tr_challenge(tr_t* t) {
    tr_hash_to_digest(t);
    return bn_from_bytes(t->digest);
}
/* grind (LinearGKR.hpp:13-32) with 256/254 = 1 challenge of 32 bytes. */
static void grind(tr_t* t, int grinding_bits) {
    uint8_t h[32];
    bn_to_bytes(tr_challenge(t), h);
    for (long i = 0; i < (1L << grinding_bits); i++) oracle_fs_hash(h, 32, h);
    tr_append(t, h, 32);
}

int oracle_bn254_num_repetitions(int grinding_bits) {
    int s = 100 - grinding_bits;
    return s / 254 + (s % 254 != 0);
}

uint64_t oracle_bn254_proof_size(const oracle_layer* L, int nl, uint32_t N) {
    uint64_t rows = 0;
    for (int l = 0; l < nl; l++) rows += 6ull * L[l].nb_input_vars + 2;
    return (1ull << L[0].nb_input_vars) * N * 32 + 32 + rows * N * 32;
}

/* ---------------------------------------------------------------- circuit */
static int check_layers(const oracle_layer* L, int nl, uint32_t N) {
    if (nl <= 0 || N == 0) return -1;
    for (int l = 0; l < nl; l++) {
        if (L[l].nb_input_vars > 30 || L[l].nb_output_vars > 30) return -1;
        if (l + 1 < nl && L[l].nb_output_vars != L[l + 1].nb_input_vars) return -1;
        uint64_t I = 1ull << L[l].nb_input_vars, O = 1ull << L[l].nb_output_vars;
        for (uint64_t g = 0; g < L[l].n_mul; g++) {
            const uint32_t* s = L[l].mul + 4 * g;
            if (s[0] >= O || s[1] >= I || s[2] >= I) return -1;
        }
        for (uint64_t g = 0; g < L[l].n_add; g++) {
            const uint32_t* s = L[l].add + 3 * g;
            if (s[0] >= O || s[1] >= I) return -1;
        }
    }
    return 0;
}

static void layer_eval(const oracle_layer* L, uint32_t N, const fe* in, fe* out) {
    uint64_t O = 1ull << L->nb_output_vars;
    for (uint64_t i = 0; i < O * N; i++) out[i] = fe_zero();
    for (uint64_t g = 0; g < L->n_mul; g++) {
        const uint32_t* s = L->mul + 4 * g;
        fe c = small(s[3]);
        fe* o = out + (uint64_t)s[0] * N;
        const fe *a = in + (uint64_t)s[1] * N, *b = in + (uint64_t)s[2] * N;
        for (uint32_t k = 0; k < N; k++) o[k] = fa(o[k], fm(fm(a[k], b[k]), c));
    }
    for (uint64_t g = 0; g < L->n_add; g++) {
        const uint32_t* s = L->add + 3 * g;
        fe c = small(s[2]);
        fe* o = out + (uint64_t)s[0] * N;
        const fe* a = in + (uint64_t)s[1] * N;
        for (uint32_t k = 0; k < N; k++) o[k] = fa(o[k], fm(a[k], c));
    }
}

static uint64_t values_rows(const oracle_layer* L, int nl) {
    uint64_t rows = 0;
    for (int l = 0; l < nl; l++) rows += 1ull << L[l].nb_input_vars;
    return rows + (1ull << L[nl - 1].nb_output_vars);
}

/* Canonical input (rows x N x 4 limbs) -> Montgomery values of every layer.  -1 if an
 * input element is not below r. */
static int eval_all(const oracle_layer* L, int nl, uint32_t N, const uint64_t* input, fe* buf, fe** vals) {
    uint64_t off = 0;
    for (int l = 0; l <= nl; l++) {
        vals[l] = buf + off;
        off += (l < nl ? (1ull << L[l].nb_input_vars) : (1ull << L[nl - 1].nb_output_vars)) * N;
    }
    uint64_t n = (1ull << L[0].nb_input_vars) * N;
    for (uint64_t i = 0; i < n; i++) {
        fe x;
        memcpy(x.v, input + 4 * i, 32);
        if (bn_geq_r(x.v)) return -1;
        vals[0][i] = to_m(x);
    }
    for (int l = 0; l < nl; l++) layer_eval(&L[l], N, vals[l], vals[l + 1]);
    return 0;
}

int oracle_bn254_evaluate(const oracle_layer* L, int nl, uint32_t N, const uint64_t* input, uint64_t* out) {
    if (check_layers(L, nl, N)) return -1;
    uint64_t rows = values_rows(L, nl);
    fe* buf = (fe*)malloc(rows * N * sizeof(fe));
    fe** vals = (fe**)malloc(sizeof(fe*) * (nl + 1));
    int rc = eval_all(L, nl, N, input, buf, vals);
    if (rc == 0)
        for (uint64_t i = 0; i < rows * N; i++) {
            fe c = from_m(buf[i]);
            memcpy(out + 4 * i, c.v, 32);
        }
    free(buf);
    free(vals);
    return rc;
}

/* eq(r, .) * factor over 2^nr points (sumcheck_common.hpp:9-53: _eq(r, 0) = 1 - r, _eq(r, 1) = r). */
static void eq_table(const fe* r, uint32_t nr, fe factor, fe* out) {
    const fe one = small(1);
    out[0] = factor;
    uint64_t cur = 1;
    for (uint32_t i = 0; i < nr; i++) {
        fe e0 = fs(one, r[i]), e1 = r[i];
        for (uint64_t j = 0; j < cur; j++) {
            out[j + cur] = fm(out[j], e1);
            out[j] = fm(out[j], e0);
        }
        cur <<= 1;
    }
}

/* eval_multilinear (poly.hpp:88-104) of rows x N Montgomery values at r. */
static void eval_ml(const fe* evals, uint32_t nb_vars, uint32_t N, const fe* r, fe* out) {
    uint64_t n = 1ull << nb_vars;
    fe* s = (fe*)malloc(n * N * sizeof(fe));
    memcpy(s, evals, n * N * sizeof(fe));
    uint64_t cur = n >> 1;
    for (uint32_t v = 0; v < nb_vars; v++) {
        for (uint64_t i = 0; i < cur; i++)
            for (uint32_t k = 0; k < N; k++) {
                fe a = s[2 * i * N + k], b = s[(2 * i + 1) * N + k];
                s[i * N + k] = fa(a, fm(fs(b, a), r[v]));
            }
        cur >>= 1;
    }
    memcpy(out, s, N * sizeof(fe));
    free(s);
}

/* ---------------------------------------------------------------- sumcheck prover */
typedef struct {
    fe *f, *hg, *eqz, *eq2, *eqx;
    fe *evals;
    uint32_t N;
} pad_t;

/* One phase over n variables: rounds of poly_eval_at (sumcheck_helper.hpp:68-102) and
 * receive_challenge (:104-133).  f starts as a copy of the layer input.  In the last round
 * the 2->1 fold leaves the claim in f[0..N). */
static void phase(pad_t* p, const fe* v, uint32_t n, tr_t* t, fe* rs, int append_claim) {
    const uint32_t N = p->N;
    const fe six = small(6), three = small(3), two = small(2);
    memcpy(p->f, v, ((uint64_t)1 << n) * N * sizeof(fe));
    for (uint32_t i = 0; i < n; i++) {
        uint64_t pairs = 1ull << (n - i - 1);
        fe *p0 = p->evals, *p1 = p->evals + N, *p2 = p->evals + 2 * N;
        for (uint32_t k = 0; k < 3 * N; k++) p->evals[k] = fe_zero();
        for (uint64_t q = 0; q < pairs; q++)
            for (uint32_t k = 0; k < N; k++) {
                fe f0 = p->f[2 * q * N + k], f1 = p->f[(2 * q + 1) * N + k];
                fe h0 = p->hg[2 * q * N + k], h1 = p->hg[(2 * q + 1) * N + k];
                p0[k] = fa(p0[k], fm(f0, h0));
                p1[k] = fa(p1[k], fm(f1, h1));
                p2[k] = fa(p2[k], fm(fa(f0, f1), fa(h0, h1)));
            }
        for (uint32_t k = 0; k < N; k++) p2[k] = fs(fa(fm(p1[k], six), fm(p0[k], three)), fm(p2[k], two));
        tr_append_row(t, p0, N);
        tr_append_row(t, p1, N);
        tr_append_row(t, p2, N);
        fe r = to_m(tr_challenge(t));
        rs[i] = r;
        for (uint64_t q = 0; q < pairs; q++)
            for (uint32_t k = 0; k < N; k++) {
                fe a = p->f[2 * q * N + k], b = p->f[(2 * q + 1) * N + k];
                fe ga = p->hg[2 * q * N + k], gb = p->hg[(2 * q + 1) * N + k];
                p->f[q * N + k] = fa(a, fm(fs(b, a), r));
                p->hg[q * N + k] = fa(ga, fm(fs(gb, ga), r));
            }
        if (i == n - 1 && append_claim) tr_append_row(t, p->f, N);
    }
}

/* sumcheck_prove_gkr_layer (sumcheck.hpp:52-111) for one repetition. */
static void prove_layer(const oracle_layer* L, const fe* v, const fe* rz1, const fe* rz2, fe alpha, fe beta, tr_t* t,
                        pad_t* p, fe* rx, fe* ry) {
    const uint32_t N = p->N, n = L->nb_input_vars, m = L->nb_output_vars;
    uint64_t I = 1ull << n, O = 1ull << m;
    /* phase one: hg(x) = sum_mul c eq(z) v(y) + sum_add c eq(z) (_prepare_g_x_vals, :172-231) */
    eq_table(rz1, m, alpha, p->eqz);
    eq_table(rz2, m, beta, p->eq2);
    for (uint64_t z = 0; z < O; z++) p->eqz[z] = fa(p->eqz[z], p->eq2[z]);
    for (uint64_t i = 0; i < I * N; i++) p->hg[i] = fe_zero();
    for (uint64_t g = 0; g < L->n_mul; g++) {
        const uint32_t* s = L->mul + 4 * g;
        fe w = fm(small(s[3]), p->eqz[s[0]]);
        for (uint32_t k = 0; k < N; k++)
            p->hg[(uint64_t)s[1] * N + k] = fa(p->hg[(uint64_t)s[1] * N + k], fm(v[(uint64_t)s[2] * N + k], w));
    }
    for (uint64_t g = 0; g < L->n_add; g++) {
        const uint32_t* s = L->add + 3 * g;
        fe w = fm(small(s[2]), p->eqz[s[0]]);
        for (uint32_t k = 0; k < N; k++) p->hg[(uint64_t)s[1] * N + k] = fa(p->hg[(uint64_t)s[1] * N + k], w);
    }
    phase(p, v, n, t, rx, 1);
    fe* vx = (fe*)malloc(N * sizeof(fe));
    memcpy(vx, p->f, N * sizeof(fe));
    /* phase two: hg(y) = sum_mul c eq(z) eq(rx, x) vx (_prepare_h_y_vals, :233-261) */
    eq_table(rx, n, small(1), p->eqx);
    for (uint64_t i = 0; i < I * N; i++) p->hg[i] = fe_zero();
    for (uint64_t g = 0; g < L->n_mul; g++) {
        const uint32_t* s = L->mul + 4 * g;
        fe w = fm(fm(p->eqz[s[0]], p->eqx[s[1]]), small(s[3]));
        for (uint32_t k = 0; k < N; k++)
            p->hg[(uint64_t)s[2] * N + k] = fa(p->hg[(uint64_t)s[2] * N + k], fm(vx[k], w));
    }
    phase(p, v, n, t, ry, 0);
    tr_append_row(t, p->f, N); /* vy */
    free(vx);
}

int oracle_bn254_prove(const oracle_layer* L, int nl, uint32_t N, const uint64_t* input, int grinding_bits,
                       uint8_t* proof_out, uint64_t proof_cap, uint64_t* proof_len, uint64_t* claimed_v) {
    if (check_layers(L, nl, N)) return -1;
    for (int l = 0; l < nl; l++)
        if (L[l].nb_input_vars == 0) return -1;
    if (oracle_bn254_num_repetitions(grinding_bits) != 1) return -1;
    uint64_t need = oracle_bn254_proof_size(L, nl, N);
    *proof_len = need;
    if (need > proof_cap) return 2;

    fe** vals = (fe**)malloc(sizeof(fe*) * (nl + 1));
    fe* vbuf = (fe*)malloc(values_rows(L, nl) * N * sizeof(fe));
    if (eval_all(L, nl, N, input, vbuf, vals)) {
        free(vals);
        free(vbuf);
        return -1;
    }
    uint32_t max_in = 0, max_out = 0;
    for (int l = 0; l < nl; l++) {
        if (L[l].nb_input_vars > max_in) max_in = L[l].nb_input_vars;
        if (L[l].nb_output_vars > max_out) max_out = L[l].nb_output_vars;
    }
    pad_t p;
    p.N = N;
    p.f = (fe*)malloc((1ull << max_in) * N * sizeof(fe));
    p.hg = (fe*)malloc((1ull << max_in) * N * sizeof(fe));
    p.eqz = (fe*)malloc((1ull << max_out) * sizeof(fe));
    p.eq2 = (fe*)malloc((1ull << max_out) * sizeof(fe));
    p.eqx = (fe*)malloc((1ull << max_in) * sizeof(fe));
    p.evals = (fe*)malloc(3ull * N * sizeof(fe));

    tr_t t;
    tr_init(&t, proof_out, proof_cap);
    tr_append(&t, input, (1ull << L[0].nb_input_vars) * N * 32); /* RAW commitment */
    grind(&t, grinding_bits);

    fe rz1[32], rz2[32], rx[32], ry[32];
    uint32_t nz = L[nl - 1].nb_output_vars;
    for (uint32_t i = 0; i < nz; i++) {
        rz1[i] = to_m(tr_challenge(&t));
        rz2[i] = fe_zero();
    }
    fe alpha = small(1), beta = fe_zero();
    fe* cv = (fe*)malloc(N * sizeof(fe));
    eval_ml(vals[nl], nz, N, rz1, cv);
    for (uint32_t k = 0; k < N; k++) {
        fe c = from_m(cv[k]);
        memcpy(claimed_v + 4ull * k, c.v, 32);
    }
    for (int i = nl - 1; i >= 0; i--) {
        prove_layer(&L[i], vals[i], rz1, rz2, alpha, beta, &t, &p, rx, ry);
        alpha = to_m(tr_challenge(&t));
        beta = to_m(tr_challenge(&t));
        memcpy(rz1, rx, sizeof(fe) * L[i].nb_input_vars);
        memcpy(rz2, ry, sizeof(fe) * L[i].nb_input_vars);
    }
    free(cv);
    free(p.f);
    free(p.hg);
    free(p.eqz);
    free(p.eq2);
    free(p.eqx);
    free(p.evals);
    free(vbuf);
    free(vals);
    return t.overflow ? 2 : 0;
}

/* ---------------------------------------------------------------- verifier (as in gkr_oracle.c) */
static fe eval_sparse(const oracle_layer* L, int is_mul, const fe* rz1, const fe* rz2, uint32_t nz, fe alpha,
                      fe beta, const fe* rx, const fe* ry, uint32_t nx) {
    uint64_t O = 1ull << nz, I = 1ull << nx;
    fe *e1 = (fe*)malloc(O * sizeof(fe)), *e2 = (fe*)malloc(O * sizeof(fe));
    fe *ex = (fe*)malloc(I * sizeof(fe)), *ey = (fe*)malloc(I * sizeof(fe));
    eq_table(rz1, nz, alpha, e1);
    eq_table(rz2, nz, beta, e2);
    eq_table(rx, nx, small(1), ex);
    if (is_mul) eq_table(ry, nx, small(1), ey);
    fe v = fe_zero();
    if (is_mul) {
        for (uint64_t g = 0; g < L->n_mul; g++) {
            const uint32_t* s = L->mul + 4 * g;
            fe prod = fm(fm(fa(e1[s[0]], e2[s[0]]), ex[s[1]]), ey[s[2]]);
            v = fa(v, fm(prod, small(s[3])));
        }
    } else {
        for (uint64_t g = 0; g < L->n_add; g++) {
            const uint32_t* s = L->add + 3 * g;
            v = fa(v, fm(fm(fa(e1[s[0]], e2[s[0]]), ex[s[1]]), small(s[2])));
        }
    }
    free(e1);
    free(e2);
    free(ex);
    free(ey);
    return v;
}

typedef struct {
    const uint8_t* bytes;
    uint64_t idx, len;
    int bad;
} reader_t;

/* Next N elements of the proof (from_bytes reduces), as Montgomery values. */
static void rd_next(reader_t* p, uint32_t N, fe* out) {
    for (uint32_t k = 0; k < N; k++) {
        if (p->idx + 32 > p->len) {
            p->bad = 1;
            out[k] = fe_zero();
            continue;
        }
        out[k] = to_m(bn_from_bytes(p->bytes + p->idx));
        p->idx += 32;
    }
}

int oracle_bn254_verify(const oracle_layer* L, int nl, uint32_t N, const uint64_t* input, int grinding_bits,
                        const uint8_t* proof, uint64_t proof_len, const uint64_t* claimed_v) {
    (void)input;
    if (check_layers(L, nl, N)) return -1;
    if (oracle_bn254_num_repetitions(grinding_bits) != 1) return -1;
    uint64_t I0 = 1ull << L[0].nb_input_vars;
    uint64_t com_bytes = I0 * N * 32;
    if (proof_len < com_bytes + 32) return 0;
    fe* commitment = (fe*)malloc(I0 * N * sizeof(fe));
    for (uint64_t i = 0; i < I0 * N; i++) commitment[i] = to_m(bn_from_bytes(proof + 32 * i));

    uint64_t tcap = proof_len + 64;
    uint8_t* tbuf = (uint8_t*)malloc(tcap);
    tr_t t;
    tr_init(&t, tbuf, tcap);
    tr_append(&t, proof, com_bytes);
    grind(&t, grinding_bits);
    reader_t pr = {proof, com_bytes + 32, proof_len, 0};

    fe rz1[32], rz2[32], rx[32], ry[32];
    uint32_t nz = L[nl - 1].nb_output_vars;
    for (uint32_t i = 0; i < nz; i++) {
        rz1[i] = to_m(tr_challenge(&t));
        rz2[i] = fe_zero();
    }
    fe alpha = small(1), beta = fe_zero();
    const fe inv2 = to_m((fe){{0xa1f0fac9f8000001ull, 0x9419f4243cdcb848ull, 0xdc2822db40c0ac2eull,
                               0x183227397098d014ull}}); /* (r + 1) / 2 */
    fe *cv1 = (fe*)malloc(N * sizeof(fe)), *cv2 = (fe*)malloc(N * sizeof(fe)), *sum = (fe*)malloc(N * sizeof(fe));
    fe *vx = (fe*)malloc(N * sizeof(fe)), *vy = (fe*)malloc(N * sizeof(fe)), *ev = (fe*)malloc(3ull * N * sizeof(fe));
    for (uint32_t k = 0; k < N; k++) {
        fe c;
        memcpy(c.v, claimed_v + 4ull * k, 32);
        while (bn_geq_r(c.v)) bn_sub_r(c.v);
        cv1[k] = to_m(c);
        cv2[k] = fe_zero();
    }
    int verified = 1;
    for (int li = nl - 1; li >= 0; li--) {
        const oracle_layer* Ly = &L[li];
        uint32_t n = Ly->nb_input_vars;
        for (uint32_t k = 0; k < N; k++) sum[k] = fa(fm(cv1[k], alpha), fm(cv2[k], beta));
        for (uint32_t i_var = 0; i_var < 2 * n; i_var++) {
            rd_next(&pr, N, ev);
            rd_next(&pr, N, ev + N);
            rd_next(&pr, N, ev + 2 * N);
            tr_append_row(&t, ev, 3 * N);
            fe r = to_m(tr_challenge(&t));
            if (i_var < n) rx[i_var] = r; else ry[i_var - n] = r;
            for (uint32_t k = 0; k < N; k++) {
                if (!fe_eq(fa(ev[k], ev[N + k]), sum[k])) verified = 0;
                /* degree_2_eval (sumcheck_verifier_utils.hpp:10-18) */
                fe c0 = ev[k], v1 = ev[N + k], v2 = ev[2 * N + k];
                fe c2 = fm(inv2, fa(fs(v2, fa(v1, v1)), c0));
                fe c1 = fs(fs(v1, c0), c2);
                sum[k] = fa(c0, fm(fa(fm(c2, r), c1), r));
            }
            if (i_var == n - 1) {
                rd_next(&pr, N, vx);
                fe a = eval_sparse(Ly, 0, rz1, rz2, Ly->nb_output_vars, alpha, beta, rx, NULL, n);
                for (uint32_t k = 0; k < N; k++) sum[k] = fs(sum[k], fm(vx[k], a));
                tr_append_row(&t, vx, N);
            }
        }
        rd_next(&pr, N, vy);
        fe mm = eval_sparse(Ly, 1, rz1, rz2, Ly->nb_output_vars, alpha, beta, rx, ry, n);
        for (uint32_t k = 0; k < N; k++)
            if (!fe_eq(sum[k], fm(fm(vx[k], vy[k]), mm))) verified = 0;
        tr_append_row(&t, vy, N);
        alpha = to_m(tr_challenge(&t));
        beta = to_m(tr_challenge(&t));
        memcpy(rz1, rx, sizeof(fe) * n);
        memcpy(rz2, ry, sizeof(fe) * n);
        memcpy(cv1, vx, N * sizeof(fe));
        memcpy(cv2, vy, N * sizeof(fe));
    }
    /* RawPC::verify at rz1 and rz2 against the commitment */
    uint32_t n0 = L[0].nb_input_vars;
    fe* e = (fe*)malloc(N * sizeof(fe));
    eval_ml(commitment, n0, N, rz1, e);
    for (uint32_t k = 0; k < N; k++)
        if (!fe_eq(e[k], cv1[k])) verified = 0;
    eval_ml(commitment, n0, N, rz2, e);
    for (uint32_t k = 0; k < N; k++)
        if (!fe_eq(e[k], cv2[k])) verified = 0;
    if (pr.bad) verified = 0; /* like the reference, bytes after the last claim are not read */
    free(e);
    free(commitment);
    free(tbuf);
    free(cv1);
    free(cv2);
    free(sum);
    free(vx);
    free(vy);
    free(ev);
    return verified;
}

/* ---------------------------------------------------------------- throughput harness */
typedef struct {
    const oracle_layer* L;
    int nl;
    uint32_t N;
    const uint64_t* input;
    int grinding_bits, reps, rc;
} bench_arg;

static void* bench_thread(void* q) {
    bench_arg* a = (bench_arg*)q;
    uint64_t need = oracle_bn254_proof_size(a->L, a->nl, a->N);
    uint8_t* proof = (uint8_t*)malloc(need);
    uint64_t* cv = (uint64_t*)malloc((size_t)a->N * 32);
    uint64_t len;
    a->rc = 0;
    for (int i = 0; i < a->reps; i++)
        if (oracle_bn254_prove(a->L, a->nl, a->N, a->input, a->grinding_bits, proof, need, &len, cv)) a->rc = -1;
    free(proof);
    free(cv);
    return NULL;
}

double oracle_bn254_bench(const oracle_layer* L, int nl, uint32_t N, const uint64_t* input, int grinding_bits,
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
    for (int i = 0; i < n_threads; i++) {
        pthread_join(th[i], NULL);
        rc |= args[i].rc;
    }
    clock_gettime(CLOCK_MONOTONIC, &t1);
    free(th);
    free(args);
    if (rc) return -1;
    return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}
