// GPU-assisted verifier (M31: Verifier, BN254: BnVerifier): Verifier::verify (include/LinearGKR/LinearGKR.hpp:
// 105-149), gkr_verify (include/LinearGKR/gkr.hpp:75-122) and sumcheck_verify_gkr_layer
// (include/LinearGKR/sumcheck.hpp:113-176).  Part of prover.cu's translation unit (included
// inside its anonymous namespace after the provers, whose lanes and circuit it uses).
//
// The host replays the transcript (the same SHA-256 schedule as the prover) and does the
// per-lane round checks; the device does what scales with the circuit and the input: the eq
// tables and gate sums of eval_sparse_circuit_connect_poly
// (include/LinearGKR/sumcheck_verifier_utils.hpp:22-56) per layer, and RawPC::verify's
// eval_multilinear of the whole committed input at rz1_j and rz2_j (include/poly_commit/
// raw.hpp:75-78, include/poly_commit/poly.hpp:88-104).
//
// Decisions follow the reference: proof values are read with from_bytes (reduced mod p), the
// proof's grinding bytes are skipped rather than compared (LinearGKR.hpp:121-124), bytes
// after the last claim are ignored, and a proof that runs out is rejected.
#pragma once

struct Verifier {
    gkrgpu_ctx& X;
    Lane& c;
    const gkrgpu_circuit& C;
    uint32_t N;
    int R;
    char* block = nullptr;
    uint32_t *com = nullptr, *eqz = nullptr, *eqx = nullptr, *eqy = nullptr, *sums = nullptr, *cv = nullptr;
    unsigned long long *gacc = nullptr, *wacc = nullptr;
    unsigned int *gticket = nullptr, *wticket = nullptr;

    Verifier(gkrgpu_ctx& ctx, Lane& lane, const gkrgpu_circuit& circ, uint32_t n, int reps)
        : X(ctx), c(lane), C(circ), N(n), R(reps) {}
    ~Verifier() {
        if (block) cudaFreeAsync(block, c.stream);
    }

    void reserve() {
        const uint64_t I0 = C.in_rows(0), maxI = 1ull << C.max_in_vars, maxO = 1ull << C.max_out_vars;
        size_t o = 0;
        std::vector<std::pair<void**, size_t>> parts = {
            {(void**)&com, I0 * N * 4},      {(void**)&eqz, R * maxO * 4},   {(void**)&eqx, R * maxI * 4},
            {(void**)&eqy, R * maxI * 4},    {(void**)&sums, 16},            {(void**)&cv, (size_t)R * N * 4},
            {(void**)&gacc, 3 * 8},          {(void**)&gticket, 16},         {(void**)&wacc, 9ull * N * 8},
            {(void**)&wticket, 4096},
        };
        size_t zero_from = 0;
        for (auto& p : parts) {
            if (p.first == (void**)&gacc) zero_from = o;
            o += align_up(std::max<size_t>(p.second, 16), 256);
        }
        void* base = nullptr;
        ck(cudaMallocFromPoolAsync(&base, o, X.pool, c.stream), "verifier workspace allocation");
        block = static_cast<char*>(base);
        o = 0;
        for (auto& p : parts) {
            *p.first = block + o;
            o += align_up(std::max<size_t>(p.second, 16), 256);
        }
        ck(cudaMemsetAsync(block + zero_from, 0, o - zero_from, c.stream), "cudaMemsetAsync");
        c.h_cv.ensure((size_t)R * N * 4 + 64, "pinned verifier results");
    }

    void eq_table(uint32_t* out, uint32_t (*r1)[32], uint32_t (*r2)[32], uint32_t f1, uint32_t f2, uint32_t nvars) {
        EqArgs a;
        memset(&a, 0, sizeof(a));
        for (int j = 0; j < R; j++) {
            memcpy(a.r1[j], r1[j], 4 * nvars);
            if (r2) memcpy(a.r2[j], r2[j], 4 * nvars);
        }
        a.f1 = f1;
        a.f2 = r2 ? f2 : 0u;
        a.nvars = nvars;
        a.reps = R;
        c.launch(K_EQ, 4.0 * R * (double)(1ull << nvars), [&] { return launch_eq(out, a, c.stream); });
    }

    // eval_sparse_circuit_connect_poly of layer li for every repetition: the add part (needs
    // rx) or the mul part (needs rx and ry).
    void gate_sums(size_t li, bool mul_part, uint32_t (*rz1)[32], uint32_t (*rz2)[32], uint32_t alpha, uint32_t beta,
                   uint32_t (*rx)[32], uint32_t (*ry)[32], uint32_t out[3]) {
        const DevLayer& Ly = C.layers[li];
        const uint64_t O = 1ull << Ly.nout, I = 1ull << Ly.nin;
        eq_table(eqz, rz1, rz2, alpha, beta, Ly.nout);
        eq_table(eqx, rx, nullptr, 1u, 0u, Ly.nin);
        if (mul_part) eq_table(eqy, ry, nullptr, 1u, 0u, Ly.nin);
        const double gates = mul_part ? (double)Ly.nmul : (double)Ly.nadd;
        c.launch(K_GATE_SUMS, (mul_part ? 16.0 : 8.0) * gates + 4.0 * (O + 1) + 4.0 * R * (O + 2 * I), [&] {
            return launch_gate_sums(mul_part, O, I, mul_part ? Ly.mo_off : Ly.ao_off,
                                    mul_part ? reinterpret_cast<const uint32_t*>(Ly.mo_g)
                                             : reinterpret_cast<const uint32_t*>(Ly.ao_g),
                                    eqz, eqx, eqy, (uint32_t)R, gacc, gticket, sums, c.stream);
        });
        c.copy(c.h_cv.p, sums, 4 * R, cudaMemcpyDeviceToHost, "gate sums readback");
        c.sync();
        memcpy(out, c.h_cv.p, 4 * R);
    }

    // eval_multilinear of the committed input at the R points r[j]; equal to `claims`?
    bool raw_pc_verify(uint32_t (*r)[32], const std::vector<uint32_t>& claims) {
        const uint32_t n0 = C.layers[0].nin;
        const uint64_t rows = 1ull << n0;
        eq_table(eqx, r, nullptr, 1u, 0u, n0);
        const Geo g = X.geo(N, K_WSUM);
        c.launch(K_WSUM, 4.0 * N * rows + 4.0 * R * rows, [&] {
            return launch_wsum(R, com, rows, eqx, g, X.block, X.cta_budget(K_WSUM), RedScratch{wacc, wticket}, cv,
                               c.stream);
        });
        c.copy(c.h_cv.p, cv, (size_t)R * N * 4, cudaMemcpyDeviceToHost, "multilinear evaluation readback");
        c.sync();
        return memcmp(c.h_cv.p, claims.data(), (size_t)R * N * 4) == 0;
    }

    bool run(int grinding_bits, const uint8_t* proof, uint64_t len, const uint32_t* claimed_v) {
        const uint64_t rowb = (uint64_t)N * 4;
        const uint64_t com_bytes = C.in_rows(0) * rowb;
        if (len < com_bytes + 32) return false;
        reserve();
        c.copy(com, proof, com_bytes, cudaMemcpyHostToDevice, "commitment upload");
        c.launch(K_CANONICAL, 8.0 * C.in_rows(0) * N, [&] { return launch_canonicalize(com, C.in_rows(0) * N, c.stream); });

        // transcript: the commitment bytes (hashed in place), grinding
        std::unique_ptr<uint8_t[]> tbuf(new uint8_t[len + 64]);
        Transcript t(tbuf.get(), len + 64, X.fs_hash);
        uint8_t d[32];
        fs_hash(X.fs_hash, proof, com_bytes, d);
        t.appended_prehashed(com_bytes, d);
        grind(t, grinding_bits);
        uint64_t pos = com_bytes + 32;
        bool bad = false;
        // Proof::get_next_and_step of one row (N lanes), reduced
        auto next_row = [&](uint32_t* out) {
            if (pos + rowb > len) {
                bad = true;
                memset(out, 0, rowb);
                return;
            }
            memcpy(out, proof + pos, rowb);
            for (uint32_t k = 0; k < N; k++) out[k] = m31::from_u32(out[k]);
            pos += rowb;
        };

        const size_t L = C.layers.size();
        uint32_t rz1[3][32], rz2[3][32], rx[3][32], ry[3][32];
        memset(rz1, 0, sizeof(rz1));
        memset(rz2, 0, sizeof(rz2));
        const uint32_t nz = C.layers[L - 1].nout;
        for (uint32_t i = 0; i < nz; i++)
            for (int j = 0; j < R; j++) rz1[j][i] = t.challenge();
        uint32_t alpha = 1, beta = 0;
        std::vector<uint32_t> cv1((size_t)R * N), cv2((size_t)R * N, 0u), sum((size_t)R * N), vx((size_t)R * N),
            vy((size_t)R * N), ev(3ull * N);
        for (size_t i = 0; i < (size_t)R * N; i++) cv1[i] = m31::from_u32(claimed_v[i]);
        bool ok = true;

        for (int li = (int)L - 1; li >= 0; li--) {
            const uint32_t n = C.layers[li].nin;
            for (size_t i = 0; i < (size_t)R * N; i++)
                sum[i] = m31::add(m31::mul(cv1[i], alpha), m31::mul(cv2[i], beta));
            for (uint32_t i_var = 0; i_var < 2 * n; i_var++) {
                for (int j = 0; j < R; j++) {
                    next_row(ev.data());
                    next_row(ev.data() + N);
                    next_row(ev.data() + 2 * N);
                    t.append(ev.data(), 3 * rowb);
                    const uint32_t r = t.challenge();
                    (i_var < n ? rx[j][i_var] : ry[j][i_var - n]) = r;
                    uint32_t* s = sum.data() + (size_t)j * N;
                    for (uint32_t k = 0; k < N; k++) {
                        // degree_2_eval (sumcheck_verifier_utils.hpp:10-18), INV_2 = 2^30
                        const uint32_t c0 = ev[k], v1 = ev[N + k], v2 = ev[2 * N + k];
                        if (m31::add(c0, v1) != s[k]) ok = false;
                        const uint32_t c2 = m31::mul(1u << 30, m31::add(m31::sub(v2, m31::mul(v1, 2)), c0));
                        const uint32_t c1 = m31::sub(m31::sub(v1, c0), c2);
                        s[k] = m31::add(c0, m31::mul(m31::add(m31::mul(c2, r), c1), r));
                    }
                    if (i_var == n - 1) {
                        next_row(vx.data() + (size_t)j * N);
                        t.append(vx.data() + (size_t)j * N, rowb);
                    }
                }
                if (i_var == n - 1) {
                    // sum -= vx * add part, for every repetition (no challenge depends on it)
                    uint32_t a[3] = {0, 0, 0};
                    gate_sums((size_t)li, false, rz1, rz2, alpha, beta, rx, ry, a);
                    for (int j = 0; j < R; j++)
                        for (uint32_t k = 0; k < N; k++) {
                            uint32_t& s = sum[(size_t)j * N + k];
                            s = m31::sub(s, m31::mul(vx[(size_t)j * N + k], a[j]));
                        }
                }
            }
            for (int j = 0; j < R; j++) {
                next_row(vy.data() + (size_t)j * N);
                t.append(vy.data() + (size_t)j * N, rowb);
            }
            uint32_t m[3] = {0, 0, 0};
            gate_sums((size_t)li, true, rz1, rz2, alpha, beta, rx, ry, m);
            for (int j = 0; j < R; j++)
                for (uint32_t k = 0; k < N; k++) {
                    const size_t i = (size_t)j * N + k;
                    if (sum[i] != m31::mul(m31::mul(vx[i], vy[i]), m[j])) ok = false;
                }
            alpha = t.challenge();
            beta = t.challenge();
            for (int j = 0; j < R; j++) {
                memcpy(rz1[j], rx[j], 4 * n);
                memcpy(rz2[j], ry[j], 4 * n);
            }
            cv1 = vx;
            cv2 = vy;
        }
        // RawPC::verify against the commitment, at rz1_j and rz2_j
        if (!raw_pc_verify(rz1, cv1)) ok = false;
        if (!raw_pc_verify(rz2, cv2)) ok = false;
        c.resolve_events();
        return ok && !bad;
    }
};

// The same verifier for BN254 circuits (one repetition; field operations of fr_host.hpp on
// canonical values on the host, Montgomery tables on the device).
struct BnVerifier {
    gkrgpu_ctx& X;
    Lane& c;
    const gkrgpu_circuit& C;
    uint32_t N;
    char* block = nullptr;
    uint32_t *raw = nullptr, *com = nullptr, *sums = nullptr, *cv = nullptr;
    bn::Fr *eqz = nullptr, *eqx = nullptr, *eqy = nullptr;
    unsigned long long *gacc = nullptr, *wacc = nullptr;
    unsigned int *gticket = nullptr, *wticket = nullptr;

    BnVerifier(gkrgpu_ctx& ctx, Lane& lane, const gkrgpu_circuit& circ, uint32_t n) : X(ctx), c(lane), C(circ), N(n) {}
    ~BnVerifier() {
        if (block) cudaFreeAsync(block, c.stream);
    }

    void reserve() {
        const uint64_t I0 = C.in_rows(0), maxI = 1ull << C.max_in_vars, maxO = 1ull << C.max_out_vars;
        std::vector<std::pair<void**, size_t>> parts = {
            {(void**)&raw, I0 * N * 32}, {(void**)&com, I0 * N * 32},  {(void**)&eqz, maxO * 32},
            {(void**)&eqx, maxI * 32},   {(void**)&eqy, maxI * 32},    {(void**)&sums, 32},
            {(void**)&cv, (size_t)N * 32}, {(void**)&gacc, 8 * 8},     {(void**)&gticket, 16},
            {(void**)&wacc, 3ull * N * 8 * 8}, {(void**)&wticket, 4096},
        };
        size_t o = 0, zero_from = 0;
        for (auto& p : parts) {
            if (p.first == (void**)&gacc) zero_from = o;
            o += align_up(std::max<size_t>(p.second, 16), 256);
        }
        void* base = nullptr;
        ck(cudaMallocFromPoolAsync(&base, o, X.pool, c.stream), "verifier workspace allocation");
        block = static_cast<char*>(base);
        o = 0;
        for (auto& p : parts) {
            *p.first = block + o;
            o += align_up(std::max<size_t>(p.second, 16), 256);
        }
        ck(cudaMemsetAsync(block + zero_from, 0, o - zero_from, c.stream), "cudaMemsetAsync");
        c.h_cv.ensure((size_t)N * 32 + 64, "pinned verifier results");
    }

    void eq_table(bn::Fr* out, const frh::Fr* r1, const frh::Fr* r2, const frh::Fr& f1, const frh::Fr& f2,
                  uint32_t nvars) {
        bn::EqArgsBn a;
        memset(&a, 0, sizeof(a));
        for (uint32_t t = 0; t < nvars; t++) {
            frh::store(frh::to_mont(r1[t]), a.r1[t]);
            if (r2) frh::store(frh::to_mont(r2[t]), a.r2[t]);
        }
        frh::store(frh::to_mont(f1), a.f1);
        frh::store(frh::to_mont(f2), a.f2);
        a.nvars = nvars;
        a.has_r2 = r2 ? 1u : 0u;
        c.launch(K_BN_EQ, 32.0 * (double)(1ull << nvars), [&] { return bn::launch_eq(out, a, c.stream); });
    }

    frh::Fr gate_sums(size_t li, bool mul_part, const frh::Fr* rz1, const frh::Fr* rz2, const frh::Fr& alpha,
                      const frh::Fr& beta, const frh::Fr* rx, const frh::Fr* ry) {
        const DevLayer& Ly = C.layers[li];
        const uint64_t O = 1ull << Ly.nout;
        eq_table(eqz, rz1, rz2, alpha, beta, Ly.nout);
        eq_table(eqx, rx, nullptr, frh::from_u32(1), frh::zero(), Ly.nin);
        if (mul_part) eq_table(eqy, ry, nullptr, frh::from_u32(1), frh::zero(), Ly.nin);
        const double gates = mul_part ? (double)Ly.nmul : (double)Ly.nadd;
        c.launch(K_GATE_SUMS, (mul_part ? 48.0 : 40.0) * gates + 4.0 * (O + 1) + 32.0 * O, [&] {
            return bn::launch_gate_sums(mul_part, O, mul_part ? Ly.mo_off : Ly.ao_off,
                                        mul_part ? reinterpret_cast<const uint32_t*>(Ly.mo_g)
                                                 : reinterpret_cast<const uint32_t*>(Ly.ao_g),
                                        mul_part ? Ly.mo_c : Ly.ao_c, eqz, eqx, eqy, gacc, gticket, sums, c.stream);
        });
        c.copy(c.h_cv.p, sums, 32, cudaMemcpyDeviceToHost, "gate sums readback");
        c.sync();
        return frh::load(c.h_cv.as<uint32_t>());
    }

    bool raw_pc_verify(const frh::Fr* r, const std::vector<uint32_t>& claims) {
        const uint32_t n0 = C.layers[0].nin;
        const uint64_t rows = 1ull << n0;
        eq_table(eqx, r, nullptr, frh::from_u32(1), frh::zero(), n0);
        const bn::GeoBn g = geo_bn(X, N, K_BN_WSUM);
        c.launch(K_BN_WSUM, 32.0 * N * rows + 32.0 * rows, [&] {
            return bn::launch_wsum(com, rows, eqx, g, X.cta_budget(K_BN_WSUM), bn::RedBn{wacc, wticket}, cv, c.stream);
        });
        c.copy(c.h_cv.p, cv, (size_t)N * 32, cudaMemcpyDeviceToHost, "multilinear evaluation readback");
        c.sync();
        return memcmp(c.h_cv.p, claims.data(), (size_t)N * 32) == 0;
    }

    bool run(int grinding_bits, const uint8_t* proof, uint64_t len, const uint32_t* claimed_v) {
        const uint64_t rowb = (uint64_t)N * 32, rowl = (uint64_t)N * 8;
        const uint64_t com_bytes = C.in_rows(0) * rowb;
        if (len < com_bytes + 32) return false;
        reserve();
        c.copy(raw, proof, com_bytes, cudaMemcpyHostToDevice, "commitment upload");
        c.launch(K_BN_LOAD, 64.0 * C.in_rows(0) * N,
                 [&] { return bn::launch_load(raw, com, C.in_rows(0) * N, nullptr, c.stream); });

        std::unique_ptr<uint8_t[]> tbuf(new uint8_t[len + 64]);
        Transcript t(tbuf.get(), len + 64, X.fs_hash);
        uint8_t d[32];
        fs_hash(X.fs_hash, proof, com_bytes, d);
        t.appended_prehashed(com_bytes, d);
        grind_bn254(t, grinding_bits);
        uint64_t pos = com_bytes + 32;
        bool bad = false;
        // one row of N canonical elements (from_bytes reduces each 32-byte word)
        auto next_row = [&](uint32_t* out) {
            if (pos + rowb > len) {
                bad = true;
                memset(out, 0, rowb);
                return;
            }
            for (uint32_t k = 0; k < N; k++) frh::store(frh::from_bytes(proof + pos + 32ull * k), out + 8ull * k);
            pos += rowb;
        };
        auto el = [](const std::vector<uint32_t>& v, uint64_t row, uint32_t N_, uint32_t k) {
            return frh::load(v.data() + (row * N_ + k) * 8);
        };

        const size_t L = C.layers.size();
        frh::Fr rz1[32], rz2[32], rx[32], ry[32];
        const uint32_t nz = C.layers[L - 1].nout;
        for (uint32_t i = 0; i < nz; i++) rz1[i] = t.challenge_bn254();
        frh::Fr alpha = frh::from_u32(1), beta = frh::zero();
        bool have_rz2 = false;
        std::vector<uint32_t> cv1(rowl), cv2(rowl, 0u), vx(rowl), vy(rowl), ev(3 * rowl);
        std::vector<frh::Fr> sum(N);
        for (uint32_t k = 0; k < N; k++) {
            uint8_t b[32];
            memcpy(b, claimed_v + 8ull * k, 32);
            frh::store(frh::from_bytes(b), cv1.data() + 8ull * k);
        }
        const frh::Fr inv2{{frh::kInv2[0], frh::kInv2[1], frh::kInv2[2], frh::kInv2[3]}};
        bool ok = true;

        for (int li = (int)L - 1; li >= 0; li--) {
            const uint32_t n = C.layers[li].nin;
            for (uint32_t k = 0; k < N; k++)
                sum[k] = frh::add(frh::mul(el(cv1, 0, N, k), alpha), frh::mul(el(cv2, 0, N, k), beta));
            for (uint32_t i_var = 0; i_var < 2 * n; i_var++) {
                next_row(ev.data());
                next_row(ev.data() + rowl);
                next_row(ev.data() + 2 * rowl);
                t.append(ev.data(), 3 * rowb);
                const frh::Fr r = t.challenge_bn254();
                (i_var < n ? rx[i_var] : ry[i_var - n]) = r;
                for (uint32_t k = 0; k < N; k++) {
                    // degree_2_eval (sumcheck_verifier_utils.hpp:10-18)
                    const frh::Fr c0 = el(ev, 0, N, k), v1 = el(ev, 1, N, k), v2 = el(ev, 2, N, k);
                    if (!frh::eq(frh::add(c0, v1), sum[k])) ok = false;
                    const frh::Fr c2 = frh::mul(inv2, frh::add(frh::sub(v2, frh::add(v1, v1)), c0));
                    const frh::Fr c1 = frh::sub(frh::sub(v1, c0), c2);
                    sum[k] = frh::add(c0, frh::mul(frh::add(frh::mul(c2, r), c1), r));
                }
                if (i_var == n - 1) {
                    next_row(vx.data());
                    t.append(vx.data(), rowb);
                    const frh::Fr a = gate_sums((size_t)li, false, rz1, have_rz2 ? rz2 : nullptr, alpha, beta, rx, ry);
                    for (uint32_t k = 0; k < N; k++) sum[k] = frh::sub(sum[k], frh::mul(el(vx, 0, N, k), a));
                }
            }
            next_row(vy.data());
            t.append(vy.data(), rowb);
            const frh::Fr m = gate_sums((size_t)li, true, rz1, have_rz2 ? rz2 : nullptr, alpha, beta, rx, ry);
            for (uint32_t k = 0; k < N; k++)
                if (!frh::eq(sum[k], frh::mul(frh::mul(el(vx, 0, N, k), el(vy, 0, N, k)), m))) ok = false;
            alpha = t.challenge_bn254();
            beta = t.challenge_bn254();
            for (uint32_t i = 0; i < n; i++) {
                rz1[i] = rx[i];
                rz2[i] = ry[i];
            }
            have_rz2 = true;
            cv1 = vx;
            cv2 = vy;
        }
        if (!raw_pc_verify(rz1, cv1)) ok = false;
        if (!raw_pc_verify(rz2, cv2)) ok = false;
        c.resolve_events();
        return ok && !bad;
    }
};
