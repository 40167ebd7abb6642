// BN254 prove path (Config::field_type = BN254, include/configuration/config.hpp:12-16,53-65):
// the same gkr_prove flow as the M31 Prover in prover.cu with 256-bit elements and one
// repetition (ceil((100 - grinding_bits) / 254) = 1).  Part of prover.cu's translation unit:
// it is included there, inside its anonymous namespace, after Lane, gkrgpu_ctx, the
// circuit and the M31 Prover, whose helpers it shares.
//
// Device tables hold Montgomery forms (bn254.cuh).  The host side keeps challenges and the
// last folds canonical (fr_host.hpp) and converts what it sends to the device.
#pragma once

// Row tile of a BN254 kernel kind: one thread per lane, tpr lanes per row slice (the largest
// divisor of N not above the kind's threads_per_row), 256 threads per CTA.
bn::GeoBn geo_bn(const gkrgpu_ctx& X, uint32_t N, int kid) {
    uint32_t tpr = std::min<uint32_t>(N, std::min<uint32_t>(X.tiles[kid].tpr, bn::kBlock));
    while (tpr > 1 && N % tpr) tpr--;
    return bn::GeoBn{N, tpr, bn::kBlock / tpr};
}

// All device tables of one BN254 proof, carved from one pool block.
struct BnWorkspace {
    uint32_t* vals = nullptr;  // every layer's values (Montgomery), layer 0's input first
    uint32_t* stage = nullptr;  // canonical input rows as uploaded (the hg table's space when proving)
    uint32_t *hg0 = nullptr, *hgA = nullptr, *fA = nullptr, *fB = nullptr;
    bn::Fr *sb[2] = {}, *eqc = nullptr, *eqrx = nullptr, *a = nullptr, *w = nullptr;
    uint32_t *vx = nullptr, *cv = nullptr;
    uint32_t* ev_dev[2] = {};  // device copies of the round evaluations (round k writes ev_dev[k & 1])
    unsigned long long* acc = nullptr;
    unsigned int* ticket = nullptr;
    unsigned int* flag = nullptr;
    size_t zero_off = 0, zero_bytes = 0, total = 0;

    void plan(char* base, const gkrgpu_circuit& C, uint32_t N, bool sumcheck) {
        size_t o = 0;
        auto take = [&](size_t bytes) -> char* {
            char* p = base ? base + o : nullptr;
            o += align_up(std::max<size_t>(bytes, 16), 256);
            return p;
        };
        const uint64_t rowb = (uint64_t)N * 32;
        const uint64_t maxI = 1ull << C.max_in_vars, maxO = 1ull << C.max_out_vars;
        vals = (uint32_t*)take(C.value_rows() * rowb);
        if (sumcheck) {
            hg0 = (uint32_t*)take(maxI * rowb);
            hgA = (uint32_t*)take(std::max<uint64_t>(maxI / 2, 1) * rowb);
            fA = (uint32_t*)take(std::max<uint64_t>(maxI / 2, 1) * rowb);
            fB = (uint32_t*)take(std::max<uint64_t>(maxI / 4, 1) * rowb);
            sb[0] = (bn::Fr*)take(maxI * 32);
            sb[1] = (bn::Fr*)take(maxI * 32);
            eqrx = (bn::Fr*)take(maxI * 32);
            a = (bn::Fr*)take(maxI * 32);
            w = (bn::Fr*)take(std::max<uint64_t>(C.max_mul, 1) * 32);
            stage = hg0;
        } else {
            stage = (uint32_t*)take(C.in_rows(0) * rowb);
        }
        eqc = (bn::Fr*)take(maxO * 32);
        vx = (uint32_t*)take(rowb);
        cv = (uint32_t*)take(rowb);
        ev_dev[0] = (uint32_t*)take(3 * rowb);
        ev_dev[1] = (uint32_t*)take(3 * rowb);
        zero_off = o;
        acc = (unsigned long long*)take(3ull * N * 8 * 8);
        ticket = (unsigned int*)take(4096);
        flag = (unsigned int*)take(16);
        zero_bytes = o - zero_off;
        total = o;
    }
};

uint64_t workspace_bytes_bn(const gkrgpu_circuit& C, uint32_t N, bool sumcheck) {
    BnWorkspace w;
    w.plan(nullptr, C, N, sumcheck);
    return w.total;
}

struct BnProver {
    gkrgpu_ctx& X;
    Lane& c;
    const gkrgpu_circuit& C;
    uint32_t N;
    bn::GeoBn gk[K_NUM_KERNELS];
    uint32_t ctas[K_NUM_KERNELS];
    BnWorkspace ws;
    char* block = nullptr;
    std::vector<uint32_t*> vals;  // vals[l]: input of layer l; vals[L]: output of the last layer
    // the layer's sum is alpha cv1 + beta cv2 (canonical, N x 8 words each): the claimed
    // values and zero for the output layer, then the previous layer's vx and vy
    std::vector<uint32_t> cv1, cv2;

    BnProver(gkrgpu_ctx& ctx, Lane& lane, const gkrgpu_circuit& circ, uint32_t n) : X(ctx), c(lane), C(circ), N(n) {
        for (int k = 0; k < K_NUM_KERNELS; k++) {
            gk[k] = geo_bn(ctx, n, k);
            ctas[k] = ctx.cta_budget(k);
        }
    }
    ~BnProver() {
        if (block) cudaFreeAsync(block, c.stream);
    }

    uint64_t rowb() const { return (uint64_t)N * 32; }
    bn::RedBn red() const { return bn::RedBn{ws.acc, ws.ticket}; }
    // Round k of a phase publishes to the mapped staging buffer and to ws.ev_dev[k & 1], and
    // takes its claim from round k - 1's copy.
    bn::RedBn red_mapped(uint32_t k) const {
        return bn::RedBn{ws.acc, ws.ticket, c.done_d(), ws.ev_dev[(k + 1) & 1], ws.ev_dev[k & 1]};
    }
    uint32_t groups(int kid) const { return N / gk[kid].tpr; }
    // The lane's mapped extra area (words): rows 0..1 of the last table (16N), the claimed
    // values (8N), vx in Montgomery form (8N), the input check flag, and from word 32N + 64
    // the claims of phase one's round 0 (8N).  Small transfers go through it by kernels,
    // never queueing on the copy engine behind another proof's bulk copies.
    uint32_t* mapped(bool dev, uint64_t word) const {
        return reinterpret_cast<uint32_t*>(dev ? c.extra_d() : c.extra_h()) + word;
    }
    volatile uint32_t* flag_h() const { return mapped(false, 32ull * N); }
    uint32_t stage(uint32_t* dst, const uint32_t* src, uint64_t words, unsigned int* done) {
        uint32_t incs = 0;
        const uint32_t* srcs[1] = {src};
        c.launch(K_STAGE, 8.0 * words, [&] {
            cudaError_t e;
            incs = launch_stage_words(dst, srcs, 1, words, done, c.stream, &e);
            return e;
        });
        return done ? incs : 0;
    }

    void reserve(bool sumcheck) {
        ws.plan(nullptr, C, N, sumcheck);
        void* p = nullptr;
        ck(cudaMallocFromPoolAsync(&p, ws.total, X.pool, c.stream), "workspace allocation");
        block = static_cast<char*>(p);
        ws.plan(block, C, N, sumcheck);
        ck(cudaMemsetAsync(block + ws.zero_off, 0, ws.zero_bytes, c.stream), "cudaMemsetAsync");
        c.ensure_mapped(3 * rowb(), (40ull * N + 64) * 4);
        c.resync_done();
    }

    void layout_values() {
        const size_t L = C.layers.size();
        vals.assign(L + 1, nullptr);
        uint64_t off = 0;
        for (size_t l = 0; l <= L; l++) {
            vals[l] = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(ws.vals) + off * rowb());
            off += (l < L) ? C.in_rows(l) : C.out_rows(L - 1);
        }
    }

    // Input (canonical, from the host or the device) -> Montgomery layer-0 values, with the
    // canonical check read back for require_canonical.
    void load_input(const uint32_t* h_input, const uint32_t* d_input) {
        const uint64_t n = C.in_rows(0) * N;
        const uint32_t* src = d_input;
        if (h_input && !d_input) {
            c.copy(ws.stage, h_input, n * 32, cudaMemcpyHostToDevice, "input upload");
            src = ws.stage;
        }
        *flag_h() = 0u;
        std::atomic_thread_fence(std::memory_order_seq_cst);
        c.launch(K_BN_LOAD, 64.0 * n,
                 [&] { return bn::launch_load(src, vals[0], n, mapped(true, 32ull * N), c.stream); });
    }
    void require_canonical() {
        if (*flag_h()) fail(GKRGPU_ERR_INVALID, "input contains a value >= r (the BN254 modulus)");
    }

    void evaluate() {
        for (size_t l = 0; l < C.layers.size(); l++) {
            const DevLayer& Ly = C.layers[l];
            const uint64_t O = 1ull << Ly.nout;
            const double b = 32.0 * N * (2.0 * Ly.nmul + Ly.nadd + O) + 48.0 * Ly.nmul + 40.0 * Ly.nadd + 8.0 * (O + 1);
            c.launch(K_BN_EVALUATE, b, [&] {
                return bn::launch_evaluate(vals[l], vals[l + 1], O, Ly.mo_off, Ly.mo_g, Ly.mo_c, Ly.ao_off, Ly.ao_g,
                                           Ly.ao_c, gk[K_BN_EVALUATE], ctas[K_BN_EVALUATE], c.stream);
            });
        }
    }

    // Waits for the round's 3 evaluation rows; optionally copies rows 0..1 of `rows_from`.
    void fetch(uint32_t groups, const uint32_t* rows_from) {
        const uint32_t more = rows_from ? stage(mapped(true, 0), rows_from, 16ull * N, c.done_d()) : 0u;
        c.wait_done(groups + more);
    }

    // One round's transcript step (sumcheck.hpp:74-96 with R = 1): append the 3 rows, take
    // the challenge; in the last round fold rows 0..1 by it into vx / vy (Montgomery copy in
    // `last_mont`, canonical in `last_canon`, appended at once when `append_last`).
    void transcript_round(Transcript& t, frh::Fr* rch, uint32_t k, bool last, bool append_last, uint32_t* last_mont,
                          uint32_t* last_canon) {
        t.append(c.evals_h(), 3 * rowb());
        rch[k] = t.challenge_bn254();
        if (!last) return;
        const frh::Fr rm = frh::to_mont(rch[k]);
        const uint32_t* f0 = mapped(false, 0);
        const uint32_t* f1 = f0 + (size_t)N * 8;
        for (uint32_t i = 0; i < N; i++) {
            const frh::Fr m = frh::fold_mont(frh::load(f0 + 8 * i), frh::load(f1 + 8 * i), rm);
            frh::store(m, last_mont + 8 * i);
            frh::store(frh::from_mont(m), last_canon + 8 * i);
        }
        if (append_last) t.append(last_canon, rowb());
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

    void sumcheck_layer(Transcript& t, size_t li, const frh::Fr* rz1, const frh::Fr* rz2, const frh::Fr& alpha,
                        const frh::Fr& beta, frh::Fr* rx, frh::Fr* ry) {
        const DevLayer& Ly = C.layers[li];
        const uint32_t n = Ly.nin, m = Ly.nout;
        const uint64_t I = 1ull << n;
        const double rb = (double)rowb();
        uint32_t* v = vals[li];
        uint32_t* vx_m = mapped(false, 24ull * N);
        std::vector<uint32_t> vx_c((size_t)N * 8), vy_m((size_t)N * 8), vy_c((size_t)N * 8);

        // phase one: eqc = alpha eq(rz1) + beta eq(rz2), gate weights, hg + round 0
        eq_table(ws.eqc, rz1, rz2, alpha, beta, m);
        // round 0's claims, alpha v(rz1) + beta v(rz2) per copy (sumcheck.hpp:129-132)
        {
            uint32_t* cl = mapped(false, 32ull * N + 64);
            for (uint32_t i = 0; i < N; i++)
                frh::store(frh::add(frh::mul(alpha, frh::load(cv1.data() + 8 * i)),
                                    frh::mul(beta, frh::load(cv2.data() + 8 * i))),
                           cl + 8 * i);
            std::atomic_thread_fence(std::memory_order_seq_cst);
        }
        c.launch(K_BN_WEIGHTS, 80.0 * Ly.nmul + 72.0 * Ly.nadd + 40.0 * I, [&] {
            return bn::launch_weights(I, Ly.nmul, ws.eqc, Ly.mx_g, Ly.mx_c, Ly.ax_off, Ly.ax_g, Ly.ax_c, ws.a, ws.w,
                                      c.stream);
        });
        c.launch(K_BN_HG_ROUND0, rb * (2.0 * I + Ly.nmul) + 52.0 * Ly.nmul + 36.0 * I, [&] {
            return bn::launch_hg_round0(v, I, Ly.mx_off, Ly.mx_g, ws.a, ws.w, ws.hg0, gk[K_BN_HG_ROUND0],
                                        ctas[K_BN_HG_ROUND0], red_mapped(0), mapped(true, 32ull * N + 64),
                                        c.evals_d(), c.stream);
        });
        fetch(groups(K_BN_HG_ROUND0), n == 1 ? v : nullptr);
        transcript_round(t, rx, 0, n == 1, true, vx_m, vx_c.data());

        const uint32_t* cur_f = v;
        const uint32_t* cur_h = ws.hg0;
        for (uint32_t k = 1; k < n; k++) {
            bn::RoundPtrsBn p;
            memset(&p, 0, sizeof(p));
            p.fsrc = cur_f;
            p.hsrc = cur_h;
            p.fdst = (k & 1) ? ws.fA : ws.fB;
            p.hdst = (k & 1) ? ws.hgA : ws.hg0;
            frh::store(frh::to_mont(rx[k - 1]), p.r);
            const uint64_t npairs = I >> (k + 1);
            c.launch(K_BN_ROUND_LANE, rb * 6.0 * npairs, [&] {
                return bn::launch_round(true, true, p, npairs, nullptr, gk[K_BN_ROUND_LANE], ctas[K_BN_ROUND_LANE],
                                        red_mapped(k), c.evals_d(), c.stream);
            });
            const bool last = (k == n - 1);
            fetch(groups(K_BN_ROUND_LANE), last ? p.fdst : nullptr);
            transcript_round(t, rx, k, last, true, vx_m, vx_c.data());
            cur_f = p.fdst;
            cur_h = p.hdst;
        }

        // phase two: h(y) = vx * s(y)
        const frh::Fr one = frh::from_u32(1), zero = frh::zero();
        eq_table(ws.eqrx, rx, nullptr, one, zero, n);
        c.launch(K_BN_S_BUILD, 16.0 * Ly.nmul + 4.0 * I + 32.0 * I + 96.0 * Ly.nmul, [&] {
            return bn::launch_s_build(I, Ly.my_off, Ly.my_g, Ly.my_c, ws.eqc, ws.eqrx, ws.sb[0], c.stream);
        });
        stage(ws.vx, mapped(true, 24ull * N), 8ull * N, nullptr);
        {
            bn::RoundPtrsBn p;
            memset(&p, 0, sizeof(p));
            p.fsrc = v;
            p.hsrc = reinterpret_cast<const uint32_t*>(ws.sb[0]);
            const uint64_t npairs = I >> 1;
            c.launch(K_BN_ROUND_SCALAR, rb * 2.0 * npairs + 64.0 * npairs, [&] {
                return bn::launch_round(false, false, p, npairs, ws.vx, gk[K_BN_ROUND_SCALAR], ctas[K_BN_ROUND_SCALAR],
                                        red_mapped(0), c.evals_d(), c.stream);
            });
            fetch(groups(K_BN_ROUND_SCALAR), n == 1 ? v : nullptr);
            transcript_round(t, ry, 0, n == 1, false, vy_m.data(), vy_c.data());
        }
        cur_f = v;
        for (uint32_t k = 1; k < n; k++) {
            bn::RoundPtrsBn p;
            memset(&p, 0, sizeof(p));
            p.fsrc = cur_f;
            p.fdst = (k & 1) ? ws.fA : ws.fB;
            p.hsrc = reinterpret_cast<const uint32_t*>(ws.sb[(k - 1) & 1]);
            p.hdst = reinterpret_cast<uint32_t*>(ws.sb[k & 1]);
            frh::store(frh::to_mont(ry[k - 1]), p.r);
            const uint64_t npairs = I >> (k + 1);
            c.launch(K_BN_ROUND_SCALAR, rb * 6.0 * npairs + 192.0 * npairs, [&] {
                return bn::launch_round(false, true, p, npairs, ws.vx, gk[K_BN_ROUND_SCALAR], ctas[K_BN_ROUND_SCALAR],
                                        red_mapped(k), c.evals_d(), c.stream);
            });
            const bool last = (k == n - 1);
            fetch(groups(K_BN_ROUND_SCALAR), last ? p.fdst : nullptr);
            transcript_round(t, ry, k, last, false, vy_m.data(), vy_c.data());
            cur_f = p.fdst;
        }
        t.append(vy_c.data(), rowb());
        // the next layer's sum is alpha vx + beta vy (gkr.hpp:113-119)
        cv1.swap(vx_c);
        cv2.swap(vy_c);
    }

    void device_front(const uint32_t* h_input, const uint32_t* d_input) {
        reserve(true);
        layout_values();
        load_input(h_input, d_input);
        evaluate();
    }

    // gkr_prove (gkr.hpp:24-73) from the transcript state left by the host stage.
    void device_back(const TranscriptState& ts, uint8_t* proof_out, uint32_t* claimed_v) {
        const size_t L = C.layers.size();
        Transcript t(proof_out, ts);
        frh::Fr rz1[32], rz2[32], rx[32], ry[32];
        const uint32_t nz = C.layers[L - 1].nout;
        for (uint32_t i = 0; i < nz; i++) rz1[i] = t.challenge_bn254();
        frh::Fr alpha = frh::from_u32(1), beta = frh::zero();
        bool have_rz2 = false;

        eq_table(ws.eqc, rz1, nullptr, alpha, beta, nz);
        const uint64_t OL = C.out_rows(L - 1);
        c.launch(K_BN_WSUM, 32.0 * N * OL + 32.0 * OL, [&] {
            return bn::launch_wsum(vals[L], OL, ws.eqc, gk[K_BN_WSUM], ctas[K_BN_WSUM], red(), mapped(true, 16ull * N),
                                   c.stream);
        });
        c.sync();
        require_canonical();
        memcpy(claimed_v, mapped(false, 16ull * N), rowb());
        cv1.assign(claimed_v, claimed_v + (size_t)N * 8);
        cv2.assign((size_t)N * 8, 0u);

        for (int li = (int)L - 1; li >= 0; li--) {
            sumcheck_layer(t, (size_t)li, rz1, have_rz2 ? rz2 : nullptr, alpha, beta, rx, ry);
            alpha = t.challenge_bn254();
            beta = t.challenge_bn254();
            const uint32_t n = C.layers[li].nin;
            for (uint32_t i = 0; i < n; i++) {
                rz1[i] = rx[i];
                rz2[i] = ry[i];
            }
            have_rz2 = true;
        }
        c.sync();
        c.resolve_events();
    }

    void evaluate_only(const uint32_t* h_input, uint32_t* out, bool all_layers) {
        reserve(false);
        layout_values();
        load_input(h_input, nullptr);
        evaluate();
        c.sync();
        require_canonical();
        const size_t L = C.layers.size();
        uint32_t* from = all_layers ? vals[0] : vals[L];
        const uint64_t rows = all_layers ? C.value_rows() : C.out_rows(L - 1);
        c.launch(K_BN_UNLOAD, 64.0 * rows * N, [&] { return bn::launch_unload(from, rows * N, c.stream); });
        c.copy(out, from, rows * rowb(), cudaMemcpyDeviceToHost, "values readback");
        c.sync();
        c.resolve_events();
    }
};
