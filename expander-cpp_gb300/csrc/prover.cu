// Host orchestration of the GB300 GKR prover and the C ABI (include/gkrgpu.h).
//
// Prove flow, following Prover::prove (include/LinearGKR/LinearGKR.hpp:58-90) and
// gkr_prove (include/LinearGKR/gkr.hpp:24-73):
//   device : input -> Circuit::evaluate of every layer, kept resident for the sumcheck
//   host   : RAW commitment bytes -> transcript, grinding, output challenges rz1
//   device : claimed_v = eval_multilinear(output, rz1_j) for every repetition j
//   per layer, top down, per sumcheck_prove_gkr_layer (include/LinearGKR/sumcheck.hpp:52-111):
//     device : eq tables, gate weights, hg build fused with round 0
//     rounds : device fold+reduce for all repetitions at once -> 3R rows to the host ->
//              host appends them and derives the R challenges in the reference's order
//     phase 2: s(y) table, rounds over the layer input with h = v(rx) * s
//   alpha, beta challenges between layers.
// The host does only transcript work: appending bytes, SHA-256, and the last 2->1 fold of
// each phase's table (vx, vy: 2 rows x N lanes), whose result must enter the transcript
// before the next repetition's challenge.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gkrgpu.h"
#include "kernels.cuh"
#include "m31.cuh"
#include "sha256.hpp"
#include "transcript.hpp"

using namespace gkrgpu;

namespace {

thread_local std::string g_last_error;

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] void fail(int code, const char* fmt, ...) {
    char b[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(b, sizeof(b), fmt, ap);
    va_end(ap);
    throw Error(code, b);
}

void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        const int code = (e == cudaErrorMemoryAllocation) ? GKRGPU_ERR_NOMEM : GKRGPU_ERR_CUDA;
        fail(code, "%s: %s", what, cudaGetErrorString(e));
    }
}

template <class F>
int guarded(F&& f) {
    try {
        f();
        return GKRGPU_OK;
    } catch (const Error& e) {
        g_last_error = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        g_last_error = "host allocation failed";
        return GKRGPU_ERR_NOMEM;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return GKRGPU_ERR_STATE;
    }
}

int reps_for(int grinding_bits) {
    // include/configuration/config.hpp:61-65: ceil((100 - grinding_bits) / 31)
    const int s = 100 - grinding_bits;
    return s / 31 + (s % 31 != 0);
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    bool pinned = false;
    void release() {
        if (p) {
            if (pinned) cudaFreeHost(p);
            else cudaFree(p);
        }
        p = nullptr;
        cap = 0;
    }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
    void ensure(size_t bytes, const char* what) {
        bytes = std::max<size_t>(align_up(bytes, 256), 256);
        if (bytes <= cap) return;
        release();
        cudaError_t e = pinned ? cudaMallocHost(&p, bytes) : cudaMalloc(&p, bytes);
        if (e != cudaSuccess) {
            p = nullptr;
            cudaGetLastError();
            fail(GKRGPU_ERR_NOMEM, "allocation of %zu bytes for %s failed: %s", bytes, what, cudaGetErrorString(e));
        }
        cap = bytes;
    }
};

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) ck(cudaSetDevice(dev), "cudaSetDevice");
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

}  // namespace

// ------------------------------------------------------------------ circuit on the device
struct DevLayer {
    uint32_t nin = 0, nout = 0;
    uint64_t nmul = 0, nadd = 0;
    // evaluate: gates grouped by output o
    uint32_t* mo_off = nullptr;  // O+1
    uint4* mo_g = nullptr;       // (i0, i1, c, 0)
    uint32_t* ao_off = nullptr;  // O+1
    uint2* ao_g = nullptr;       // (i0, c)
    // phase one: gates grouped by x = i0
    uint32_t* mx_off = nullptr;  // I+1
    uint4* mx_g = nullptr;       // (y, z, c, 0)
    uint32_t* ax_off = nullptr;  // I+1
    uint2* ax_g = nullptr;       // (z, c)
    // phase two: mul gates grouped by y = i1
    uint32_t* my_off = nullptr;  // I+1
    uint4* my_g = nullptr;       // (x, z, c, 0)
    void* block = nullptr;
};

struct gkrgpu_circuit {
    int device = 0;
    std::vector<DevLayer> layers;
    uint32_t max_in_vars = 0, max_out_vars = 0;
    uint64_t max_mul = 0;
    ~gkrgpu_circuit() {
        for (auto& l : layers)
            if (l.block) cudaFree(l.block);
    }
    uint64_t in_rows(size_t l) const { return 1ull << layers[l].nin; }
    uint64_t out_rows(size_t l) const { return 1ull << layers[l].nout; }
    uint64_t value_rows() const {
        uint64_t r = 0;
        for (size_t l = 0; l < layers.size(); l++) r += in_rows(l);
        return r + out_rows(layers.size() - 1);
    }
};

// ------------------------------------------------------------------ jobs
// One queued Prover::prove (gkrgpu_prove_submit).  The host stage fills `ts`; the device
// stage resumes from it.  The submitting thread waits on `cv` for done && host_done.
struct gkrgpu_job {
    const gkrgpu_circuit* circuit = nullptr;
    uint32_t N = 0;
    int grinding = 10, R = 3, marker = -1;
    const uint32_t* h_input = nullptr;
    const uint32_t* d_input = nullptr;
    uint8_t* proof_out = nullptr;
    uint64_t proof_len = 0;
    uint32_t* claimed_v = nullptr;

    TranscriptState ts;
    bool host_done = false, done = false;
    int host_rc = GKRGPU_OK, rc = GKRGPU_OK;
    std::string host_err, err;
    std::mutex m;
    std::condition_variable cv;
};

// ------------------------------------------------------------------ context
struct gkrgpu_ctx {
    int device = 0;
    int sm_count = 152;
    cudaStream_t stream = nullptr;
    uint32_t tpr_max = 32, block = 256, ctas = 0;

    // job pipeline: one device-stage worker, host-stage workers
    std::mutex qm;
    std::condition_variable qcv;
    std::deque<gkrgpu_job*> host_q, gpu_q;
    std::vector<std::thread> workers;
    bool stopping = false, gpu_busy = false;
    int host_workers = 2;
    void start_workers();
    void shutdown() {
        {
            std::lock_guard<std::mutex> lk(qm);
            stopping = true;
        }
        qcv.notify_all();
        for (auto& t : workers) t.join();
        workers.clear();
    }
    // Waits until no device stage is queued or running.
    void drain() {
        std::unique_lock<std::mutex> lk(qm);
        qcv.wait(lk, [&] { return gpu_q.empty() && !gpu_busy; });
    }

    DevBuf vals, eqc, eqrx, a4, w4, acc, ticket, evals, vx, cv, flag;
    DevBuf fA[3], fB[3], hg0[3], hgA[3], sb[2];
    DevBuf h_evals, h_rows, h_vx, h_cv, h_flag;  // pinned

    // launch accounting
    bool timing = false;
    std::atomic<uint64_t> h2d_bytes{0}, d2h_bytes{0};
    cudaEvent_t markers[64] = {};
    // Totals (read by gkrgpu_kernel_stats under stats_m); each job's launches accumulate
    // in job_* and are folded in when the job ends, so snapshots fall on job boundaries.
    std::mutex stats_m;
    uint64_t launches[K_NUM_KERNELS] = {};
    double ms[K_NUM_KERNELS] = {};
    double bytes[K_NUM_KERNELS] = {};
    uint64_t job_launches[K_NUM_KERNELS] = {};
    double job_bytes[K_NUM_KERNELS] = {};
    struct Rec {
        int kid;
        size_t e0, e1;
    };
    std::vector<cudaEvent_t> events;
    size_t ev_used = 0;
    std::vector<Rec> recs;

    gkrgpu_ctx() {
        for (DevBuf* b : {&h_evals, &h_rows, &h_vx, &h_cv, &h_flag}) b->pinned = true;
    }
    ~gkrgpu_ctx() {
        DeviceGuard g(device);
        for (DevBuf* b : {&vals, &eqc, &eqrx, &a4, &w4, &acc, &ticket, &evals, &vx, &cv, &flag, &h_evals, &h_rows,
                          &h_vx, &h_cv, &h_flag})
            b->release();
        for (int j = 0; j < 3; j++) {
            fA[j].release(); fB[j].release(); hg0[j].release(); hgA[j].release();
        }
        sb[0].release(); sb[1].release();
        for (auto e : events) cudaEventDestroy(e);
        for (auto e : markers)
            if (e) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
    }

    size_t next_event() {
        if (ev_used == events.size()) {
            cudaEvent_t e;
            ck(cudaEventCreate(&e), "cudaEventCreate");
            events.push_back(e);
        }
        return ev_used++;
    }
    // Brackets one launch: f() enqueues the kernel on `stream`.
    template <class F>
    void launch(int kid, double algo_bytes, F&& f) {
        size_t e0 = 0;
        if (timing) {
            e0 = next_event();
            ck(cudaEventRecord(events[e0], stream), "cudaEventRecord");
        }
        ck(f(), kKernelNames[kid]);
        job_launches[kid]++;
        job_bytes[kid] += algo_bytes;
        if (timing) {
            const size_t e1 = next_event();
            ck(cudaEventRecord(events[e1], stream), "cudaEventRecord");
            recs.push_back({kid, e0, e1});
        }
    }
    // Folds the finished job's launch counts, bytes and event times into the totals; the
    // stream must be idle.
    void resolve_events() {
        double t_ms[K_NUM_KERNELS] = {};
        for (const Rec& r : recs) {
            float t = 0.f;
            ck(cudaEventElapsedTime(&t, events[r.e0], events[r.e1]), "cudaEventElapsedTime");
            t_ms[r.kid] += t;
        }
        recs.clear();
        ev_used = 0;
        std::lock_guard<std::mutex> lk(stats_m);
        for (int k = 0; k < K_NUM_KERNELS; k++) {
            launches[k] += job_launches[k];
            bytes[k] += job_bytes[k];
            ms[k] += t_ms[k];
            job_launches[k] = 0;
            job_bytes[k] = 0;
        }
    }
    void discard_job_stats() {
        recs.clear();
        ev_used = 0;
        for (int k = 0; k < K_NUM_KERNELS; k++) {
            job_launches[k] = 0;
            job_bytes[k] = 0;
        }
    }
    void sync() { ck(cudaStreamSynchronize(stream), "cudaStreamSynchronize"); }
    // Stream-ordered copy, counted in the transfer statistics.
    void copy(void* dst, const void* src, size_t n, cudaMemcpyKind kind, const char* what) {
        ck(cudaMemcpyAsync(dst, src, n, kind, stream), what);
        if (kind == cudaMemcpyHostToDevice) h2d_bytes += n;
        if (kind == cudaMemcpyDeviceToHost) d2h_bytes += n;
    }

    Geo geo(uint32_t N) const {
        const uint32_t Q = N / 4;
        uint32_t tpr = Q;
        if (tpr > tpr_max) {
            tpr = tpr_max;
            while (tpr > 1 && Q % tpr) tpr--;
        }
        Geo g;
        g.N = N;
        g.tpr = tpr;
        g.rps = block / tpr;
        return g;
    }
    uint32_t cta_budget() const { return ctas ? ctas : (uint32_t)sm_count * 4; }
    RedScratch red() const { return RedScratch{acc.as<unsigned long long>(), ticket.as<unsigned int>()}; }
};

namespace {

// ------------------------------------------------------------------ circuit upload
void csr(uint64_t nkeys, uint64_t n, const std::vector<uint32_t>& keys, std::vector<uint32_t>& off,
         std::vector<uint32_t>& order) {
    off.assign(nkeys + 1, 0);
    for (uint64_t i = 0; i < n; i++) off[keys[i] + 1]++;
    for (uint64_t k = 0; k < nkeys; k++) off[k + 1] += off[k];
    order.resize(n);
    std::vector<uint32_t> pos(off.begin(), off.end() - 1);
    for (uint64_t i = 0; i < n; i++) order[pos[keys[i]]++] = (uint32_t)i;
}

DevLayer upload_layer(const gkrgpu_layer_desc& d) {
    const uint64_t I = 1ull << d.nb_input_vars, O = 1ull << d.nb_output_vars;
    const uint64_t Gm = d.n_mul, Ga = d.n_add;
    std::vector<uint32_t> keys, off_mo, off_ao, off_mx, off_ax, off_my, ord;
    std::vector<uint4> mo(Gm), mx(Gm), my(Gm);
    std::vector<uint2> ao(Ga), ax(Ga);

    keys.resize(Gm);
    for (uint64_t i = 0; i < Gm; i++) keys[i] = d.mul[i].o_id;
    csr(O, Gm, keys, off_mo, ord);
    for (uint64_t k = 0; k < Gm; k++) {
        const auto& g = d.mul[ord[k]];
        mo[k] = make_uint4(g.i0, g.i1, g.coef, 0);
    }
    for (uint64_t i = 0; i < Gm; i++) keys[i] = d.mul[i].i0;
    csr(I, Gm, keys, off_mx, ord);
    for (uint64_t k = 0; k < Gm; k++) {
        const auto& g = d.mul[ord[k]];
        mx[k] = make_uint4(g.i1, g.o_id, g.coef, 0);
    }
    for (uint64_t i = 0; i < Gm; i++) keys[i] = d.mul[i].i1;
    csr(I, Gm, keys, off_my, ord);
    for (uint64_t k = 0; k < Gm; k++) {
        const auto& g = d.mul[ord[k]];
        my[k] = make_uint4(g.i0, g.o_id, g.coef, 0);
    }
    keys.resize(Ga);
    for (uint64_t i = 0; i < Ga; i++) keys[i] = d.add[i].o_id;
    csr(O, Ga, keys, off_ao, ord);
    for (uint64_t k = 0; k < Ga; k++) {
        const auto& g = d.add[ord[k]];
        ao[k] = make_uint2(g.i0, g.coef);
    }
    for (uint64_t i = 0; i < Ga; i++) keys[i] = d.add[i].i0;
    csr(I, Ga, keys, off_ax, ord);
    for (uint64_t k = 0; k < Ga; k++) {
        const auto& g = d.add[ord[k]];
        ax[k] = make_uint2(g.o_id, g.coef);
    }

    struct Part {
        const void* src;
        size_t bytes;
        void** dst;
    };
    DevLayer L;
    L.nin = d.nb_input_vars;
    L.nout = d.nb_output_vars;
    L.nmul = Gm;
    L.nadd = Ga;
    std::vector<Part> parts = {
        {off_mo.data(), off_mo.size() * 4, (void**)&L.mo_off}, {mo.data(), Gm * 16, (void**)&L.mo_g},
        {off_ao.data(), off_ao.size() * 4, (void**)&L.ao_off}, {ao.data(), Ga * 8, (void**)&L.ao_g},
        {off_mx.data(), off_mx.size() * 4, (void**)&L.mx_off}, {mx.data(), Gm * 16, (void**)&L.mx_g},
        {off_ax.data(), off_ax.size() * 4, (void**)&L.ax_off}, {ax.data(), Ga * 8, (void**)&L.ax_g},
        {off_my.data(), off_my.size() * 4, (void**)&L.my_off}, {my.data(), Gm * 16, (void**)&L.my_g},
    };
    size_t total = 0;
    for (auto& p : parts) total += align_up(std::max<size_t>(p.bytes, 16), 256);
    cudaError_t e = cudaMalloc(&L.block, total);
    if (e != cudaSuccess) {
        cudaGetLastError();
        fail(GKRGPU_ERR_NOMEM, "circuit upload: cudaMalloc(%zu) failed", total);
    }
    size_t o = 0;
    for (auto& p : parts) {
        *p.dst = (char*)L.block + o;
        if (p.bytes) {
            e = cudaMemcpy(*p.dst, p.src, p.bytes, cudaMemcpyHostToDevice);
            if (e != cudaSuccess) {
                cudaFree(L.block);
                fail(GKRGPU_ERR_CUDA, "circuit upload: %s", cudaGetErrorString(e));
            }
        }
        o += align_up(std::max<size_t>(p.bytes, 16), 256);
    }
    return L;
}

void validate_layers(const gkrgpu_layer_desc* layers, int n) {
    if (!layers || n <= 0) fail(GKRGPU_ERR_INVALID, "circuit needs at least one layer");
    for (int l = 0; l < n; l++) {
        const auto& d = layers[l];
        if (d.nb_input_vars < 1 || d.nb_input_vars > 30 || d.nb_output_vars > 30)
            fail(GKRGPU_ERR_INVALID, "layer %d: nb_input_vars must be in [1, 30] and nb_output_vars in [0, 30]", l);
        if (l + 1 < n && d.nb_output_vars != layers[l + 1].nb_input_vars)
            fail(GKRGPU_ERR_INVALID, "layer %d: nb_output_vars %u != nb_input_vars %u of layer %d", l, d.nb_output_vars,
                 layers[l + 1].nb_input_vars, l + 1);
        if ((d.n_mul && !d.mul) || (d.n_add && !d.add)) fail(GKRGPU_ERR_INVALID, "layer %d: null gate list", l);
        if (d.n_mul >= (1ull << 32) || d.n_add >= (1ull << 32)) fail(GKRGPU_ERR_INVALID, "layer %d: too many gates", l);
        const uint64_t I = 1ull << d.nb_input_vars, O = 1ull << d.nb_output_vars;
        for (uint64_t g = 0; g < d.n_mul; g++) {
            const auto& m = d.mul[g];
            if (m.o_id >= O || m.i0 >= I || m.i1 >= I || m.coef >= m31::P)
                fail(GKRGPU_ERR_INVALID, "layer %d mul gate %llu: id or coefficient out of range", l, (unsigned long long)g);
        }
        for (uint64_t g = 0; g < d.n_add; g++) {
            const auto& a = d.add[g];
            if (a.o_id >= O || a.i0 >= I || a.coef >= m31::P)
                fail(GKRGPU_ERR_INVALID, "layer %d add gate %llu: id or coefficient out of range", l, (unsigned long long)g);
        }
    }
}

// ------------------------------------------------------------------ prover
struct Prover {
    gkrgpu_ctx& c;
    const gkrgpu_circuit& C;
    uint32_t N;
    int R;
    Geo g;
    std::vector<uint32_t*> vals;  // vals[l]: input of layer l; vals[L]: output of the last layer

    Prover(gkrgpu_ctx& ctx, const gkrgpu_circuit& circ, uint32_t n, int reps)
        : c(ctx), C(circ), N(n), R(reps), g(ctx.geo(n)) {}

    void reserve(bool own_input) {
        const uint64_t rowb = (uint64_t)N * 4;
        const uint64_t maxI = 1ull << C.max_in_vars, maxO = 1ull << C.max_out_vars;
        const uint64_t rows = C.value_rows() - (own_input ? 0 : C.in_rows(0));
        c.vals.ensure(rows * rowb, "layer values");
        for (int j = 0; j < R; j++) {
            c.hg0[j].ensure(maxI * rowb, "hg table");
            c.hgA[j].ensure(std::max<uint64_t>(maxI / 2, 1) * rowb, "hg table");
            c.fA[j].ensure(std::max<uint64_t>(maxI / 2, 1) * rowb, "folded table");
            c.fB[j].ensure(std::max<uint64_t>(maxI / 4, 1) * rowb, "folded table");
        }
        c.sb[0].ensure(R * align_up(maxI, 64) * 4, "phase-two table");
        c.sb[1].ensure(R * align_up(maxI, 64) * 4, "phase-two table");
        c.eqc.ensure(R * maxO * 4, "eq table");
        c.eqrx.ensure(R * maxI * 4, "eq table");
        c.a4.ensure(maxI * 16, "add weights");
        c.w4.ensure(std::max<uint64_t>(C.max_mul, 1) * 16, "mul weights");
        // The reducing kernels leave their scratch zeroed; fresh scratch is zeroed here,
        // on the context's stream, before any kernel that uses it.
        const size_t acc_need = 9ull * N * 8;
        if (c.acc.cap < acc_need) {
            c.acc.ensure(acc_need, "reduction scratch");
            ck(cudaMemsetAsync(c.acc.p, 0, c.acc.cap, c.stream), "cudaMemsetAsync");
        }
        if (!c.ticket.p) {
            c.ticket.ensure(256, "ticket");
            ck(cudaMemsetAsync(c.ticket.p, 0, c.ticket.cap, c.stream), "cudaMemsetAsync");
        }
        c.evals.ensure(9ull * N * 4, "round evaluations");
        c.vx.ensure(3ull * N * 4, "vx");
        c.cv.ensure(3ull * N * 4, "claims");
        c.flag.ensure(4, "flag");
        c.h_evals.ensure(9ull * N * 4, "pinned evaluations");
        c.h_rows.ensure(6ull * N * 4, "pinned rows");
        c.h_vx.ensure(3ull * N * 4, "pinned vx");
        c.h_cv.ensure(3ull * N * 4, "pinned claims");
        c.h_flag.ensure(4, "pinned flag");
    }

    void layout_values(const uint32_t* d_input) {
        const uint64_t rowb = (uint64_t)N * 4;
        const size_t L = C.layers.size();
        vals.assign(L + 1, nullptr);
        uint64_t off = 0;
        for (size_t l = 0; l <= L; l++) {
            if (l == 0 && d_input) {
                vals[0] = const_cast<uint32_t*>(d_input);
                continue;
            }
            vals[l] = reinterpret_cast<uint32_t*>(c.vals.as<char>() + off * rowb);
            off += (l < L) ? C.in_rows(l) : C.out_rows(L - 1);
        }
    }

    void check_input() {
        ck(cudaMemsetAsync(c.flag.p, 0, 4, c.stream), "cudaMemsetAsync");
        const uint64_t n = C.in_rows(0) * N;
        c.launch(K_CHECK, (double)n * 4, [&] { return launch_check_canonical(vals[0], n, c.flag.as<unsigned>(), c.stream); });
        c.copy(c.h_flag.p, c.flag.p, 4, cudaMemcpyDeviceToHost, "input check readback");
    }
    void require_canonical() {
        if (*c.h_flag.as<unsigned>()) fail(GKRGPU_ERR_INVALID, "input contains a value >= 2^31 - 1");
    }

    void evaluate() {
        const uint32_t ctas = c.cta_budget();
        for (size_t l = 0; l < C.layers.size(); l++) {
            const DevLayer& Ly = C.layers[l];
            const uint64_t O = 1ull << Ly.nout;
            const double b = 4.0 * N * (2.0 * Ly.nmul + Ly.nadd + O) + 16.0 * Ly.nmul + 8.0 * Ly.nadd + 8.0 * (O + 1);
            c.launch(K_EVALUATE, b, [&] {
                return launch_evaluate(vals[l], vals[l + 1], O, Ly.mo_off, Ly.mo_g, Ly.ao_off, Ly.ao_g, g, c.block,
                                       ctas * 4, c.stream);
            });
        }
    }

    // D2H of the 3R evaluation rows and optionally `rows_from` rows 0..1 for each repetition.
    void fetch(const uint32_t* const* rows_from, bool shared_rows) {
        const uint64_t rowb = (uint64_t)N * 4;
        c.copy(c.h_evals.p, c.evals.p, 3ull * R * rowb, cudaMemcpyDeviceToHost, "fetch evals");
        if (rows_from) {
            for (int j = 0; j < R; j++) {
                const uint32_t* src = shared_rows ? rows_from[0] : rows_from[j];
                c.copy(c.h_rows.as<char>() + 2 * j * rowb, src, 2 * rowb, cudaMemcpyDeviceToHost, "fetch rows");
            }
        }
        c.sync();
    }

    // Transcript step of one round for every repetition (sumcheck.hpp:74-96).  With
    // `last`, the final fold of rows 0..1 gives vx/vy, appended after rep j's challenge
    // when `append_last` (vx); vy is appended after all rounds.
    void transcript_round(Transcript& t, uint32_t (*rch)[32], uint32_t k, bool last, bool append_last,
                          uint32_t* last_out) {
        const uint64_t rowb = (uint64_t)N * 4;
        for (int j = 0; j < R; j++) {
            t.append(c.h_evals.as<char>() + 3ull * j * rowb, 3 * rowb);
            const uint32_t r = t.challenge();
            rch[j][k] = r;
            if (last) {
                const uint32_t* f0 = reinterpret_cast<const uint32_t*>(c.h_rows.as<char>() + 2 * j * rowb);
                const uint32_t* f1 = f0 + N;
                uint32_t* dst = last_out + (uint64_t)j * N;
                for (uint32_t i = 0; i < N; i++) dst[i] = m31::fold(f0[i], f1[i], r);
                if (append_last) t.append(dst, rowb);
            }
        }
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

    void sumcheck_layer(Transcript& t, size_t li, uint32_t (*rz1)[32], uint32_t (*rz2)[32], uint32_t alpha,
                        uint32_t beta, uint32_t (*rx)[32], uint32_t (*ry)[32]) {
        const DevLayer& Ly = C.layers[li];
        const uint32_t n = Ly.nin, m = Ly.nout;
        const uint64_t I = 1ull << n, O = 1ull << m;
        const uint64_t rowb = (uint64_t)N * 4;
        const double rb = 4.0 * N;
        const uint32_t ctas = c.cta_budget();
        uint32_t* v = vals[li];
        uint32_t* vxh = c.h_vx.as<uint32_t>();
        std::vector<uint32_t> vy((size_t)R * N);

        // phase one: eqc_j = alpha eq(rz1_j) + beta eq(rz2_j), gate weights, hg + round 0
        eq_table(c.eqc.as<uint32_t>(), rz1, rz2, alpha, beta, m);
        const double wb = 32.0 * Ly.nmul + 20.0 * I + 8.0 * Ly.nadd + 4.0 * R * (Ly.nmul + Ly.nadd);
        c.launch(K_WEIGHTS, wb, [&] {
            return launch_weights(I, Ly.nmul, O, c.eqc.as<uint32_t>(), Ly.mx_g, Ly.ax_off, Ly.ax_g, c.a4.as<uint4>(),
                                  c.w4.as<uint4>(), R, c.stream);
        });
        uint32_t* hg[3] = {c.hg0[0].as<uint32_t>(), R > 1 ? c.hg0[1].as<uint32_t>() : nullptr,
                           R > 2 ? c.hg0[2].as<uint32_t>() : nullptr};
        const double hb = rb * (I + Ly.nmul + (double)R * I) + 32.0 * Ly.nmul + 20.0 * I;
        c.launch(K_HG_ROUND0, hb, [&] {
            return launch_hg_round0(R, v, I, Ly.mx_off, Ly.mx_g, c.a4.as<uint4>(), c.w4.as<uint4>(), hg, g, c.block,
                                    ctas, c.red(), c.evals.as<uint32_t>(), c.stream);
        });
        const uint32_t* vsrc[1] = {v};
        fetch(n == 1 ? vsrc : nullptr, true);
        transcript_round(t, rx, 0, n == 1, true, vxh);

        const uint32_t* cur_f[3] = {v, v, v};
        const uint32_t* cur_h[3] = {hg[0], hg[1], hg[2]};
        for (uint32_t k = 1; k < n; k++) {
            RoundPtrs p;
            memset(&p, 0, sizeof(p));
            for (int j = 0; j < R; j++) {
                p.fsrc[j] = cur_f[j];
                p.hsrc[j] = cur_h[j];
                p.fdst[j] = (k & 1) ? c.fA[j].as<uint32_t>() : c.fB[j].as<uint32_t>();
                p.hdst[j] = (k & 1) ? c.hgA[j].as<uint32_t>() : c.hg0[j].as<uint32_t>();
                p.r[j] = rx[j][k - 1];
            }
            const uint64_t npairs = I >> (k + 1);
            const double S = 4.0 * npairs;
            const double b = rb * ((k == 1 ? 1.0 : R) * S + R * S + R * S);
            c.launch(K_ROUND_LANE, b, [&] {
                return launch_round(R, k == 1, true, true, p, npairs, nullptr, g, c.block, ctas, c.red(),
                                    c.evals.as<uint32_t>(), c.stream);
            });
            const bool last = (k == n - 1);
            fetch(last ? p.fdst : nullptr, false);
            transcript_round(t, rx, k, last, true, vxh);
            for (int j = 0; j < R; j++) {
                cur_f[j] = p.fdst[j];
                cur_h[j] = p.hdst[j];
            }
        }

        // phase two: h(y) = vx * s(y)
        eq_table(c.eqrx.as<uint32_t>(), rx, nullptr, 1u, 0u, n);
        const size_t sstride = align_up(1ull << C.max_in_vars, 64);
        c.launch(K_S_BUILD, 16.0 * Ly.nmul + 4.0 * I + 4.0 * R * I + 8.0 * R * Ly.nmul, [&] {
            return launch_s_build(I, O, Ly.my_off, Ly.my_g, c.eqc.as<uint32_t>(), c.eqrx.as<uint32_t>(),
                                  c.sb[0].as<uint32_t>(), sstride, R, c.stream);
        });
        c.copy(c.vx.p, vxh, R * rowb, cudaMemcpyHostToDevice, "vx upload");
        {
            RoundPtrs p;
            memset(&p, 0, sizeof(p));
            p.fsrc[0] = v;
            for (int j = 0; j < R; j++) p.hsrc[j] = c.sb[0].as<uint32_t>() + j * sstride;
            const uint64_t npairs = I >> 1;
            c.launch(K_ROUND_SCALAR, rb * 2.0 * npairs + 8.0 * R * npairs, [&] {
                return launch_round(R, true, false, false, p, npairs, c.vx.as<uint32_t>(), g, c.block, ctas, c.red(),
                                    c.evals.as<uint32_t>(), c.stream);
            });
            fetch(n == 1 ? vsrc : nullptr, true);
            transcript_round(t, ry, 0, n == 1, false, vy.data());
        }
        for (int j = 0; j < R; j++) cur_f[j] = v;
        for (uint32_t k = 1; k < n; k++) {
            RoundPtrs p;
            memset(&p, 0, sizeof(p));
            const int src = (k - 1) & 1, dst = k & 1;
            for (int j = 0; j < R; j++) {
                p.fsrc[j] = cur_f[j];
                p.fdst[j] = (k & 1) ? c.fA[j].as<uint32_t>() : c.fB[j].as<uint32_t>();
                p.hsrc[j] = c.sb[src].as<uint32_t>() + j * sstride;
                p.hdst[j] = c.sb[dst].as<uint32_t>() + j * sstride;
                p.r[j] = ry[j][k - 1];
            }
            const uint64_t npairs = I >> (k + 1);
            const double S = 4.0 * npairs;
            const double b = rb * ((k == 1 ? 1.0 : R) * S + R * S / 2) + 6.0 * R * S;
            c.launch(K_ROUND_SCALAR, b, [&] {
                return launch_round(R, k == 1, false, true, p, npairs, c.vx.as<uint32_t>(), g, c.block, ctas, c.red(),
                                    c.evals.as<uint32_t>(), c.stream);
            });
            const bool last = (k == n - 1);
            fetch(last ? p.fdst : nullptr, false);
            transcript_round(t, ry, k, last, false, vy.data());
            for (int j = 0; j < R; j++) cur_f[j] = p.fdst[j];
        }
        for (int j = 0; j < R; j++) t.append(vy.data() + (size_t)j * N, rowb);
    }

    // Device front half of a proof: input upload and check, Circuit::evaluate of every layer.
    // Asynchronous on the context's stream; it needs no transcript.
    void device_front(const uint32_t* h_input, const uint32_t* d_input) {
        const uint64_t in_bytes = C.in_rows(0) * (uint64_t)N * 4;
        reserve(d_input == nullptr);
        layout_values(d_input);
        if (h_input) c.copy(vals[0], h_input, in_bytes, cudaMemcpyHostToDevice, "input upload");
        check_input();
        evaluate();
    }

    // Device back half: gkr_prove from the transcript state left by the host stage (RAW
    // commitment + grinding), writing the rest of the proof and the claimed values.
    void device_back(const TranscriptState& ts, uint8_t* proof_out, uint32_t* claimed_v) {
        const size_t L = C.layers.size();
        const uint64_t rowb = (uint64_t)N * 4;
        Transcript t(proof_out, ts);

        // gkr_prove (gkr.hpp:42-55): rz1 challenges (i outer, j inner), rz2 = 0, alpha = 1, beta = 0.
        uint32_t rz1[3][32], rz2[3][32], rx[3][32], ry[3][32];
        memset(rz1, 0, sizeof(rz1));
        memset(rz2, 0, sizeof(rz2));
        const uint32_t nz = C.layers[L - 1].nout;
        for (uint32_t i = 0; i < nz; i++)
            for (int j = 0; j < R; j++) rz1[j][i] = t.challenge();
        uint32_t alpha = 1, beta = 0;

        // claimed_v[j] = eval_multilinear(output, rz1[j]) = sum_z eq(rz1_j, z) out[z]
        eq_table(c.eqc.as<uint32_t>(), rz1, nullptr, 1u, 0u, nz);
        const uint64_t OL = C.out_rows(L - 1);
        c.launch(K_WSUM, 4.0 * N * OL + 4.0 * R * OL, [&] {
            return launch_wsum(R, vals[L], OL, c.eqc.as<uint32_t>(), g, c.block, c.cta_budget(), c.red(),
                               c.cv.as<uint32_t>(), c.stream);
        });
        c.copy(c.h_cv.p, c.cv.p, R * rowb, cudaMemcpyDeviceToHost, "claims readback");
        c.sync();
        require_canonical();
        memcpy(claimed_v, c.h_cv.p, R * rowb);

        for (int li = (int)L - 1; li >= 0; li--) {
            sumcheck_layer(t, (size_t)li, rz1, rz2, alpha, beta, rx, ry);
            alpha = t.challenge();
            beta = t.challenge();
            const uint32_t n = C.layers[li].nin;
            for (int j = 0; j < R; j++) {
                memcpy(rz1[j], rx[j], 4 * n);
                memcpy(rz2[j], ry[j], 4 * n);
            }
        }
        // RawPC::open: the openings are empty (raw.hpp:61-66, LinearGKR.hpp:77-86).
        c.sync();
        c.resolve_events();
    }

    void evaluate_only(const uint32_t* h_input, uint32_t* out, bool all_layers) {
        const uint64_t rowb = (uint64_t)N * 4;
        reserve(true);
        layout_values(nullptr);
        c.copy(vals[0], h_input, C.in_rows(0) * rowb, cudaMemcpyHostToDevice, "input upload");
        check_input();
        evaluate();
        c.sync();
        require_canonical();
        const size_t L = C.layers.size();
        if (all_layers) {
            ck(cudaMemcpy(out, vals[0], C.value_rows() * rowb, cudaMemcpyDeviceToHost), "values readback");
        } else {
            ck(cudaMemcpy(out, vals[L], C.out_rows(L - 1) * rowb, cudaMemcpyDeviceToHost), "output readback");
        }
        c.resolve_events();
    }
};

void check_ctx(gkrgpu_ctx* ctx) {
    if (!ctx) fail(GKRGPU_ERR_INVALID, "null context");
}

void check_run(gkrgpu_ctx* ctx, const gkrgpu_circuit* circuit, uint32_t n_copies) {
    check_ctx(ctx);
    if (!circuit) fail(GKRGPU_ERR_INVALID, "null circuit");
    if (circuit->device != ctx->device) fail(GKRGPU_ERR_INVALID, "circuit was loaded on another device");
    if (n_copies < 4 || n_copies % 4 || n_copies > (1u << 16))
        fail(GKRGPU_ERR_INVALID, "n_copies must be a multiple of 4 in [4, 65536], got %u", n_copies);
    const uint32_t Q = n_copies / 4;
    const Geo g = ctx->geo(n_copies);
    if (g.tpr * (Q / g.tpr) != Q) fail(GKRGPU_ERR_INVALID, "no row tile divides %u copies", n_copies);
}

uint64_t proof_bytes(const gkrgpu_circuit* c, uint32_t N, int R) {
    uint64_t rows = 0;
    for (const auto& l : c->layers) rows += (uint64_t)R * (6ull * l.nin + 2);
    return c->in_rows(0) * N * 4 + 32 + rows * N * 4;
}

// ------------------------------------------------------------------ job pipeline
// A proof is two stages: the host stage (RAW commitment bytes into the proof buffer, their
// SHA-256, grinding) and the device stage (upload, evaluate, then gkr_prove resuming the
// transcript).  The device stage of proof k runs on the GPU worker while host workers
// hash the commitments of proofs k+1, k+2, ...; device stages run one at a time in
// submission order because they share the context's workspace.

// Copies n bytes in helper threads while this thread hashes the source.
void parallel_copy_and_hash(uint8_t* dst, const uint8_t* src, uint64_t n, uint8_t digest[32]) {
    const unsigned k = n >= (64ull << 20) ? 4 : (n >= (4ull << 20) ? 2 : 0);
    std::vector<std::thread> th;
    if (k) {
        const uint64_t chunk = (n + k - 1) / k;
        for (unsigned i = 0; i < k; i++) {
            const uint64_t a = i * chunk, b = std::min<uint64_t>(n, a + chunk);
            if (a < b) th.emplace_back([=] { memcpy(dst + a, src + a, b - a); });
        }
    } else {
        memcpy(dst, src, n);
    }
    sha256(src, n, digest);
    for (auto& t : th) t.join();
}

TranscriptState host_stage(gkrgpu_ctx& c, gkrgpu_job& j, cudaStream_t s) {
    const uint64_t in_bytes = j.circuit->in_rows(0) * (uint64_t)j.N * 4;
    uint8_t d[32];
    if (j.h_input) {
        parallel_copy_and_hash(j.proof_out, reinterpret_cast<const uint8_t*>(j.h_input), in_bytes, d);
    } else {
        ck(cudaMemcpyAsync(j.proof_out, j.d_input, in_bytes, cudaMemcpyDeviceToHost, s), "commitment readback");
        ck(cudaStreamSynchronize(s), "cudaStreamSynchronize");
        c.d2h_bytes += in_bytes;
        sha256(j.proof_out, in_bytes, d);
    }
    Transcript t(j.proof_out, ~0ull);
    t.appended_prehashed(in_bytes, d);
    grind(t, j.grinding);
    return t.state();
}

void host_worker(gkrgpu_ctx* c) {
    cudaSetDevice(c->device);
    cudaStream_t s = nullptr;
    cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    for (;;) {
        gkrgpu_job* j;
        {
            std::unique_lock<std::mutex> lk(c->qm);
            c->qcv.wait(lk, [&] { return c->stopping || !c->host_q.empty(); });
            if (c->host_q.empty()) break;
            j = c->host_q.front();
            c->host_q.pop_front();
        }
        int rc = GKRGPU_OK;
        std::string err;
        try {
            if (!s) fail(GKRGPU_ERR_CUDA, "host worker stream creation failed");
            j->ts = host_stage(*c, *j, s);
        } catch (const Error& e) {
            rc = e.code;
            err = e.what();
        } catch (const std::exception& e) {
            rc = GKRGPU_ERR_STATE;
            err = e.what();
        }
        {
            std::lock_guard<std::mutex> lk(j->m);
            j->host_rc = rc;
            j->host_err = err;
            j->host_done = true;
        }
        j->cv.notify_all();
    }
    if (s) cudaStreamDestroy(s);
}

void gpu_worker(gkrgpu_ctx* c) {
    cudaSetDevice(c->device);
    for (;;) {
        gkrgpu_job* j;
        {
            std::unique_lock<std::mutex> lk(c->qm);
            c->qcv.wait(lk, [&] { return c->stopping || !c->gpu_q.empty(); });
            if (c->gpu_q.empty()) break;
            j = c->gpu_q.front();
            c->gpu_q.pop_front();
            c->gpu_busy = true;
        }
        int rc = GKRGPU_OK;
        std::string err;
        try {
            Prover p(*c, *j->circuit, j->N, j->R);
            p.device_front(j->h_input, j->d_input);
            {
                std::unique_lock<std::mutex> lk(j->m);
                j->cv.wait(lk, [&] { return j->host_done; });
            }
            if (j->host_rc) throw Error(j->host_rc, j->host_err);
            p.device_back(j->ts, j->proof_out, j->claimed_v);
            if (j->marker >= 0) {
                if (!c->markers[j->marker]) ck(cudaEventCreate(&c->markers[j->marker]), "cudaEventCreate");
                ck(cudaEventRecord(c->markers[j->marker], c->stream), "cudaEventRecord");
            }
        } catch (const Error& e) {
            rc = e.code;
            err = e.what();
        } catch (const std::exception& e) {
            rc = GKRGPU_ERR_STATE;
            err = e.what();
        }
        if (rc != GKRGPU_OK) {
            cudaStreamSynchronize(c->stream);
            c->discard_job_stats();
        }
        {
            std::lock_guard<std::mutex> lk(j->m);
            j->rc = rc;
            j->err = err;
            j->done = true;
        }
        j->cv.notify_all();
        {
            std::lock_guard<std::mutex> lk(c->qm);
            c->gpu_busy = false;
        }
        c->qcv.notify_all();
    }
}

gkrgpu_job* submit(gkrgpu_ctx* ctx, const gkrgpu_circuit* circuit, uint32_t n_copies, int grinding_bits,
                   const uint32_t* h_input, const uint32_t* d_input, uint8_t* proof_out, uint64_t proof_cap,
                   uint32_t* claimed_v, int marker, uint64_t* need_out) {
    check_run(ctx, circuit, n_copies);
    if (grinding_bits < 0 || grinding_bits > 30) fail(GKRGPU_ERR_INVALID, "grinding_bits must be in [0, 30]");
    const int R = reps_for(grinding_bits);
    if (R < 1 || R > 3) fail(GKRGPU_ERR_INVALID, "grinding_bits %d gives %d repetitions (1..3 supported)", grinding_bits, R);
    if (!(h_input || d_input) || !proof_out || !claimed_v) fail(GKRGPU_ERR_INVALID, "null buffer");
    if (d_input && ((uintptr_t)d_input & 15)) fail(GKRGPU_ERR_INVALID, "device input must be 16-byte aligned");
    if (marker < -1 || marker >= 64) fail(GKRGPU_ERR_INVALID, "marker slot must be -1 or in [0, 64)");
    const uint64_t need = proof_bytes(circuit, n_copies, R);
    if (need_out) *need_out = need;
    if (proof_cap < need)
        fail(GKRGPU_ERR_CAPACITY, "proof needs %llu bytes, buffer has %llu", (unsigned long long)need,
             (unsigned long long)proof_cap);
    gkrgpu_job* j = new gkrgpu_job();
    j->circuit = circuit;
    j->N = n_copies;
    j->grinding = grinding_bits;
    j->R = R;
    j->h_input = h_input;
    j->d_input = d_input;
    j->proof_out = proof_out;
    j->proof_len = need;
    j->claimed_v = claimed_v;
    j->marker = marker;
    ctx->start_workers();
    {
        std::lock_guard<std::mutex> lk(ctx->qm);
        ctx->host_q.push_back(j);
        ctx->gpu_q.push_back(j);
    }
    ctx->qcv.notify_all();
    return j;
}

int wait_job(gkrgpu_job* j, uint64_t* proof_len) {
    {
        std::unique_lock<std::mutex> lk(j->m);
        j->cv.wait(lk, [&] { return j->done && j->host_done; });
    }
    const int rc = j->rc;
    if (rc != GKRGPU_OK) g_last_error = j->err;
    if (proof_len) *proof_len = j->proof_len;
    delete j;
    return rc;
}

int prove_entry(gkrgpu_ctx* ctx, const gkrgpu_circuit* circuit, uint32_t n_copies, int grinding_bits,
                const uint32_t* h_input, const uint32_t* d_input, uint8_t* proof_out, uint64_t proof_cap,
                uint64_t* proof_len, uint32_t* claimed_v) {
    gkrgpu_job* j = nullptr;
    const int rc = guarded([&] {
        if (!proof_len) fail(GKRGPU_ERR_INVALID, "null proof_len");
        j = submit(ctx, circuit, n_copies, grinding_bits, h_input, d_input, proof_out, proof_cap, claimed_v, -1,
                   proof_len);
    });
    if (rc != GKRGPU_OK) return rc;
    return wait_job(j, proof_len);
}

}  // namespace

void gkrgpu_ctx::start_workers() {
    std::lock_guard<std::mutex> lk(qm);
    if (!workers.empty()) return;
    stopping = false;
    workers.emplace_back(gpu_worker, this);
    for (int i = 0; i < host_workers; i++) workers.emplace_back(host_worker, this);
}

namespace gkrgpu {
// Records the calling thread's error text (shared with the other translation units).
void set_last_error(const char* msg) { g_last_error = msg ? msg : ""; }
}  // namespace gkrgpu

// ------------------------------------------------------------------ C ABI
extern "C" {

const char* gkrgpu_last_error(void) { return g_last_error.c_str(); }

const char* gkrgpu_version(void) {
    static std::string v = std::string("gkrgpu 0.1 (sm_103a; host sha256: ") + sha256_impl_name() + ")";
    return v.c_str();
}

int gkrgpu_num_repetitions(int grinding_bits) { return reps_for(grinding_bits); }

int gkrgpu_create(int device, gkrgpu_ctx** out) {
    return guarded([&] {
        if (!out) fail(GKRGPU_ERR_INVALID, "null output");
        *out = nullptr;
        int n = 0;
        ck(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
        if (device < 0 || device >= n) fail(GKRGPU_ERR_INVALID, "device %d out of range (%d devices)", device, n);
        DeviceGuard dg(device);
        gkrgpu_ctx* c = new gkrgpu_ctx();
        c->device = device;
        cudaDeviceProp prop;
        if (cudaGetDeviceProperties(&prop, device) == cudaSuccess) c->sm_count = prop.multiProcessorCount;
        cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            delete c;
            ck(e, "cudaStreamCreate");
        }
        *out = c;
    });
}

void gkrgpu_destroy(gkrgpu_ctx* ctx) {
    if (!ctx) return;
    try {
        ctx->shutdown();
        delete ctx;
    } catch (...) {
    }
}

int gkrgpu_circuit_load(gkrgpu_ctx* ctx, const gkrgpu_layer_desc* layers, int n_layers, gkrgpu_circuit** out) {
    return guarded([&] {
        check_ctx(ctx);
        if (!out) fail(GKRGPU_ERR_INVALID, "null output");
        *out = nullptr;
        validate_layers(layers, n_layers);
        DeviceGuard dg(ctx->device);
        gkrgpu_circuit* c = new gkrgpu_circuit();
        c->device = ctx->device;
        try {
            for (int l = 0; l < n_layers; l++) {
                c->layers.push_back(upload_layer(layers[l]));
                c->max_in_vars = std::max(c->max_in_vars, layers[l].nb_input_vars);
                c->max_out_vars = std::max(c->max_out_vars, layers[l].nb_output_vars);
                c->max_mul = std::max<uint64_t>(c->max_mul, layers[l].n_mul);
            }
        } catch (...) {
            delete c;
            throw;
        }
        *out = c;
    });
}

void gkrgpu_circuit_free(gkrgpu_circuit* circuit) {
    if (!circuit) return;
    try {
        DeviceGuard dg(circuit->device);
        delete circuit;
    } catch (...) {
    }
}

uint64_t gkrgpu_proof_size(const gkrgpu_circuit* circuit, uint32_t n_copies, int grinding_bits) {
    if (!circuit) return 0;
    return proof_bytes(circuit, n_copies, reps_for(grinding_bits));
}

uint64_t gkrgpu_value_rows(const gkrgpu_circuit* circuit, int all_layers) {
    if (!circuit) return 0;
    return all_layers ? circuit->value_rows() : circuit->out_rows(circuit->layers.size() - 1);
}

int gkrgpu_evaluate(gkrgpu_ctx* ctx, const gkrgpu_circuit* circuit, uint32_t n_copies, const uint32_t* input,
                    uint32_t* out, int all_layers) {
    return guarded([&] {
        check_run(ctx, circuit, n_copies);
        if (!input || !out) fail(GKRGPU_ERR_INVALID, "null buffer");
        ctx->drain();
        DeviceGuard dg(ctx->device);
        Prover p(*ctx, *circuit, n_copies, 1);
        p.evaluate_only(input, out, all_layers != 0);
    });
}

int gkrgpu_prove_submit(gkrgpu_ctx* ctx, const gkrgpu_circuit* circuit, uint32_t n_copies, int grinding_bits,
                        const uint32_t* input, int input_on_device, uint8_t* proof_out, uint64_t proof_cap,
                        uint32_t* claimed_v, int marker_slot, gkrgpu_job** job) {
    return guarded([&] {
        if (!job) fail(GKRGPU_ERR_INVALID, "null job output");
        *job = nullptr;
        *job = submit(ctx, circuit, n_copies, grinding_bits, input_on_device ? nullptr : input,
                      input_on_device ? input : nullptr, proof_out, proof_cap, claimed_v, marker_slot, nullptr);
    });
}

int gkrgpu_prove_wait(gkrgpu_job* job, uint64_t* proof_len) {
    if (!job) {
        g_last_error = "null job";
        return GKRGPU_ERR_INVALID;
    }
    return wait_job(job, proof_len);
}

int gkrgpu_prove(gkrgpu_ctx* ctx, const gkrgpu_circuit* circuit, uint32_t n_copies, int grinding_bits,
                 const uint32_t* input, uint8_t* proof_out, uint64_t proof_cap, uint64_t* proof_len,
                 uint32_t* claimed_v) {
    return prove_entry(ctx, circuit, n_copies, grinding_bits, input, nullptr, proof_out, proof_cap, proof_len,
                       claimed_v);
}

int gkrgpu_prove_device(gkrgpu_ctx* ctx, const gkrgpu_circuit* circuit, uint32_t n_copies, int grinding_bits,
                        const uint32_t* d_input, uint8_t* proof_out, uint64_t proof_cap, uint64_t* proof_len,
                        uint32_t* claimed_v) {
    if (d_input && ((uintptr_t)d_input & 15)) {
        g_last_error = "d_input must be 16-byte aligned";
        return GKRGPU_ERR_INVALID;
    }
    return prove_entry(ctx, circuit, n_copies, grinding_bits, nullptr, d_input, proof_out, proof_cap, proof_len,
                       claimed_v);
}

int gkrgpu_eval_multilinear(gkrgpu_ctx* ctx, const uint32_t* d_evals, uint32_t nb_vars, uint32_t n_copies,
                            const uint32_t* r, int n_points, uint32_t* out) {
    return guarded([&] {
        check_ctx(ctx);
        ctx->drain();
        if (!d_evals || !r || !out) fail(GKRGPU_ERR_INVALID, "null buffer");
        if ((uintptr_t)d_evals & 15) fail(GKRGPU_ERR_INVALID, "d_evals must be 16-byte aligned");
        if (n_points < 1 || n_points > 3) fail(GKRGPU_ERR_INVALID, "n_points must be in [1, 3]");
        if (nb_vars > 30) fail(GKRGPU_ERR_INVALID, "nb_vars must be <= 30");
        if (n_copies < 4 || n_copies % 4 || n_copies > (1u << 16))
            fail(GKRGPU_ERR_INVALID, "n_copies must be a multiple of 4 in [4, 65536]");
        for (int j = 0; j < n_points; j++)
            for (uint32_t t = 0; t < nb_vars; t++)
                if (r[(size_t)j * nb_vars + t] >= m31::P) fail(GKRGPU_ERR_INVALID, "point coordinate >= p");
        const Geo g = ctx->geo(n_copies);
        if (g.tpr * ((n_copies / 4) / g.tpr) != n_copies / 4) fail(GKRGPU_ERR_INVALID, "no row tile divides n_copies");
        DeviceGuard dg(ctx->device);
        const uint64_t rows = 1ull << nb_vars, rowb = (uint64_t)n_copies * 4;
        ctx->eqc.ensure(n_points * rows * 4, "eq table");
        if (ctx->acc.cap < 9ull * n_copies * 8) {
            ctx->acc.ensure(9ull * n_copies * 8, "reduction scratch");
            ck(cudaMemsetAsync(ctx->acc.p, 0, ctx->acc.cap, ctx->stream), "cudaMemsetAsync");
        }
        if (!ctx->ticket.p) {
            ctx->ticket.ensure(256, "ticket");
            ck(cudaMemsetAsync(ctx->ticket.p, 0, ctx->ticket.cap, ctx->stream), "cudaMemsetAsync");
        }
        ctx->cv.ensure(3 * rowb, "claims");
        ctx->h_cv.ensure(3 * rowb, "pinned claims");
        EqArgs a;
        memset(&a, 0, sizeof(a));
        for (int j = 0; j < n_points; j++) memcpy(a.r1[j], r + (size_t)j * nb_vars, 4 * nb_vars);
        a.f1 = 1u;
        a.nvars = nb_vars;
        a.reps = n_points;
        ctx->launch(K_EQ, 4.0 * n_points * rows, [&] { return launch_eq(ctx->eqc.as<uint32_t>(), a, ctx->stream); });
        ctx->launch(K_WSUM, 4.0 * n_copies * rows + 4.0 * n_points * rows, [&] {
            return launch_wsum(n_points, d_evals, rows, ctx->eqc.as<uint32_t>(), g, ctx->block, ctx->cta_budget(),
                               ctx->red(), ctx->cv.as<uint32_t>(), ctx->stream);
        });
        ctx->copy(ctx->h_cv.p, ctx->cv.p, n_points * rowb, cudaMemcpyDeviceToHost, "result readback");
        ctx->sync();
        memcpy(out, ctx->h_cv.p, n_points * rowb);
        ctx->resolve_events();
    });
}

int gkrgpu_device_alloc(gkrgpu_ctx* ctx, uint64_t bytes, void** out) {
    return guarded([&] {
        check_ctx(ctx);
        if (!out) fail(GKRGPU_ERR_INVALID, "null output");
        DeviceGuard dg(ctx->device);
        ck(cudaMalloc(out, bytes ? bytes : 1), "cudaMalloc");
    });
}

int gkrgpu_device_free(gkrgpu_ctx* ctx, void* p) {
    return guarded([&] {
        check_ctx(ctx);
        DeviceGuard dg(ctx->device);
        ck(cudaFree(p), "cudaFree");
    });
}

int gkrgpu_host_alloc(uint64_t bytes, void** out) {
    return guarded([&] {
        if (!out) fail(GKRGPU_ERR_INVALID, "null output");
        ck(cudaMallocHost(out, bytes ? bytes : 1), "cudaMallocHost");
    });
}

int gkrgpu_host_free(void* p) {
    return guarded([&] { ck(cudaFreeHost(p), "cudaFreeHost"); });
}

int gkrgpu_memcpy_h2d(gkrgpu_ctx* ctx, void* dst, const void* src, uint64_t bytes) {
    return guarded([&] {
        check_ctx(ctx);
        ctx->drain();
        DeviceGuard dg(ctx->device);
        ck(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream), "cudaMemcpyAsync");
        ctx->sync();
    });
}

int gkrgpu_memcpy_d2h(gkrgpu_ctx* ctx, void* dst, const void* src, uint64_t bytes) {
    return guarded([&] {
        check_ctx(ctx);
        ctx->drain();
        DeviceGuard dg(ctx->device);
        ck(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync");
        ctx->sync();
    });
}

int gkrgpu_set_timing(gkrgpu_ctx* ctx, int enabled) {
    return guarded([&] {
        check_ctx(ctx);
        ctx->drain();
        ctx->timing = enabled != 0;
    });
}

int gkrgpu_reset_stats(gkrgpu_ctx* ctx) {
    return guarded([&] {
        check_ctx(ctx);
        ctx->drain();
        ctx->discard_job_stats();
        std::lock_guard<std::mutex> lk(ctx->stats_m);
        for (int k = 0; k < K_NUM_KERNELS; k++) {
            ctx->launches[k] = 0;
            ctx->ms[k] = 0;
            ctx->bytes[k] = 0;
        }
        ctx->h2d_bytes = ctx->d2h_bytes = 0;
    });
}

int gkrgpu_mark(gkrgpu_ctx* ctx, int slot) {
    return guarded([&] {
        check_ctx(ctx);
        if (slot < 0 || slot >= 64) fail(GKRGPU_ERR_INVALID, "marker slot must be in [0, 64)");
        DeviceGuard dg(ctx->device);
        if (!ctx->markers[slot]) ck(cudaEventCreate(&ctx->markers[slot]), "cudaEventCreate");
        ck(cudaEventRecord(ctx->markers[slot], ctx->stream), "cudaEventRecord");
    });
}

int gkrgpu_elapsed_ms(gkrgpu_ctx* ctx, int from_slot, int to_slot, double* ms) {
    return guarded([&] {
        check_ctx(ctx);
        if (!ms || from_slot < 0 || from_slot >= 64 || to_slot < 0 || to_slot >= 64 || !ctx->markers[from_slot] ||
            !ctx->markers[to_slot])
            fail(GKRGPU_ERR_INVALID, "unrecorded marker slot");
        DeviceGuard dg(ctx->device);
        ck(cudaEventSynchronize(ctx->markers[to_slot]), "cudaEventSynchronize");
        float t = 0.f;
        ck(cudaEventElapsedTime(&t, ctx->markers[from_slot], ctx->markers[to_slot]), "cudaEventElapsedTime");
        *ms = t;
    });
}

int gkrgpu_transfer_stats(gkrgpu_ctx* ctx, uint64_t* h2d_bytes, uint64_t* d2h_bytes) {
    return guarded([&] {
        check_ctx(ctx);
        if (h2d_bytes) *h2d_bytes = ctx->h2d_bytes;
        if (d2h_bytes) *d2h_bytes = ctx->d2h_bytes;
    });
}

int gkrgpu_kernel_stats(gkrgpu_ctx* ctx, gkrgpu_kernel_stat* out, int cap) {
    if (!ctx) return -GKRGPU_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->stats_m);
    for (int k = 0; k < K_NUM_KERNELS && k < cap; k++) {
        out[k].name = kKernelNames[k];
        out[k].launches = ctx->launches[k];
        out[k].total_ms = ctx->ms[k];
        out[k].algorithmic_bytes = ctx->bytes[k];
    }
    return K_NUM_KERNELS;
}

int gkrgpu_set_tile(gkrgpu_ctx* ctx, uint32_t threads_per_row, uint32_t block, uint32_t ctas) {
    return guarded([&] {
        check_ctx(ctx);
        ctx->drain();
        const uint32_t b = block ? block : ctx->block;
        const uint32_t t = threads_per_row ? threads_per_row : ctx->tpr_max;
        if (b < 32 || b > 256 || b % 32) fail(GKRGPU_ERR_INVALID, "block must be a multiple of 32 in [32, 256]");
        if (t < 1 || t > b) fail(GKRGPU_ERR_INVALID, "threads_per_row must be in [1, block]");
        ctx->block = b;
        ctx->tpr_max = t;
        if (ctas) ctx->ctas = ctas;
    });
}

}  // extern "C"
