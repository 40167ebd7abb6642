// Host orchestration of the GB300 GKR prover and the C ABI (include/gkrgpu.h).
//
// Prove flow, following Prover::prove (include/LinearGKR/LinearGKR.hpp:58-90) and
// gkr_prove (include/LinearGKR/gkr.hpp:24-73):
//   host   : RAW commitment bytes -> transcript, grinding (a host worker, overlapped)
//   device : input -> Circuit::evaluate of every layer, kept resident for the sumcheck
//   device : claimed_v = eval_multilinear(output, rz1_j) for every repetition j
//   per layer, top down, per sumcheck_prove_gkr_layer (include/LinearGKR/sumcheck.hpp:52-111):
//     device : eq tables, gate weights, hg build fused with round 0
//     rounds : device fold+reduce for all repetitions -> 3R rows to the host -> the host
//              appends them and derives the R challenges in the reference's order
//     phase 2: s(y) table, rounds over the layer input with h = v(rx) * s
//   alpha, beta challenges between layers.
// The host does only transcript work: appending bytes, SHA-256, and the last 2->1 fold of
// each phase's table (vx, vy: 2 rows x N lanes), whose result must enter the transcript
// before the next repetition's challenge.
//
// Concurrency: a context owns `lanes` device workers, each with its own stream, so the
// device stages of several proofs overlap (continuous batching: a queued proof starts as
// soon as a lane is free and its device workspace fits in the HBM budget).  Each proof's
// workspace is one block from a stream-ordered memory pool, returned when the proof ends.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>
#ifdef __linux__
#include <sys/prctl.h>
#endif

#include "../../include/gkrgpu.h"
#include "bn254.cuh"
#include "fr_host.hpp"
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

// The same for a field of `field_size` bits (254 for BN254).
int reps_for_field(int field, int grinding_bits) {
    if (field != GKRGPU_FIELD_BN254) return reps_for(grinding_bits);
    const int s = 100 - grinding_bits;
    return s / 254 + (s % 254 != 0);
}

bool field_supported(int field) { return field == GKRGPU_FIELD_M31 || field == GKRGPU_FIELD_BN254; }

// Bytes of one field element: M31 4, BN254 32.
uint32_t elem_bytes(int field) { return field == GKRGPU_FIELD_BN254 ? 32u : 4u; }

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Pinned host buffer that grows on demand.
struct PinnedBuf {
    void* p = nullptr;
    size_t cap = 0;
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
    }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
    void ensure(size_t bytes, const char* what) {
        bytes = std::max<size_t>(align_up(bytes, 256), 256);
        if (bytes <= cap) return;
        release();
        cudaError_t e = cudaMallocHost(&p, bytes);
        if (e != cudaSuccess) {
            p = nullptr;
            cudaGetLastError();
            fail(GKRGPU_ERR_NOMEM, "pinned allocation of %zu bytes for %s failed: %s", bytes, what, cudaGetErrorString(e));
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
    // phase-one rows q < I/2 after round 0 whose input rows 2q, 2q+1 have no mul gates: their
    // hg is the same for every copy, is not stored by round 1 and is recomputed in round 2
    uint64_t h1_scalar_rows = 0;
    // the same after round 1: rows q < I/4 whose input rows 4q .. 4q+3 have no mul gates (not
    // stored by round 2, recomputed in round 3)
    uint64_t h2_scalar_rows = 0;
    // Groups of input rows that have gates, for the kernels that skip the rest (the
    // reference's gate_exists, sumcheck_helper.hpp:82-84,118-130): pairs (2q, 2q+1) and
    // quads 4q .. 4q+3 with a gate whose first input is in them (phase one, rounds 0 and 1),
    // quads with a mul gate whose second input is in them (phase two, rounds 0 and 1).  A
    // null list means every group (used when nearly all of them have gates).
    const uint32_t *p1_pairs = nullptr, *p1_quads = nullptr, *p2_quads = nullptr;
    uint64_t n_p1_pairs = 0, n_p1_quads = 0, n_p2_quads = 0;
    // BN254 circuits: each gate's coefficient in Montgomery form, in the order of the table above
    const bn::Fr *mo_c = nullptr, *ao_c = nullptr, *mx_c = nullptr, *ax_c = nullptr, *my_c = nullptr;
    void* block = nullptr;
};

struct gkrgpu_circuit {
    int device = 0;
    int field = GKRGPU_FIELD_M31;
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
    int fs_hash = kFsSha256;  // transcript hash (FiatShamir_hash_type)
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

// ------------------------------------------------------------------ lanes
// One device worker's state: its stream, pinned staging buffers, launch accounting.
constexpr size_t kMinMapped = 2u << 20;  // mapped staging per lane: enough for 16384 copies of M31
struct Lane {
    gkrgpu_ctx* X = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t done_ev = nullptr;
    PinnedBuf h_evals, h_rows, h_vx, h_cv, h_flag;

    struct Rec {
        int kid;
        size_t e0, e1;
        double bytes;
        uint32_t tag;
        double host_ms;  // host clock at the launch call, ms after the context's epoch
    };
    // (layer << 16) | (phase << 8) | round of the launches that follow, for the trace
    uint32_t tag = 0;
    std::vector<cudaEvent_t> events;
    size_t ev_used = 0;
    std::vector<Rec> recs;
    uint64_t job_launches[K_NUM_KERNELS] = {};
    double job_bytes[K_NUM_KERNELS] = {};

    // Host-mapped staging: the round evaluations written by the finishing CTAs, then an extra
    // area for the other small transfers of a proof (rows, claims, vx, the input check flag;
    // moved by kernels, so the lane's stream never queues behind another proof's bulk copies
    // on the copy engine), then the completion counter the kernels increment (RedScratch::done).
    char* map_h = nullptr;
    char* map_d = nullptr;
    size_t map_cap = 0, map_extra = 0;
    uint32_t done_seen = 0;
    // algorithmic bytes launched since the last wait, and when the first of them was launched
    double pending_bytes = 0;
    int X_lanes = 1;  // the context's lane count when this lane's worker started
    std::chrono::steady_clock::time_point pending_t0;
    // tail kernels: tags of their mailbox challenges (never reused within a lane) and the
    // mapped word a tail kernel sets when one of its waits expires (null: no tail running)
    uint32_t tail_tag = 0;
    const volatile uint32_t* tail_err = nullptr;
    uint32_t* evals_h() const { return reinterpret_cast<uint32_t*>(map_h); }
    uint32_t* evals_d() const { return reinterpret_cast<uint32_t*>(map_d); }
    char* extra_h() const { return map_h + map_extra; }
    char* extra_d() const { return map_d + map_extra; }
    unsigned int* done_d() const { return reinterpret_cast<unsigned int*>(map_d + map_cap - 256); }
    volatile uint32_t* done_h() const { return reinterpret_cast<volatile uint32_t*>(map_h + map_cap - 256); }
    // The stream must be idle (a new block resets the counter).
    void ensure_mapped(size_t evals_bytes, size_t extra_bytes = 0) {
        const size_t ev = align_up(evals_bytes, 256), ex = align_up(extra_bytes, 256);
        if (map_h && ev <= map_extra && map_extra + ex + 256 <= map_cap) return;
        // at least kMinMapped bytes at once: freeing a pinned block synchronizes the whole device,
        // so a lane should not grow it proof by proof
        const size_t ev_new = std::max({ev, map_extra, kMinMapped / 4}),
                     ex_new = std::max({ex, map_h ? map_cap - 256 - map_extra : 0, kMinMapped - kMinMapped / 4});
        const size_t need = ev_new + ex_new + 256;
        if (map_h) cudaFreeHost(map_h);
        map_h = map_d = nullptr;
        map_cap = map_extra = 0;
        void* p = nullptr;
        ck(cudaHostAlloc(&p, need, cudaHostAllocMapped | cudaHostAllocPortable), "mapped staging allocation");
        map_h = static_cast<char*>(p);
        void* d = nullptr;
        ck(cudaHostGetDevicePointer(&d, p, 0), "cudaHostGetDevicePointer");
        map_d = static_cast<char*>(d);
        map_cap = need;
        map_extra = ev_new;
        memset(map_h, 0, need);
        done_seen = 0;
    }
    // The stream is idle: take the counter as consumed.
    void resync_done() { done_seen = *done_h(); }
    // Waits until `groups` more finishing CTAs have published their results.  A stream that
    // went idle or failed without them is an error; the wait is bounded.
    void wait_done(uint32_t groups) {
        const uint32_t target = done_seen + groups;
        // Sleep through most of the expected run time of what was launched since the last
        // wait (its algorithmic bytes at about the copy peak, woken early), then spin: a lane
        // thread spinning through a long kernel takes a core from the host stages' hashing.
        if (pending_bytes > 0 && (int32_t)(*done_h() - target) < 0) {
            const auto wake = pending_t0 + std::chrono::nanoseconds((int64_t)(pending_bytes / 7.5e3));
            if (wake - std::chrono::steady_clock::now() > std::chrono::microseconds(30))
                std::this_thread::sleep_until(wake);
        }
        pending_bytes = 0;
        const auto t0 = std::chrono::steady_clock::now();
        // With several lanes the host cores are shared with the host stages' hashing: after a
        // short spin, poll in 10 us sleeps instead of spinning.
        const bool share_cores = X_lanes >= 4;
        for (uint64_t it = 0;; it++) {
            if ((int32_t)(*done_h() - target) >= 0) break;
            if (share_cores && it >= 2048) std::this_thread::sleep_for(std::chrono::microseconds(10));
            if ((it & 1023) == 1023 || (share_cores && it >= 2048)) {
                const cudaError_t e = cudaStreamQuery(stream);
                if (e != cudaSuccess && e != cudaErrorNotReady) ck(e, "round kernel");
                if (e == cudaSuccess && (int32_t)(*done_h() - target) < 0)
                    fail(GKRGPU_ERR_STATE, "round kernel finished without publishing its results");
                if (tail_err && *tail_err)
                    fail(GKRGPU_ERR_TIMEOUT, "a device wait for a round challenge expired");
                if (std::chrono::steady_clock::now() - t0 > std::chrono::seconds(60))
                    fail(GKRGPU_ERR_TIMEOUT, "round results not published within 60 s");
                std::this_thread::yield();
            }
        }
        std::atomic_thread_fence(std::memory_order_acquire);
        done_seen = target;
    }

    ~Lane() {
        if (map_h) cudaFreeHost(map_h);
        for (PinnedBuf* b : {&h_evals, &h_rows, &h_vx, &h_cv, &h_flag}) b->release();
        for (auto e : events) cudaEventDestroy(e);
        if (done_ev) cudaEventDestroy(done_ev);
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
    template <class F>
    void launch(int kid, double algo_bytes, F&& f);
    void resolve_events();
    void discard_job_stats() {
        recs.clear();
        ev_used = 0;
        for (int k = 0; k < K_NUM_KERNELS; k++) {
            job_launches[k] = 0;
            job_bytes[k] = 0;
        }
    }
    // Waits for the stream: short spin, then yields the core (many lanes may be waiting).
    void sync() {
        ck(cudaEventRecord(done_ev, stream), "cudaEventRecord");
        const auto t0 = std::chrono::steady_clock::now();
        for (;;) {
            const cudaError_t e = cudaEventQuery(done_ev);
            if (e == cudaSuccess) return;
            if (e != cudaErrorNotReady) ck(e, "cudaEventQuery");
            if (std::chrono::steady_clock::now() - t0 > std::chrono::microseconds(50)) std::this_thread::yield();
        }
    }
    void copy(void* dst, const void* src, size_t n, cudaMemcpyKind kind, const char* what);
};

// ------------------------------------------------------------------ context
struct gkrgpu_ctx {
    int device = 0;
    int sm_count = 152;
    // Row tile per kernel kind: threads per row slice (4 copies each) and CTA budget
    // (0 = the kind's default); chosen by gkrgpu_autotune or set with gkrgpu_set_tile.
    struct Tile {
        uint32_t tpr = 32, ctas = 0;
    };
    Tile tiles[K_NUM_KERNELS];
    uint32_t block = 256;

    // device memory: per-proof workspaces from a stream-ordered pool, admitted by budget
    cudaMemPool_t pool = nullptr;
    uint64_t hbm_budget = 0, hbm_in_use = 0, hbm_peak = 0;
    std::mutex mem_m;
    std::condition_variable mem_cv;

    // job pipeline: `n_lanes` device-stage workers, host-stage workers
    std::mutex qm;
    std::condition_variable qcv;
    std::deque<gkrgpu_job*> host_q, gpu_q;
    std::vector<std::thread> workers;
    std::vector<std::unique_ptr<Lane>> lanes;
    // host stages (commitment hash, grinding) run on host_workers threads (host_threads_set:
    // the caller's count, else max(4, min(lanes, 8))): the SHA-256 of a
    // large commitment is sequential, so several proofs' hashes overlap each other
    int n_lanes = 1, host_workers = 4, running = 0, host_threads_set = 0;
    int fs_hash = kFsSha256;  // transcript hash of jobs submitted from now on
    bool stopping = false;
    // the last rounds of a phase in one persistent launch (k_tail) when their tables are small
    bool round_tail = true;
    // copies of gkrgpu_upload: their own stream, so queued and running proofs go on
    std::mutex xfer_m;
    cudaStream_t xfer = nullptr;

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
        qcv.wait(lk, [&] { return gpu_q.empty() && running == 0; });
    }
    Lane& lane(int i) {
        while ((int)lanes.size() <= i) {
            auto L = std::make_unique<Lane>();
            L->X = this;
            ck(cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking), "cudaStreamCreate");
            ck(cudaEventCreateWithFlags(&L->done_ev, cudaEventDisableTiming), "cudaEventCreate");
            lanes.push_back(std::move(L));
        }
        return *lanes[i];
    }

    // launch accounting: totals read under stats_m; lanes fold each finished job in
    bool timing = false;
    std::atomic<uint64_t> h2d_bytes{0}, d2h_bytes{0};
    // timing markers: slots 0..63 hold gkrgpu_mark events and the device-stage ends of
    // proofs submitted with marker k (slot k); slots 64..127 the device-stage beginnings
    // of those proofs (slot 64 + k) and further gkrgpu_mark events
    cudaEvent_t markers[128] = {};
    std::mutex stats_m;
    uint64_t launches[K_NUM_KERNELS] = {};
    double ms[K_NUM_KERNELS] = {};
    double bytes[K_NUM_KERNELS] = {};
    // per-launch CSV (kernel, lane, layer, phase, round, algorithmic bytes, ms, device start
    // and host launch time in ms after the epoch) of timed jobs, appended to the file named by
    // the environment variable GKRGPU_TRACE
    FILE* trace = nullptr;
    cudaEvent_t epoch = nullptr;  // recorded at creation when tracing: the trace's time zero
    std::chrono::steady_clock::time_point epoch_host;
    int lane_index(const Lane* l) const {
        for (size_t k = 0; k < lanes.size(); k++)
            if (lanes[k].get() == l) return (int)k;
        return -1;
    }

    ~gkrgpu_ctx() {
        DeviceGuard g(device);
        lanes.clear();
        if (trace) fclose(trace);
        if (epoch) cudaEventDestroy(epoch);
        for (auto e : markers)
            if (e) cudaEventDestroy(e);
        if (xfer) cudaStreamDestroy(xfer);
        if (pool) cudaMemPoolDestroy(pool);
    }

    // Tile of kernel kind `kid` for N copies: the largest divisor of N/4 not above its tpr.
    Geo geo(uint32_t N, int kid) const {
        const uint32_t Q = N / 4;
        uint32_t tpr = Q;
        const uint32_t want = std::min<uint32_t>(tiles[kid].tpr, block);
        if (tpr > want) {
            tpr = want;
            while (tpr > 1 && Q % tpr) tpr--;
        }
        Geo g;
        g.N = N;
        g.tpr = tpr;
        g.rps = block / tpr;
        return g;
    }
    uint32_t cta_budget(int kid) const {
        if (tiles[kid].ctas) return tiles[kid].ctas;
        return (uint32_t)sm_count * (kid == K_EVALUATE ? 16u : 4u);
    }

    // Blocks until `bytes` fit in the budget (a proof larger than the whole budget runs alone).
    void acquire_hbm(uint64_t bytes) {
        std::unique_lock<std::mutex> lk(mem_m);
        mem_cv.wait(lk, [&] { return hbm_in_use == 0 || hbm_in_use + bytes <= hbm_budget; });
        hbm_in_use += bytes;
        hbm_peak = std::max(hbm_peak, hbm_in_use);
    }
    void release_hbm(uint64_t bytes) {
        {
            std::lock_guard<std::mutex> lk(mem_m);
            hbm_in_use -= bytes;
        }
        mem_cv.notify_all();
    }
};

template <class F>
void Lane::launch(int kid, double algo_bytes, F&& f) {
    if (pending_bytes == 0) pending_t0 = std::chrono::steady_clock::now();
    pending_bytes += algo_bytes;
    size_t e0 = 0;
    if (X->timing) {
        e0 = next_event();
        ck(cudaEventRecord(events[e0], stream), "cudaEventRecord");
    }
    ck(f(), kKernelNames[kid]);
    job_launches[kid]++;
    job_bytes[kid] += algo_bytes;
    if (X->timing) {
        const size_t e1 = next_event();
        ck(cudaEventRecord(events[e1], stream), "cudaEventRecord");
        const double host_ms =
            std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - X->epoch_host).count();
        recs.push_back({kid, e0, e1, algo_bytes, tag, host_ms});
    }
}

// Folds the finished job's launch counts, bytes and event times into the context's totals;
// the stream must be idle.
void Lane::resolve_events() {
    double t_ms[K_NUM_KERNELS] = {};
    std::vector<float> each(recs.size());
    for (size_t i = 0; i < recs.size(); i++) {
        const Rec& r = recs[i];
        ck(cudaEventElapsedTime(&each[i], events[r.e0], events[r.e1]), "cudaEventElapsedTime");
        t_ms[r.kid] += each[i];
    }
    std::vector<float> start(X->trace && X->epoch ? recs.size() : 0);
    for (size_t i = 0; i < start.size(); i++)
        ck(cudaEventElapsedTime(&start[i], X->epoch, events[recs[i].e0]), "cudaEventElapsedTime");
    std::lock_guard<std::mutex> lk(X->stats_m);
    if (X->trace) {
        const int li = X->lane_index(this);
        for (size_t i = 0; i < recs.size(); i++)
            fprintf(X->trace, "%s,%d,%u,%u,%u,%.0f,%.6f,%.4f,%.4f\n", kKernelNames[recs[i].kid], li, recs[i].tag >> 16,
                    (recs[i].tag >> 8) & 0xff, recs[i].tag & 0xff, recs[i].bytes, (double)each[i],
                    start.empty() ? -1.0 : (double)start[i], recs[i].host_ms);
        fflush(X->trace);
    }
    recs.clear();
    ev_used = 0;
    for (int k = 0; k < K_NUM_KERNELS; k++) {
        X->launches[k] += job_launches[k];
        X->bytes[k] += job_bytes[k];
        X->ms[k] += t_ms[k];
        job_launches[k] = 0;
        job_bytes[k] = 0;
    }
}

void Lane::copy(void* dst, const void* src, size_t n, cudaMemcpyKind kind, const char* what) {
    ck(cudaMemcpyAsync(dst, src, n, kind, stream), what);
    if (kind == cudaMemcpyHostToDevice) X->h2d_bytes += n;
    if (kind == cudaMemcpyDeviceToHost) X->d2h_bytes += n;
}

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

DevLayer upload_layer(const gkrgpu_layer_desc& d, int field) {
    const uint64_t I = 1ull << d.nb_input_vars, O = 1ull << d.nb_output_vars;
    const uint64_t Gm = d.n_mul, Ga = d.n_add;
    const bool bn = field == GKRGPU_FIELD_BN254;
    std::vector<uint32_t> keys, off_mo, off_ao, off_mx, off_ax, off_my, ord;
    std::vector<uint4> mo(Gm), mx(Gm), my(Gm);
    std::vector<uint2> ao(Ga), ax(Ga);
    // BN254: Montgomery coefficients per gate, then permuted into each table's order
    std::vector<frh::Fr> cm, ca, mo_c, mx_c, my_c, ao_c, ax_c;
    if (bn) {
        cm.resize(Gm);
        ca.resize(Ga);
        for (uint64_t i = 0; i < Gm; i++) cm[i] = frh::to_mont(frh::from_u32(d.mul[i].coef));
        for (uint64_t i = 0; i < Ga; i++) ca[i] = frh::to_mont(frh::from_u32(d.add[i].coef));
        mo_c.resize(Gm);
        mx_c.resize(Gm);
        my_c.resize(Gm);
        ao_c.resize(Ga);
        ax_c.resize(Ga);
    }

    keys.resize(Gm);
    for (uint64_t i = 0; i < Gm; i++) keys[i] = d.mul[i].o_id;
    csr(O, Gm, keys, off_mo, ord);
    for (uint64_t k = 0; k < Gm; k++) {
        const auto& g = d.mul[ord[k]];
        mo[k] = make_uint4(g.i0, g.i1, g.coef, 0);
        if (bn) mo_c[k] = cm[ord[k]];
    }
    for (uint64_t i = 0; i < Gm; i++) keys[i] = d.mul[i].i0;
    csr(I, Gm, keys, off_mx, ord);
    uint64_t h1_scalar = 0, h2_scalar = 0;
    for (uint64_t q = 0; q < I / 2; q++) h1_scalar += off_mx[2 * q] == off_mx[2 * q + 2];
    for (uint64_t q = 0; q < I / 4; q++) h2_scalar += off_mx[4 * q] == off_mx[4 * q + 4];
    for (uint64_t k = 0; k < Gm; k++) {
        const auto& g = d.mul[ord[k]];
        mx[k] = make_uint4(g.i1, g.o_id, g.coef, 0);
        if (bn) mx_c[k] = cm[ord[k]];
    }
    for (uint64_t i = 0; i < Gm; i++) keys[i] = d.mul[i].i1;
    csr(I, Gm, keys, off_my, ord);
    for (uint64_t k = 0; k < Gm; k++) {
        const auto& g = d.mul[ord[k]];
        my[k] = make_uint4(g.i0, g.o_id, g.coef, 0);
        if (bn) my_c[k] = cm[ord[k]];
    }
    keys.resize(Ga);
    for (uint64_t i = 0; i < Ga; i++) keys[i] = d.add[i].o_id;
    csr(O, Ga, keys, off_ao, ord);
    for (uint64_t k = 0; k < Ga; k++) {
        const auto& g = d.add[ord[k]];
        ao[k] = make_uint2(g.i0, g.coef);
        if (bn) ao_c[k] = ca[ord[k]];
    }
    for (uint64_t i = 0; i < Ga; i++) keys[i] = d.add[i].i0;
    csr(I, Ga, keys, off_ax, ord);
    for (uint64_t k = 0; k < Ga; k++) {
        const auto& g = d.add[ord[k]];
        ax[k] = make_uint2(g.o_id, g.coef);
        if (bn) ax_c[k] = ca[ord[k]];
    }

    // groups with gates (see DevLayer); a list is kept only when it leaves out more than a
    // tenth of the groups, since walking it costs a dependent load per group
    std::vector<uint32_t> l_p1_pairs, l_p1_quads, l_p2_quads;
    if (!bn) {
        auto gated = [](const std::vector<uint32_t>& off, uint64_t a, uint64_t b) { return off[b] > off[a]; };
        for (uint64_t q = 0; q < I / 2; q++)
            if (gated(off_mx, 2 * q, 2 * q + 2) || gated(off_ax, 2 * q, 2 * q + 2)) l_p1_pairs.push_back((uint32_t)q);
        for (uint64_t q = 0; q < I / 4; q++) {
            if (gated(off_mx, 4 * q, 4 * q + 4) || gated(off_ax, 4 * q, 4 * q + 4)) l_p1_quads.push_back((uint32_t)q);
            if (gated(off_my, 4 * q, 4 * q + 4)) l_p2_quads.push_back((uint32_t)q);
        }
    }
    const bool use_p1p = l_p1_pairs.size() * 10 <= (I / 2) * 9;
    const bool use_p1q = l_p1_quads.size() * 10 <= (I / 4) * 9;
    const bool use_p2q = l_p2_quads.size() * 10 <= (I / 4) * 9;

    struct Part {
        const void* src;
        size_t bytes;
        void** dst;
    };
    DevLayer L;
    L.n_p1_pairs = use_p1p ? l_p1_pairs.size() : I / 2;
    L.n_p1_quads = use_p1q ? l_p1_quads.size() : I / 4;
    L.n_p2_quads = use_p2q ? l_p2_quads.size() : I / 4;
    L.h1_scalar_rows = h1_scalar;
    L.h2_scalar_rows = h2_scalar;
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
    if (!bn && use_p1p) parts.push_back({l_p1_pairs.data(), l_p1_pairs.size() * 4, (void**)&L.p1_pairs});
    if (!bn && use_p1q) parts.push_back({l_p1_quads.data(), l_p1_quads.size() * 4, (void**)&L.p1_quads});
    if (!bn && use_p2q) parts.push_back({l_p2_quads.data(), l_p2_quads.size() * 4, (void**)&L.p2_quads});
    if (bn) {
        parts.push_back({mo_c.data(), Gm * 32, (void**)&L.mo_c});
        parts.push_back({ao_c.data(), Ga * 32, (void**)&L.ao_c});
        parts.push_back({mx_c.data(), Gm * 32, (void**)&L.mx_c});
        parts.push_back({ax_c.data(), Ga * 32, (void**)&L.ax_c});
        parts.push_back({my_c.data(), Gm * 32, (void**)&L.my_c});
    }
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

void validate_layers(const gkrgpu_layer_desc* layers, int n, int field) {
    if (!field_supported(field)) fail(GKRGPU_ERR_INVALID, "unsupported field type %d (M31 = 0, BN254 = 2)", field);
    // every u32 coefficient is a canonical BN254 element; M31 coefficients must be below p
    const uint32_t coef_limit = field == GKRGPU_FIELD_BN254 ? 0xffffffffu : m31::P - 1;
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
            if (m.o_id >= O || m.i0 >= I || m.i1 >= I || m.coef > coef_limit)
                fail(GKRGPU_ERR_INVALID, "layer %d mul gate %llu: id or coefficient out of range", l, (unsigned long long)g);
        }
        for (uint64_t g = 0; g < d.n_add; g++) {
            const auto& a = d.add[g];
            if (a.o_id >= O || a.i0 >= I || a.coef > coef_limit)
                fail(GKRGPU_ERR_INVALID, "layer %d add gate %llu: id or coefficient out of range", l, (unsigned long long)g);
        }
    }
}

// ------------------------------------------------------------------ per-proof device workspace
// All device tables of one proof, carved from one pool block (256-byte aligned parts).
struct Workspace {
    uint32_t* vals = nullptr;  // every layer's values (the input's rows excluded when it is on the device)
    uint32_t *hg0[3] = {}, *hgA[3] = {}, *fA[3] = {}, *fB[3] = {};
    uint32_t* sb[2] = {};
    uint32_t *eqc = nullptr, *eqrx = nullptr, *evals = nullptr, *vx = nullptr, *cv = nullptr;
    uint32_t* p2s = nullptr;  // 9R x N sums of phase-two rounds 0 and 1 (launch_p2_round01)
    uint4 *a4 = nullptr, *w4 = nullptr, *w4r = nullptr;
    unsigned long long* acc = nullptr;
    unsigned int* ticket = nullptr;
    unsigned int* flag = nullptr;
    size_t zero_off = 0, zero_bytes = 0;  // acc + ticket + flag: zeroed at the start of a proof
    size_t sstride = 0;
    size_t total = 0;

    // Lays the parts out from `base` (null: only sizes the block).
    void plan(char* base, const gkrgpu_circuit& C, uint32_t N, int R, bool own_input, bool sumcheck) {
        size_t o = 0;
        auto take = [&](size_t bytes) -> char* {
            char* p = base ? base + o : nullptr;
            o += align_up(std::max<size_t>(bytes, 16), 256);
            return p;
        };
        const uint64_t rowb = (uint64_t)N * 4;
        const uint64_t maxI = 1ull << C.max_in_vars, maxO = 1ull << C.max_out_vars;
        const uint64_t rows = C.value_rows() - (own_input ? 0 : C.in_rows(0));
        vals = (uint32_t*)take(rows * rowb);
        if (sumcheck) {
            for (int j = 0; j < R; j++) {
                hg0[j] = (uint32_t*)take(std::max<uint64_t>(maxI / 4, 1) * rowb);  // rounds >= 2 only
                hgA[j] = (uint32_t*)take(std::max<uint64_t>(maxI / 2, 1) * rowb);
                fA[j] = (uint32_t*)take(std::max<uint64_t>(maxI / 2, 1) * rowb);
                fB[j] = (uint32_t*)take(std::max<uint64_t>(maxI / 4, 1) * rowb);
            }
            sstride = align_up(maxI, 64);
            sb[0] = (uint32_t*)take(R * sstride * 4);
            sb[1] = (uint32_t*)take(R * sstride * 4);
            eqrx = (uint32_t*)take(R * maxI * 4);
            a4 = (uint4*)take(maxI * 16);
            w4 = (uint4*)take(std::max<uint64_t>(C.max_mul, 1) * 16);
            w4r = (uint4*)take(std::max<uint64_t>(C.max_mul, 1) * 16);
            p2s = (uint32_t*)take(27ull * N * 4);
        }
        eqc = (uint32_t*)take(R * maxO * 4);
        evals = (uint32_t*)take(9ull * N * 4);
        vx = (uint32_t*)take(3ull * N * 4);
        cv = (uint32_t*)take(3ull * N * 4);
        zero_off = o;
        acc = (unsigned long long*)take(27ull * N * 8);  // up to 9R components (launch_p2_round01)
        ticket = (unsigned int*)take(4096);
        flag = (unsigned int*)take(16);
        zero_bytes = o - zero_off;
        total = o;
    }
};

uint64_t workspace_bytes(const gkrgpu_circuit& C, uint32_t N, int R, bool own_input, bool sumcheck) {
    Workspace w;
    w.plan(nullptr, C, N, R, own_input, sumcheck);
    return w.total;
}

// ------------------------------------------------------------------ prover
struct Prover {
    gkrgpu_ctx& X;
    Lane& c;
    const gkrgpu_circuit& C;
    uint32_t N;
    int R;
    Geo gk[K_NUM_KERNELS];
    uint32_t ck_ctas[K_NUM_KERNELS];
    Workspace ws;
    char* block = nullptr;
    std::vector<uint32_t*> vals;  // vals[l]: input of layer l; vals[L]: output of the last layer
    // the layer's sum is alpha cv1 + beta cv2: the claimed values and zero for the output
    // layer, then the previous layer's vx and vy (R x N each)
    std::vector<uint32_t> cv1, cv2;

    Prover(gkrgpu_ctx& ctx, Lane& lane, const gkrgpu_circuit& circ, uint32_t n, int reps)
        : X(ctx), c(lane), C(circ), N(n), R(reps) {
        for (int k = 0; k < K_NUM_KERNELS; k++) {
            gk[k] = ctx.geo(n, k);
            ck_ctas[k] = ctx.cta_budget(k);
        }
    }
    ~Prover() {
        // a tail kernel still waiting for a challenge returns at once
        if (tail_running) {
            mbox_h()[0] = 1u;
            std::atomic_thread_fence(std::memory_order_seq_cst);
        }
        c.tail_err = nullptr;
        if (block) cudaFreeAsync(block, c.stream);
    }

    // Rounds kt .. n-1 of a phase in one k_tail launch: after each round's evaluations the
    // host appends them, derives the challenges and writes them to the mailbox, from which
    // the kernel's next round reads them.  The last round's rows 0..1 come with its
    // evaluations (vx / vy as in transcript_round).
    void run_tail(Transcript& t, bool lane_hg, uint32_t kt, uint32_t n, uint32_t (*rch)[32], uint32_t* const* fA,
                  uint32_t* const* fB, uint32_t* const* hA, uint32_t* const* hB, bool append_last, uint32_t* last_out,
                  double bytes) {
        TailArgs a;
        memset(&a, 0, sizeof(a));
        for (int j = 0; j < R; j++) {
            a.fA[j] = fA[j];
            a.fB[j] = fB[j];
            a.hA[j] = hA[j];
            a.hB[j] = hB[j];
            a.r_first[j] = rch[j][kt - 1];
        }
        a.vx = lane_hg ? nullptr : ws.vx;
        a.kt = kt;
        a.n = n;
        a.reps = (uint32_t)R;
        a.tag_base = c.tail_tag;
        c.tail_tag += kMboxRounds;
        a.mbox = mapped(true, 12ull * N + 64);
        a.evals_out = c.evals_d();
        a.rows_out = mapped(true, 0);
        a.done = c.done_d();
        a.err = mapped(true, 12ull * N + 1);
        a.wait_ns = 10ull * 1000 * 1000 * 1000;
        a.g = tail_geo(N);
        const uint32_t groups = N / (4 * a.g.tpr);
        volatile uint32_t* mb = mbox_h();
        mb[0] = 0u;
        *err_h() = 0u;
        std::atomic_thread_fence(std::memory_order_seq_cst);
        c.launch(K_TAIL, bytes, [&] { return launch_tail(lane_hg, a, c.stream); });
        c.pending_bytes = 0;  // its rounds are short and each waits for the host: no sleeping
        tail_running = true;
        c.tail_err = err_h();
        for (uint32_t k = kt; k < n; k++) {
            c.wait_done(groups);
            const bool last = k + 1 == n;
            transcript_round(t, rch, k, last, append_last, last_out);
            if (!last) {
                for (int j = 0; j < R; j++) mb[4 + 4 * k + 1 + j] = rch[j][k];
                std::atomic_thread_fence(std::memory_order_release);
                mb[4 + 4 * k] = a.tag_base + k;
                std::atomic_thread_fence(std::memory_order_seq_cst);
            }
        }
        tail_running = false;
        c.tail_err = nullptr;
    }
    // First round of a phase's tail, n if the phase has none: the rounds whose source tables
    // have at most tail_max_rows rows, from round `first` on.
    uint32_t tail_start(uint32_t n, uint32_t first, bool lane_hg) const {
        if (!X.round_tail || n < first + 1) return n;
        const uint32_t mr = tail_max_rows(N, R, lane_hg);
        uint32_t lg = 0;
        while ((1u << (lg + 1)) <= mr) lg++;
        // source rows of round k: 2^(n - k + 1) <= mr  <=>  k >= n + 1 - lg
        const uint32_t k0 = n + 1 > lg ? n + 1 - lg : 0;
        const uint32_t kt = std::max(first, k0);
        return kt < n ? kt : n;
    }

    RedScratch red() const { return RedScratch{ws.acc, ws.ticket}; }
    // Round kernels publish their evaluations into the lane's mapped staging buffer and keep a
    // device copy (ws.evals), from which the next round takes its claim.
    RedScratch red_mapped() const { return RedScratch{ws.acc, ws.ticket, c.done_d(), ws.evals}; }
    // The lane's mapped extra area: rows 0..1 of each repetition's last table (6N words), the
    // claimed values (3N), vx (3N), the input check flag, the tail kernels' error word and
    // mailbox, and the claims of phase one's round 0 (3N).
    uint32_t* mapped(bool dev, uint64_t word) const {
        return reinterpret_cast<uint32_t*>(dev ? c.extra_d() : c.extra_h()) + word;
    }
    uint32_t* rows_h() const { return mapped(false, 0); }
    uint32_t* cv_h() const { return mapped(false, 6ull * N); }
    uint32_t* vx_h() const { return mapped(false, 9ull * N); }
    volatile uint32_t* flag_h() const { return mapped(false, 12ull * N); }
    // tail kernels: error word and challenge mailbox
    volatile uint32_t* err_h() const { return mapped(false, 12ull * N + 1); }
    volatile uint32_t* mbox_h() const { return mapped(false, 12ull * N + 64); }
    // phase-one round 0's claims (R x N), after the mailbox
    uint64_t claim_word() const { return align_up(12ull * N + 64 + kMboxWords, 64); }
    uint64_t mapped_words() const { return claim_word() + 3ull * N; }
    bool tail_running = false;
    // Moves nsrc tables of n words into dst with k_stage_words (launch accounting as stage_words);
    // returns the number of completion increments when `done` is given.
    uint32_t stage(uint32_t* dst, const uint32_t* const* srcs, uint32_t nsrc, uint64_t n, unsigned int* done) {
        uint32_t incs = 0;
        c.launch(K_STAGE, 8.0 * n * nsrc, [&] {
            cudaError_t e;
            incs = launch_stage_words(dst, srcs, nsrc, n, done, c.stream, &e);
            return e;
        });
        return done ? incs : 0;
    }
    uint32_t groups(int kid) const { return N / (4 * gk[kid].tpr); }

    void reserve(bool own_input, bool sumcheck) {
        ws.plan(nullptr, C, N, R, own_input, sumcheck);
        void* p = nullptr;
        ck(cudaMallocFromPoolAsync(&p, ws.total, X.pool, c.stream), "workspace allocation");
        block = static_cast<char*>(p);
        ws.plan(block, C, N, R, own_input, sumcheck);
        ck(cudaMemsetAsync(block + ws.zero_off, 0, ws.zero_bytes, c.stream), "cudaMemsetAsync");
        c.ensure_mapped(9ull * N * 4, mapped_words() * 4);
        c.resync_done();
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
            vals[l] = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(ws.vals) + off * rowb);
            off += (l < L) ? C.in_rows(l) : C.out_rows(L - 1);
        }
    }

    // The check writes its flag straight into mapped memory; the host reads it after the
    // stream has passed the claims (require_canonical).
    void check_input() {
        const uint64_t n = C.in_rows(0) * N;
        *flag_h() = 0u;
        std::atomic_thread_fence(std::memory_order_seq_cst);
        c.launch(K_CHECK, (double)n * 4, [&] { return launch_check_canonical(vals[0], n, mapped(true, 12ull * N), c.stream); });
    }
    void require_canonical() {
        if (*flag_h()) fail(GKRGPU_ERR_INVALID, "input contains a value >= 2^31 - 1");
    }

    void evaluate() {
        for (size_t l = 0; l < C.layers.size(); l++) {
            const DevLayer& Ly = C.layers[l];
            const uint64_t O = 1ull << Ly.nout;
            const double b = 4.0 * N * (2.0 * Ly.nmul + Ly.nadd + O) + 16.0 * Ly.nmul + 8.0 * Ly.nadd + 8.0 * (O + 1);
            c.tag = (uint32_t)l << 16;
            c.launch(K_EVALUATE, b, [&] {
                return launch_evaluate(vals[l], vals[l + 1], O, Ly.mo_off, Ly.mo_g, Ly.ao_off, Ly.ao_g,
                                       gk[K_EVALUATE], X.block, ck_ctas[K_EVALUATE], c.stream);
            });
        }
    }

    // Waits for the round's 3R evaluation rows (published by `groups` finishing CTAs into the
    // mapped staging buffer) and optionally for rows 0..1 of `rows_from` per repetition, which
    // a small kernel publishes into the mapped rows area the same way.
    void fetch(uint32_t groups, const uint32_t* const* rows_from, bool shared_rows) {
        uint32_t more = 0;
        if (rows_from) {
            const uint32_t* srcs[3];
            for (int j = 0; j < R; j++) srcs[j] = shared_rows ? rows_from[0] : rows_from[j];
            more = stage(mapped(true, 0), srcs, (uint32_t)R, 2ull * N, c.done_d());
        }
        c.wait_done(groups + more);
    }

    // Transcript step of one round for every repetition (sumcheck.hpp:74-96).  With
    // `last`, the final fold of rows 0..1 gives vx/vy, appended after rep j's challenge
    // when `append_last` (vx); vy is appended after all rounds.
    void transcript_round(Transcript& t, uint32_t (*rch)[32], uint32_t k, bool last, bool append_last,
                          uint32_t* last_out) {
        const uint64_t rowb = (uint64_t)N * 4;
        const char* ev = reinterpret_cast<const char*>(c.evals_h());
        if (R == 3 && !last) {
            const uint8_t* msgs[3] = {(const uint8_t*)ev, (const uint8_t*)ev + 3 * rowb, (const uint8_t*)ev + 6 * rowb};
            uint32_t r3[3];
            if (t.append_challenge3(msgs, 3 * rowb, r3)) {
                for (int j = 0; j < 3; j++) rch[j][k] = r3[j];
                return;
            }
        }
        for (int j = 0; j < R; j++) {
            t.append(ev + 3ull * j * rowb, 3 * rowb);
            const uint32_t r = t.challenge();
            rch[j][k] = r;
            if (last) {
                const uint32_t* f0 = rows_h() + 2ull * j * N;
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
        uint32_t* v = vals[li];
        uint32_t* vxh = vx_h();
        std::vector<uint32_t> vy((size_t)R * N);
        const uint64_t RN = (uint64_t)R * N;

        // phase one: eqc_j = alpha eq(rz1_j) + beta eq(rz2_j), gate weights, hg + round 0
        c.tag = ((uint32_t)li << 16) | (1u << 8);
        eq_table(ws.eqc, rz1, rz2, alpha, beta, m);
        const double wb = 32.0 * Ly.nmul + 20.0 * I + 8.0 * Ly.nadd + 4.0 * R * (Ly.nmul + Ly.nadd);
        c.launch(K_WEIGHTS, wb, [&] {
            return launch_weights(I, Ly.nmul, O, ws.eqc, Ly.mx_g, Ly.ax_off, Ly.ax_g, ws.a4, ws.w4, R, c.stream);
        });
        // round 0's claims, alpha v(rz1) + beta v(rz2) per repetition and copy
        // (sumcheck.hpp:129-132), while the eq table and the weights are computed
        {
            uint32_t* cl = mapped(false, claim_word());
            for (uint64_t i = 0; i < RN; i++) cl[i] = m31::add(m31::mul(alpha, cv1[i]), m31::mul(beta, cv2[i]));
            std::atomic_thread_fence(std::memory_order_seq_cst);
        }
        // round 0 only reduces hg; round 1 rebuilds it (k_hg_round1), so no full-width hg
        // table is ever written
        // pairs of input rows without gates have hg = 0 and are skipped
        const double np0 = (double)Ly.n_p1_pairs;
        const double hb = rb * (2.0 * np0 + Ly.nmul) + 32.0 * Ly.nmul + 44.0 * np0;
        c.launch(K_HG_ROUND0, hb, [&] {
            return launch_hg_round0(R, v, Ly.n_p1_pairs, Ly.p1_pairs, Ly.mx_off, Ly.mx_g, ws.a4, ws.w4,
                                    gk[K_HG_ROUND0], X.block, ck_ctas[K_HG_ROUND0], red_mapped(),
                                    mapped(true, claim_word()), c.evals_d(), c.stream);
        });
        const uint32_t* vsrc[1] = {v};
        fetch(groups(K_HG_ROUND0), n == 1 ? vsrc : nullptr, true);
        transcript_round(t, rx, 0, n == 1, true, vxh);

        const uint32_t* cur_f[3] = {v, v, v};
        const uint32_t* cur_h[3] = {nullptr, nullptr, nullptr};  // round 1 rebuilds hg
        // the last rounds, on small tables, run in one persistent launch (from round 4 on:
        // rounds 2 and 3 refold the input and recompute copy-independent hg rows)
        const uint32_t kt1 = tail_start(n, 4, true);
        for (uint32_t k = 1; k < n; k++) {
            if (k == kt1) {
                double bytes = 0;
                for (uint32_t kk = kt1; kk < n; kk++) bytes += rb * 3.0 * R * 4.0 * (double)(I >> (kk + 1));
                c.tag = ((uint32_t)li << 16) | (1u << 8) | k;
                run_tail(t, true, kt1, n, rx, ws.fA, ws.fB, ws.hgA, ws.hg0, true, vxh, bytes);
                break;
            }
            RoundPtrs p;
            memset(&p, 0, sizeof(p));
            for (int j = 0; j < R; j++) {
                p.fsrc[j] = cur_f[j];
                p.hsrc[j] = cur_h[j];
                p.fdst[j] = (k & 1) ? ws.fA[j] : ws.fB[j];
                p.hdst[j] = (k & 1) ? ws.hgA[j] : ws.hg0[j];
                p.r[j] = rx[j][k - 1];
            }
            const uint64_t npairs = I >> (k + 1);
            const double S = 4.0 * npairs;
            c.tag = ((uint32_t)li << 16) | (1u << 8) | k;
            int kid = K_ROUND_LANE;
            // with a round 2, round 1 stores no folded copies of the layer input (they would be
            // written once and read once): round 2 refolds v at the round-0 challenges
            const bool refold1 = n >= 3;
            if (k == 1) {
                // hg rebuilt from the weights: v read once, the gathers again, f and hg halves out
                kid = K_HG_ROUND1;
                if (refold1)
                    for (int j = 0; j < R; j++) p.fdst[j] = nullptr;
                const double f_out = refold1 ? 0.0 : (double)R * I / 2;
                // without stored folded copies, groups of four input rows without gates
                // (hg = 0) are skipped
                const uint32_t* quads = refold1 ? Ly.p1_quads : nullptr;
                const uint64_t nq = refold1 ? Ly.n_p1_quads : npairs;
                const double vin = 4.0 * nq;
                c.launch(K_WEIGHTS, 4.0 * (I + 1) + 32.0 * Ly.nmul, [&] {
                    return launch_scale_weights(I, Ly.mx_off, ws.w4, ws.w4r, p.r, R, c.stream);
                });
                c.launch(K_HG_ROUND1, rb * (vin + Ly.nmul + f_out + (double)R * I / 2 - (double)R * Ly.h1_scalar_rows) + 32.0 * Ly.nmul + 20.0 * vin, [&] {
                    return launch_hg_round1(R, v, nq, quads, Ly.mx_off, Ly.mx_g, ws.a4, ws.w4r, p, gk[K_HG_ROUND1],
                                            X.block, ck_ctas[K_HG_ROUND1], red_mapped(), c.evals_d(), c.stream);
                });
            } else if (k == 2 || k == 3) {
                // the previous round's hg rows whose input rows have no mul gates were not
                // stored: recomputed from the add weights at the earlier challenges
                p.hoff = Ly.mx_off;
                p.ha = ws.a4;
                for (int j = 0; j < R; j++) {
                    p.hr[0][j] = rx[j][0];
                    p.hr[1][j] = rx[j][1];
                }
                // rows not read (k = 2, 3) and not written (k = 2); a4 words and offsets instead
                const double in_sc = (double)R * (k == 2 ? Ly.h1_scalar_rows : Ly.h2_scalar_rows);
                const double out_sc = k == 2 ? (double)R * Ly.h2_scalar_rows : 0.0;
                const double span = k == 2 ? 2.0 : 4.0;
                const bool vref = k == 2 && refold1;
                if (vref)
                    for (int j = 0; j < R; j++) p.fsrc[j] = v;
                // f rows read: R S stored copies, or the 2 S input rows they fold (k_p1_round2
                // reads each once for the R repetitions)
                const double f_in = vref ? 2.0 * S : (double)R * S;
                const double hb2 = rb * (f_in + 2.0 * R * S - in_sc - out_sc) + in_sc * 16.0 * span + 20.0 * npairs * R;
                c.launch(K_ROUND_LANE, hb2, [&] {
                    return vref ? launch_p1_round2(R, p, npairs, gk[K_ROUND_LANE], X.block, ck_ctas[K_ROUND_LANE],
                                                   red_mapped(), c.evals_d(), c.stream)
                                : launch_round_hr((int)k, R, p, npairs, gk[K_ROUND_LANE], X.block,
                                                  ck_ctas[K_ROUND_LANE], red_mapped(), c.evals_d(), c.stream);
                });
            } else {
                c.launch(K_ROUND_LANE, rb * 3.0 * R * S, [&] {
                    return launch_round(R, false, true, true, p, npairs, nullptr, gk[K_ROUND_LANE], X.block,
                                        ck_ctas[K_ROUND_LANE], red_mapped(), c.evals_d(), c.stream);
                });
            }
            const bool last = (k == n - 1);
            fetch(groups(kid), last ? p.fdst : nullptr, false);
            transcript_round(t, rx, k, last, true, vxh);
            for (int j = 0; j < R; j++) {
                cur_f[j] = p.fdst[j];
                cur_h[j] = p.hdst[j];
            }
        }

        // phase two: h(y) = vx * s(y)
        c.tag = ((uint32_t)li << 16) | (2u << 8);
        eq_table(ws.eqrx, rx, nullptr, 1u, 0u, n);
        const size_t sstride = ws.sstride;
        // with at least three rounds, rounds 0 and 1 come from one pass over the layer input
        // (their sums are quadratic in round 0's challenge) and round 2 refolds the input
        const bool fused01 = n >= 3 && p2_round01_groups(N) > 0;
        const bool refold = n >= 3;
        c.launch(K_S_BUILD, 16.0 * Ly.nmul + 4.0 * I + 4.0 * R * I + 8.0 * R * Ly.nmul + (fused01 ? 4.0 * R * I : 0.0),
                 [&] {
                     return fused01 ? launch_s_build4(I, O, Ly.my_off, Ly.my_g, ws.eqc, ws.eqrx, ws.sb[0], ws.sb[1],
                                                      sstride, R, c.stream)
                                    : launch_s_build(I, O, Ly.my_off, Ly.my_g, ws.eqc, ws.eqrx, ws.sb[0], sstride,
                                                     R, c.stream);
                 });
        {
            const uint32_t* src[1] = {mapped(true, 9ull * N)};
            stage(ws.vx, src, 1, (uint64_t)R * N, nullptr);
        }
        uint32_t k_first = 1;
        if (fused01) {
            const uint64_t ngroups = I / 4;
            const uint32_t* sj[3] = {ws.sb[0], ws.sb[0] + sstride, ws.sb[0] + 2 * sstride};
            const uint32_t* tj[3] = {ws.sb[1], ws.sb[1] + sstride, ws.sb[1] + 2 * sstride};
            // groups of four rows without mul gates on their second input (s = 0) are skipped
            const double rows2 = 4.0 * Ly.n_p2_quads;
            c.launch(K_P2_ROUND0, rb * rows2 + 8.0 * R * rows2 + 4.0 * 9 * R * N, [&] {
                return launch_p2_round01(R, v, sj, tj, Ly.n_p2_quads, Ly.p2_quads, ws.vx, N, ck_ctas[K_P2_ROUND0],
                                         red_mapped(), c.evals_d(), ws.p2s, c.stream);
            });
            fetch(p2_round01_groups(N), nullptr, true);
            transcript_round(t, ry, 0, false, false, vy.data());
            // round 1 from the sums; the scalar tables folded at ry_j[0] replace the pair sums
            c.tag = ((uint32_t)li << 16) | (2u << 8) | 1u;
            uint32_t* sd[3] = {ws.sb[1], ws.sb[1] + sstride, ws.sb[1] + 2 * sstride};
            uint32_t r0[3] = {ry[0][0], R > 1 ? ry[1][0] : 0u, R > 2 ? ry[2][0] : 0u};
            c.launch(K_ROUND_SCALAR, 4.0 * 9 * R * N + 4.0 * R * N + 6.0 * R * I, [&] {
                return launch_p2_round1_fin(R, ws.p2s, ws.vx, sj, sd, r0, ngroups, N, c.evals_d(), ws.evals,
                                            c.done_d(), c.stream);
            });
            fetch(1, nullptr, false);
            transcript_round(t, ry, 1, false, false, vy.data());
            k_first = 2;
        } else {
            RoundPtrs p;
            memset(&p, 0, sizeof(p));
            p.fsrc[0] = v;
            for (int j = 0; j < R; j++) p.hsrc[j] = ws.sb[0] + j * sstride;
            const uint64_t npairs = I >> 1;
            c.launch(K_P2_ROUND0, rb * 2.0 * npairs + 8.0 * R * npairs, [&] {
                return launch_round(R, true, false, false, p, npairs, ws.vx, gk[K_P2_ROUND0], X.block,
                                    ck_ctas[K_P2_ROUND0], red_mapped(), c.evals_d(), c.stream);
            });
            fetch(groups(K_P2_ROUND0), n == 1 ? vsrc : nullptr, true);
            transcript_round(t, ry, 0, n == 1, false, vy.data());
        }
        for (int j = 0; j < R; j++) cur_f[j] = v;
        // phase two's tail from round 3 on (round 2 refolds the layer input)
        const uint32_t kt2 = refold ? tail_start(n, 3, false) : n;
        for (uint32_t k = k_first; k < n; k++) {
            if (k == kt2) {
                double bytes = 0;
                for (uint32_t kk = kt2; kk < n; kk++) {
                    const double S = 4.0 * (double)(I >> (kk + 1));
                    bytes += rb * (R * S + R * S / 2) + 6.0 * R * S;
                }
                uint32_t *sA[3], *sB[3];
                for (int j = 0; j < R; j++) {
                    sA[j] = ws.sb[1] + j * sstride;
                    sB[j] = ws.sb[0] + j * sstride;
                }
                c.tag = ((uint32_t)li << 16) | (2u << 8) | k;
                run_tail(t, false, kt2, n, ry, ws.fA, ws.fB, sA, sB, false, vy.data(), bytes);
                break;
            }
            RoundPtrs p;
            memset(&p, 0, sizeof(p));
            const int src = (k - 1) & 1, dst = k & 1;
            for (int j = 0; j < R; j++) {
                p.fsrc[j] = cur_f[j];
                p.fdst[j] = (k & 1) ? ws.fA[j] : ws.fB[j];
                p.hsrc[j] = ws.sb[src] + j * sstride;
                p.hdst[j] = ws.sb[dst] + j * sstride;
                p.r[j] = ry[j][k - 1];
            }
            const uint64_t npairs = I >> (k + 1);
            const double S = 4.0 * npairs;
            c.tag = ((uint32_t)li << 16) | (2u << 8) | k;
            // with a round 2, round 1 stores no folded copies (they would be written once and
            // read once): round 2 refolds the layer input
            if (k == 1 && refold)
                for (int j = 0; j < R; j++) p.fdst[j] = nullptr;
            if (k == 2 && refold) {
                for (int j = 0; j < R; j++) {
                    p.fsrc[j] = v;
                    p.hr[0][j] = ry[j][0];
                }
                const double b = rb * (2.0 * S + R * S / 2) + 6.0 * R * S;
                c.launch(K_ROUND_SCALAR, b, [&] {
                    return launch_p2_round2(R, p, npairs, ws.vx, gk[K_ROUND_SCALAR], X.block, ck_ctas[K_ROUND_SCALAR],
                                            red_mapped(), c.evals_d(), c.stream);
                });
            } else {
                const double b = rb * ((k == 1 ? 1.0 : R) * S + (k == 1 && refold ? 0.0 : R * S / 2)) + 6.0 * R * S;
                c.launch(K_ROUND_SCALAR, b, [&] {
                    return launch_round(R, k == 1, false, true, p, npairs, ws.vx, gk[K_ROUND_SCALAR], X.block,
                                        ck_ctas[K_ROUND_SCALAR], red_mapped(), c.evals_d(), c.stream);
                });
            }
            const bool last = (k == n - 1);
            fetch(groups(K_ROUND_SCALAR), last ? p.fdst : nullptr, false);
            transcript_round(t, ry, k, last, false, vy.data());
            for (int j = 0; j < R; j++) cur_f[j] = p.fdst[j];
        }
        for (int j = 0; j < R; j++) t.append(vy.data() + (size_t)j * N, rowb);
        // the next layer's sum is alpha vx + beta vy (gkr.hpp:113-119)
        cv1.assign(vxh, vxh + RN);
        cv2.swap(vy);
    }

    // Device front half of a proof: workspace, input upload and check, Circuit::evaluate of
    // every layer.  Asynchronous on the lane's stream; it needs no transcript.
    void device_front(const uint32_t* h_input, const uint32_t* d_input) {
        const uint64_t in_bytes = C.in_rows(0) * (uint64_t)N * 4;
        reserve(d_input == nullptr, true);
        layout_values(d_input);
        if (h_input && !d_input) c.copy(vals[0], h_input, in_bytes, cudaMemcpyHostToDevice, "input upload");
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
        eq_table(ws.eqc, rz1, nullptr, 1u, 0u, nz);
        const uint64_t OL = C.out_rows(L - 1);
        c.launch(K_WSUM, 4.0 * N * OL + 4.0 * R * OL, [&] {
            return launch_wsum(R, vals[L], OL, ws.eqc, gk[K_WSUM], X.block, ck_ctas[K_WSUM], red(),
                               mapped(true, 6ull * N), c.stream);
        });
        c.sync();
        require_canonical();
        memcpy(claimed_v, cv_h(), R * rowb);
        cv1.assign(claimed_v, claimed_v + (size_t)R * N);
        cv2.assign((size_t)R * N, 0u);

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
        reserve(true, false);
        layout_values(nullptr);
        c.copy(vals[0], h_input, C.in_rows(0) * rowb, cudaMemcpyHostToDevice, "input upload");
        check_input();
        evaluate();
        c.sync();
        require_canonical();
        const size_t L = C.layers.size();
        if (all_layers) {
            c.copy(out, vals[0], C.value_rows() * rowb, cudaMemcpyDeviceToHost, "values readback");
        } else {
            c.copy(out, vals[L], C.out_rows(L - 1) * rowb, cudaMemcpyDeviceToHost, "output readback");
        }
        c.sync();
        c.resolve_events();
    }
};

#include "bn254_prover.cuh"
#include "verifier.cuh"

void check_ctx(gkrgpu_ctx* ctx) {
    if (!ctx) fail(GKRGPU_ERR_INVALID, "null context");
}

void check_run(gkrgpu_ctx* ctx, const gkrgpu_circuit* circuit, uint32_t n_copies) {
    check_ctx(ctx);
    if (!circuit) fail(GKRGPU_ERR_INVALID, "null circuit");
    if (circuit->device != ctx->device) fail(GKRGPU_ERR_INVALID, "circuit was loaded on another device");
    if (circuit->field == GKRGPU_FIELD_BN254) {
        // one thread per copy: any count whose row tiles leave at most 1024 lane groups
        if (n_copies < 1 || n_copies > (1u << 16)) fail(GKRGPU_ERR_INVALID, "n_copies must be in [1, 65536], got %u", n_copies);
        for (int k = K_BN_LOAD; k < K_NUM_KERNELS; k++)
            if (n_copies / geo_bn(*ctx, n_copies, k).tpr > 1024)
                fail(GKRGPU_ERR_INVALID, "more than 1024 lane groups for %u copies; raise threads_per_row", n_copies);
        return;
    }
    if (n_copies < 4 || n_copies % 4 || n_copies > (1u << 16))
        fail(GKRGPU_ERR_INVALID, "n_copies must be a multiple of 4 in [4, 65536], got %u", n_copies);
    const uint32_t Q = n_copies / 4;
    for (int k = 0; k < K_BN_LOAD; k++) {
        const Geo g = ctx->geo(n_copies, k);
        if (g.tpr * (Q / g.tpr) != Q) fail(GKRGPU_ERR_INVALID, "no row tile divides %u copies", n_copies);
        if (Q / g.tpr > 1024) fail(GKRGPU_ERR_INVALID, "more than 1024 lane groups; raise threads_per_row");
    }
}

// Commitment (the input rows) + grinding + per layer R x (2n rounds x 3 rows + vx + vy).
uint64_t proof_bytes(const gkrgpu_circuit* c, uint32_t N, int R) {
    const uint64_t eb = elem_bytes(c->field);
    uint64_t rows = 0;
    for (const auto& l : c->layers) rows += (uint64_t)R * (6ull * l.nin + 2);
    return c->in_rows(0) * N * eb + 32 + rows * N * eb;
}

// ------------------------------------------------------------------ job pipeline
// A proof is two stages: the host stage (RAW commitment bytes into the proof buffer, their
// SHA-256, grinding) and the device stage (workspace, upload, evaluate, then gkr_prove
// resuming the transcript).  Host workers run host stages in submission order; each lane
// worker takes the next queued device stage once the proof's workspace fits the budget.

// Copies n bytes in helper threads while this thread hashes the source.
void parallel_copy_and_hash(uint8_t* dst, const uint8_t* src, uint64_t n, int hash, uint8_t digest[32]) {
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
    fs_hash(hash, src, n, digest);
    for (auto& t : th) t.join();
}

TranscriptState host_stage(gkrgpu_ctx& c, gkrgpu_job& j, cudaStream_t s) {
    const bool bn = j.circuit->field == GKRGPU_FIELD_BN254;
    const uint64_t in_bytes = j.circuit->in_rows(0) * (uint64_t)j.N * elem_bytes(j.circuit->field);
    uint8_t d[32];
    if (j.h_input) {
        parallel_copy_and_hash(j.proof_out, reinterpret_cast<const uint8_t*>(j.h_input), in_bytes, j.fs_hash, d);
    } else {
        // the commitment is read back in chunks; SHA-256 hashes each chunk as it lands
        const uint64_t chunk = 64ull << 20, nch = (in_bytes + chunk - 1) / chunk;
        std::vector<cudaEvent_t> evs(nch, nullptr);
        struct Evs {
            std::vector<cudaEvent_t>& v;
            ~Evs() {
                for (auto e : v)
                    if (e) cudaEventDestroy(e);
            }
        } guard{evs};
        const uint8_t* src = reinterpret_cast<const uint8_t*>(j.d_input);
        for (uint64_t k = 0; k < nch; k++) {
            const uint64_t a = k * chunk, n = std::min(chunk, in_bytes - a);
            ck(cudaEventCreateWithFlags(&evs[k], cudaEventDisableTiming), "cudaEventCreate");
            ck(cudaMemcpyAsync(j.proof_out + a, src + a, n, cudaMemcpyDeviceToHost, s), "commitment readback");
            ck(cudaEventRecord(evs[k], s), "cudaEventRecord");
        }
        if (j.fs_hash == kFsSha256) {
            Sha256 h;
            for (uint64_t k = 0; k < nch; k++) {
                const uint64_t a = k * chunk, n = std::min(chunk, in_bytes - a);
                ck(cudaEventSynchronize(evs[k]), "commitment readback");
                h.update(j.proof_out + a, n);
            }
            h.final(d);
        } else {
            ck(cudaStreamSynchronize(s), "commitment readback");
            fs_hash(j.fs_hash, j.proof_out, in_bytes, d);
        }
        c.d2h_bytes += in_bytes;
    }
    Transcript t(j.proof_out, ~0ull, j.fs_hash);
    t.appended_prehashed(in_bytes, d);
    if (bn)
        grind_bn254(t, j.grinding);
    else
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

void gpu_worker(gkrgpu_ctx* c, Lane* lane) {
    cudaSetDevice(c->device);
    lane->X_lanes = c->n_lanes;
#ifdef __linux__
    // wake from the sleeps of Lane::wait_done within a microsecond of the requested time
    prctl(PR_SET_TIMERSLACK, 1000UL, 0, 0, 0);
#endif
    for (;;) {
        gkrgpu_job* j;
        {
            std::unique_lock<std::mutex> lk(c->qm);
            c->qcv.wait(lk, [&] { return c->stopping || !c->gpu_q.empty(); });
            if (c->gpu_q.empty()) break;
            j = c->gpu_q.front();
            c->gpu_q.pop_front();
            c->running++;
        }
        int rc = GKRGPU_OK;
        std::string err;
        const bool bn = j->circuit->field == GKRGPU_FIELD_BN254;
        const uint64_t need = bn ? workspace_bytes_bn(*j->circuit, j->N, true)
                                 : workspace_bytes(*j->circuit, j->N, j->R, j->d_input == nullptr, true);
        c->acquire_hbm(need);
        if (j->marker >= 0) {
            // the device stage begins: this lane's stream has finished its previous proof
            std::lock_guard<std::mutex> lk(c->stats_m);
            cudaEvent_t& ev = c->markers[64 + j->marker];
            if (!ev) cudaEventCreate(&ev);
            if (ev) cudaEventRecord(ev, lane->stream);
        }
        try {
            auto wait_host = [&] {
                std::unique_lock<std::mutex> lk(j->m);
                j->cv.wait(lk, [&] { return j->host_done; });
                if (j->host_rc) throw Error(j->host_rc, j->host_err);
            };
            auto wait_host_traced = [&] {
                if (!c->trace) return wait_host();
                const auto t0 = std::chrono::steady_clock::now();
                wait_host();
                const auto t1 = std::chrono::steady_clock::now();
                std::lock_guard<std::mutex> lk(c->stats_m);
                fprintf(c->trace, "host_stage_wait,%d,0,0,0,0,%.6f,-1,%.4f\n", c->lane_index(lane),
                        std::chrono::duration<double, std::milli>(t1 - t0).count(),
                        std::chrono::duration<double, std::milli>(t0 - c->epoch_host).count());
            };
            if (bn) {
                BnProver p(*c, *lane, *j->circuit, j->N);
                p.device_front(j->h_input, j->d_input);
                wait_host_traced();
                p.device_back(j->ts, j->proof_out, j->claimed_v);
            } else {
                Prover p(*c, *lane, *j->circuit, j->N, j->R);
                p.device_front(j->h_input, j->d_input);
                wait_host_traced();
                p.device_back(j->ts, j->proof_out, j->claimed_v);
            }
            if (j->marker >= 0) {
                std::lock_guard<std::mutex> lk(c->stats_m);
                if (!c->markers[j->marker]) ck(cudaEventCreate(&c->markers[j->marker]), "cudaEventCreate");
                ck(cudaEventRecord(c->markers[j->marker], lane->stream), "cudaEventRecord");
            }
        } catch (const Error& e) {
            rc = e.code;
            err = e.what();
        } catch (const std::exception& e) {
            rc = GKRGPU_ERR_STATE;
            err = e.what();
        }
        // The workspace was returned to the pool (stream-ordered) when the Prover went out of
        // scope; once the stream has passed that point the budget is released.
        cudaStreamSynchronize(lane->stream);
        if (rc != GKRGPU_OK) lane->discard_job_stats();
        c->release_hbm(need);
        {
            std::lock_guard<std::mutex> lk(j->m);
            j->rc = rc;
            j->err = err;
            j->done = true;
        }
        j->cv.notify_all();
        {
            std::lock_guard<std::mutex> lk(c->qm);
            c->running--;
        }
        c->qcv.notify_all();
    }
}

gkrgpu_job* submit(gkrgpu_ctx* ctx, const gkrgpu_circuit* circuit, uint32_t n_copies, int grinding_bits,
                   const uint32_t* h_input, const uint32_t* d_input, uint8_t* proof_out, uint64_t proof_cap,
                   uint32_t* claimed_v, int marker, uint64_t* need_out) {
    check_run(ctx, circuit, n_copies);
    if (grinding_bits < 0 || grinding_bits > 30) fail(GKRGPU_ERR_INVALID, "grinding_bits must be in [0, 30]");
    const int R = reps_for_field(circuit->field, grinding_bits);
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
    j->fs_hash = ctx->fs_hash;
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

// Runs f on lane 0 with every queued proof finished first (the synchronous entry points).
template <class F>
void on_idle_lane(gkrgpu_ctx* ctx, F&& f) {
    ctx->drain();
    std::lock_guard<std::mutex> lk(ctx->qm);  // keeps workers from starting while lane 0 is used
    DeviceGuard dg(ctx->device);
    f(ctx->lane(0));
}

}  // namespace

void gkrgpu_ctx::start_workers() {
    std::lock_guard<std::mutex> lk(qm);
    if (!workers.empty()) return;
    stopping = false;
    for (int i = 0; i < n_lanes; i++) workers.emplace_back(gpu_worker, this, &lane(i));
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
    static std::string v = std::string("gkrgpu 0.2 (sm_103a; host sha256: ") + sha256_impl_name() + ")";
    return v.c_str();
}

int gkrgpu_num_repetitions(int grinding_bits) { return reps_for(grinding_bits); }

int gkrgpu_num_repetitions_field(int field, int grinding_bits) {
    return field_supported(field) ? reps_for_field(field, grinding_bits) : -GKRGPU_ERR_INVALID;
}

uint32_t gkrgpu_field_bytes(int field) { return field_supported(field) ? elem_bytes(field) : 0u; }

int gkrgpu_create(int device, gkrgpu_ctx** out) {
    return guarded([&] {
        if (!out) fail(GKRGPU_ERR_INVALID, "null output");
        *out = nullptr;
        int n = 0;
        ck(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
        if (device < 0 || device >= n) fail(GKRGPU_ERR_INVALID, "device %d out of range (%d devices)", device, n);
        DeviceGuard dg(device);
        std::unique_ptr<gkrgpu_ctx> c(new gkrgpu_ctx());
        c->device = device;
        cudaDeviceProp prop;
        if (cudaGetDeviceProperties(&prop, device) == cudaSuccess) c->sm_count = prop.multiProcessorCount;
        size_t free_b = 0, total_b = 0;
        ck(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
        c->hbm_budget = (uint64_t)(free_b * 0.9);
        cudaMemPoolProps pp;
        memset(&pp, 0, sizeof(pp));
        pp.allocType = cudaMemAllocationTypePinned;
        pp.location.type = cudaMemLocationTypeDevice;
        pp.location.id = device;
        ck(cudaMemPoolCreate(&c->pool, &pp), "cudaMemPoolCreate");
        uint64_t keep = c->hbm_budget;
        ck(cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &keep), "cudaMemPoolSetAttribute");
        if (const char* tp = getenv("GKRGPU_TRACE"))
            if (*tp) c->trace = fopen(tp, "a");
        // Under a CUDA injection tool (a profiler) kernels may run one at a time with the
        // launching thread blocked until each finishes; a phase tail, which waits on the device
        // for its own host thread's challenges, would then only end at its wait limit.
        if (const char* inj = getenv("CUDA_INJECTION64_PATH"))
            if (*inj) c->round_tail = false;
        c->lane(0);
        if (c->trace) {
            ck(cudaEventCreate(&c->epoch), "cudaEventCreate");
            ck(cudaEventRecord(c->epoch, c->lane(0).stream), "cudaEventRecord");
            ck(cudaEventSynchronize(c->epoch), "cudaEventSynchronize");
            c->epoch_host = std::chrono::steady_clock::now();
        }
        *out = c.release();
    });
}

void gkrgpu_destroy(gkrgpu_ctx* ctx) {
    if (!ctx) return;
    try {
        ctx->shutdown();
        DeviceGuard dg(ctx->device);
        delete ctx;
    } catch (...) {
    }
}

int gkrgpu_set_concurrency(gkrgpu_ctx* ctx, int lanes, uint64_t hbm_budget_bytes) {
    return guarded([&] {
        check_ctx(ctx);
        if (lanes < 0 || lanes > 64) fail(GKRGPU_ERR_INVALID, "lanes must be in [1, 64] (0 keeps the current value)");
        ctx->drain();
        ctx->shutdown();
        DeviceGuard dg(ctx->device);
        if (lanes) {
            ctx->n_lanes = lanes;
            ctx->host_workers = ctx->host_threads_set ? ctx->host_threads_set : std::max(4, std::min(lanes, 8));
        }
        if (hbm_budget_bytes) {
            ctx->hbm_budget = hbm_budget_bytes;
            uint64_t keep = hbm_budget_bytes;
            ck(cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &keep), "cudaMemPoolSetAttribute");
        }
        {
            std::lock_guard<std::mutex> lk(ctx->qm);
            ctx->stopping = false;
        }
    });
}

int gkrgpu_set_host_threads(gkrgpu_ctx* ctx, int threads) {
    return guarded([&] {
        check_ctx(ctx);
        if (threads < 0 || threads > 64) fail(GKRGPU_ERR_INVALID, "threads must be in [1, 64] (0: the default)");
        ctx->drain();
        ctx->shutdown();
        ctx->host_threads_set = threads;
        ctx->host_workers = threads ? threads : std::max(4, std::min(ctx->n_lanes, 8));
        std::lock_guard<std::mutex> lk(ctx->qm);
        ctx->stopping = false;
    });
}

int gkrgpu_memory_stats(gkrgpu_ctx* ctx, uint64_t* in_use, uint64_t* peak, uint64_t* budget) {
    return guarded([&] {
        check_ctx(ctx);
        std::lock_guard<std::mutex> lk(ctx->mem_m);
        if (in_use) *in_use = ctx->hbm_in_use;
        if (peak) *peak = ctx->hbm_peak;
        if (budget) *budget = ctx->hbm_budget;
    });
}

uint64_t gkrgpu_workspace_bytes(const gkrgpu_circuit* circuit, uint32_t n_copies, int grinding_bits, int input_on_device) {
    if (!circuit) return 0;
    if (circuit->field == GKRGPU_FIELD_BN254) return workspace_bytes_bn(*circuit, n_copies, true);
    return workspace_bytes(*circuit, n_copies, reps_for(grinding_bits), input_on_device == 0, true);
}

int gkrgpu_circuit_load(gkrgpu_ctx* ctx, const gkrgpu_layer_desc* layers, int n_layers, gkrgpu_circuit** out) {
    return gkrgpu_circuit_load_field(ctx, layers, n_layers, GKRGPU_FIELD_M31, out);
}

int gkrgpu_circuit_field(const gkrgpu_circuit* circuit) { return circuit ? circuit->field : -GKRGPU_ERR_INVALID; }

int gkrgpu_circuit_load_field(gkrgpu_ctx* ctx, const gkrgpu_layer_desc* layers, int n_layers, int field,
                              gkrgpu_circuit** out) {
    return guarded([&] {
        check_ctx(ctx);
        if (!out) fail(GKRGPU_ERR_INVALID, "null output");
        *out = nullptr;
        validate_layers(layers, n_layers, field);
        DeviceGuard dg(ctx->device);
        gkrgpu_circuit* c = new gkrgpu_circuit();
        c->device = ctx->device;
        c->field = field;
        try {
            for (int l = 0; l < n_layers; l++) {
                c->layers.push_back(upload_layer(layers[l], field));
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
        on_idle_lane(ctx, [&](Lane& lane) {
            if (circuit->field == GKRGPU_FIELD_BN254) {
                BnProver p(*ctx, lane, *circuit, n_copies);
                p.evaluate_only(input, out, all_layers != 0);
            } else {
                Prover p(*ctx, lane, *circuit, n_copies, 1);
                p.evaluate_only(input, out, all_layers != 0);
            }
        });
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

int gkrgpu_prove_submit_resident(gkrgpu_ctx* ctx, const gkrgpu_circuit* circuit, uint32_t n_copies,
                                 int grinding_bits, const uint32_t* h_input, const uint32_t* d_input,
                                 uint8_t* proof_out, uint64_t proof_cap, uint32_t* claimed_v, int marker_slot,
                                 gkrgpu_job** job) {
    return guarded([&] {
        if (!job) fail(GKRGPU_ERR_INVALID, "null job output");
        *job = nullptr;
        if (!h_input || !d_input) fail(GKRGPU_ERR_INVALID, "both the host and the device copy of the input are needed");
        *job = submit(ctx, circuit, n_copies, grinding_bits, h_input, d_input, proof_out, proof_cap, claimed_v,
                      marker_slot, nullptr);
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

int gkrgpu_set_fs_hash(gkrgpu_ctx* ctx, int fs_hash_type) {
    return guarded([&] {
        check_ctx(ctx);
        if (fs_hash_type != kFsSha256 && fs_hash_type != kFsKeccak256)
            fail(GKRGPU_ERR_INVALID, "unsupported transcript hash %d (SHA256 = 0, Keccak256 = 1)", fs_hash_type);
        ctx->drain();
        ctx->fs_hash = fs_hash_type;
    });
}

int gkrgpu_verify(gkrgpu_ctx* ctx, const gkrgpu_circuit* circuit, uint32_t n_copies, int grinding_bits,
                  const uint8_t* proof, uint64_t proof_len, const uint32_t* claimed_v, int* accepted) {
    return guarded([&] {
        check_run(ctx, circuit, n_copies);
        if (!proof || !claimed_v || !accepted) fail(GKRGPU_ERR_INVALID, "null buffer");
        *accepted = 0;
        if (grinding_bits < 0 || grinding_bits > 30) fail(GKRGPU_ERR_INVALID, "grinding_bits must be in [0, 30]");
        const int R = reps_for_field(circuit->field, grinding_bits);
        if (R < 1 || R > 3) fail(GKRGPU_ERR_INVALID, "grinding_bits %d gives %d repetitions (1..3 supported)", grinding_bits, R);
        on_idle_lane(ctx, [&](Lane& lane) {
            if (circuit->field == GKRGPU_FIELD_BN254) {
                BnVerifier v(*ctx, lane, *circuit, n_copies);
                *accepted = v.run(grinding_bits, proof, proof_len, claimed_v) ? 1 : 0;
            } else {
                Verifier v(*ctx, lane, *circuit, n_copies, R);
                *accepted = v.run(grinding_bits, proof, proof_len, claimed_v) ? 1 : 0;
            }
        });
    });
}

int gkrgpu_eval_multilinear(gkrgpu_ctx* ctx, const uint32_t* d_evals, uint32_t nb_vars, uint32_t n_copies,
                            const uint32_t* r, int n_points, uint32_t* out) {
    return guarded([&] {
        check_ctx(ctx);
        if (!d_evals || !r || !out) fail(GKRGPU_ERR_INVALID, "null buffer");
        if ((uintptr_t)d_evals & 15) fail(GKRGPU_ERR_INVALID, "d_evals must be 16-byte aligned");
        if (n_points < 1 || n_points > 3) fail(GKRGPU_ERR_INVALID, "n_points must be in [1, 3]");
        if (nb_vars > 30) fail(GKRGPU_ERR_INVALID, "nb_vars must be <= 30");
        if (n_copies < 4 || n_copies % 4 || n_copies > (1u << 16))
            fail(GKRGPU_ERR_INVALID, "n_copies must be a multiple of 4 in [4, 65536]");
        for (int j = 0; j < n_points; j++)
            for (uint32_t t = 0; t < nb_vars; t++)
                if (r[(size_t)j * nb_vars + t] >= m31::P) fail(GKRGPU_ERR_INVALID, "point coordinate >= p");
        const Geo g = ctx->geo(n_copies, K_WSUM);
        if (g.tpr * ((n_copies / 4) / g.tpr) != n_copies / 4) fail(GKRGPU_ERR_INVALID, "no row tile divides n_copies");
        if ((n_copies / 4) / g.tpr > 1024) fail(GKRGPU_ERR_INVALID, "more than 1024 lane groups");
        on_idle_lane(ctx, [&](Lane& c) {
            const uint64_t rows = 1ull << nb_vars, rowb = (uint64_t)n_copies * 4;
            const size_t eq_b = align_up(n_points * rows * 4, 256), acc_b = align_up(9ull * n_copies * 8, 256);
            const size_t cv_b = align_up(3 * rowb, 256), total = eq_b + acc_b + 4096 + cv_b;
            void* p = nullptr;
            ck(cudaMallocFromPoolAsync(&p, total, ctx->pool, c.stream), "workspace allocation");
            char* base = static_cast<char*>(p);
            uint32_t* eq = reinterpret_cast<uint32_t*>(base);
            RedScratch red{reinterpret_cast<unsigned long long*>(base + eq_b),
                           reinterpret_cast<unsigned int*>(base + eq_b + acc_b)};
            uint32_t* cv = reinterpret_cast<uint32_t*>(base + eq_b + acc_b + 4096);
            struct Free {
                void* p;
                cudaStream_t s;
                ~Free() { cudaFreeAsync(p, s); }
            } guard{p, c.stream};
            ck(cudaMemsetAsync(base + eq_b, 0, acc_b + 4096, c.stream), "cudaMemsetAsync");
            c.h_cv.ensure(3 * rowb, "pinned claims");
            EqArgs a;
            memset(&a, 0, sizeof(a));
            for (int j = 0; j < n_points; j++) memcpy(a.r1[j], r + (size_t)j * nb_vars, 4 * nb_vars);
            a.f1 = 1u;
            a.nvars = nb_vars;
            a.reps = n_points;
            c.launch(K_EQ, 4.0 * n_points * rows, [&] { return launch_eq(eq, a, c.stream); });
            c.launch(K_WSUM, 4.0 * n_copies * rows + 4.0 * n_points * rows, [&] {
                return launch_wsum(n_points, d_evals, rows, eq, g, ctx->block, ctx->cta_budget(K_WSUM), red, cv,
                                   c.stream);
            });
            c.copy(c.h_cv.p, cv, n_points * rowb, cudaMemcpyDeviceToHost, "result readback");
            c.sync();
            memcpy(out, c.h_cv.p, n_points * rowb);
            c.resolve_events();
        });
    });
}

int gkrgpu_set_round_tail(gkrgpu_ctx* ctx, int enabled) {
    return guarded([&] {
        check_ctx(ctx);
        ctx->drain();
        ctx->round_tail = enabled != 0;
    });
}

int gkrgpu_check_device_wait(gkrgpu_ctx* ctx, uint32_t timeout_us, int* expired, int* rounds_published) {
    return guarded([&] {
        check_ctx(ctx);
        if (!expired || !rounds_published) fail(GKRGPU_ERR_INVALID, "null output");
        if (timeout_us < 1 || timeout_us > 10u * 1000 * 1000) fail(GKRGPU_ERR_INVALID, "timeout_us must be in [1, 10^7]");
        on_idle_lane(ctx, [&](Lane& c) {
            // a two-round tail over 8 x 4 tables whose second round's challenge is never written
            const uint32_t N = 4, n = 3, kt = 1;
            const size_t tb = 8 * N * 4;
            void* p = nullptr;
            ck(cudaMallocFromPoolAsync(&p, 4 * tb, ctx->pool, c.stream), "workspace allocation");
            struct Free {
                void* p;
                cudaStream_t s;
                ~Free() {
                    cudaFreeAsync(p, s);
                    cudaStreamSynchronize(s);
                }
            } guard{p, c.stream};
            ck(cudaMemsetAsync(p, 0, 4 * tb, c.stream), "cudaMemsetAsync");
            c.ensure_mapped(9ull * N * 4, (12ull * N + 64 + kMboxWords) * 4);
            c.resync_done();
            uint32_t* base_h = reinterpret_cast<uint32_t*>(c.extra_h());
            uint32_t* base_d = reinterpret_cast<uint32_t*>(c.extra_d());
            TailArgs a;
            memset(&a, 0, sizeof(a));
            char* b = static_cast<char*>(p);
            a.fA[0] = reinterpret_cast<uint32_t*>(b);
            a.fB[0] = reinterpret_cast<uint32_t*>(b + tb);
            a.hA[0] = reinterpret_cast<uint32_t*>(b + 2 * tb);
            a.hB[0] = reinterpret_cast<uint32_t*>(b + 3 * tb);
            a.kt = kt;
            a.n = n;
            a.reps = 1;
            a.tag_base = c.tail_tag;
            c.tail_tag += kMboxRounds;
            a.mbox = base_d + 12 * N + 64;
            a.evals_out = c.evals_d();
            a.rows_out = base_d;
            a.done = c.done_d();
            a.err = base_d + 12 * N + 1;
            a.wait_ns = (unsigned long long)timeout_us * 1000;
            a.g = tail_geo(N);
            volatile uint32_t* mb = base_h + 12 * N + 64;
            volatile uint32_t* err = base_h + 12 * N + 1;
            mb[0] = 0u;
            *err = 0u;
            std::atomic_thread_fence(std::memory_order_seq_cst);
            ck(launch_tail(true, a, c.stream), "round_tail");
            ck(cudaStreamSynchronize(c.stream), "round_tail");  // returns once the wait expires
            std::atomic_thread_fence(std::memory_order_acquire);
            *expired = *err ? 1 : 0;
            *rounds_published = (int)(*c.done_h() - c.done_seen);
            c.resync_done();
        });
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
        on_idle_lane(ctx, [&](Lane& c) {
            c.copy(dst, src, bytes, cudaMemcpyHostToDevice, "cudaMemcpyAsync");
            c.sync();
        });
    });
}

int gkrgpu_upload(gkrgpu_ctx* ctx, void* d_dst, const void* h_src, uint64_t bytes) {
    return guarded([&] {
        check_ctx(ctx);
        if (!d_dst || (!h_src && bytes)) fail(GKRGPU_ERR_INVALID, "null buffer");
        std::lock_guard<std::mutex> lk(ctx->xfer_m);
        DeviceGuard dg(ctx->device);
        if (!ctx->xfer) ck(cudaStreamCreateWithFlags(&ctx->xfer, cudaStreamNonBlocking), "cudaStreamCreate");
        ck(cudaMemcpyAsync(d_dst, h_src, bytes, cudaMemcpyHostToDevice, ctx->xfer), "cudaMemcpyAsync");
        ck(cudaStreamSynchronize(ctx->xfer), "cudaStreamSynchronize");
        ctx->h2d_bytes += bytes;
    });
}

int gkrgpu_memcpy_d2h(gkrgpu_ctx* ctx, void* dst, const void* src, uint64_t bytes) {
    return guarded([&] {
        check_ctx(ctx);
        on_idle_lane(ctx, [&](Lane& c) {
            c.copy(dst, src, bytes, cudaMemcpyDeviceToHost, "cudaMemcpyAsync");
            c.sync();
        });
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
        for (auto& l : ctx->lanes) l->discard_job_stats();
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
        if (slot < 0 || slot >= 128) fail(GKRGPU_ERR_INVALID, "marker slot must be in [0, 128)");
        on_idle_lane(ctx, [&](Lane& c) {
            std::lock_guard<std::mutex> lk(ctx->stats_m);
            if (!ctx->markers[slot]) ck(cudaEventCreate(&ctx->markers[slot]), "cudaEventCreate");
            ck(cudaEventRecord(ctx->markers[slot], c.stream), "cudaEventRecord");
        });
    });
}

int gkrgpu_elapsed_ms(gkrgpu_ctx* ctx, int from_slot, int to_slot, double* ms) {
    return guarded([&] {
        check_ctx(ctx);
        cudaEvent_t a, b;
        {
            std::lock_guard<std::mutex> lk(ctx->stats_m);
            if (!ms || from_slot < 0 || from_slot >= 128 || to_slot < 0 || to_slot >= 128 ||
                !ctx->markers[from_slot] || !ctx->markers[to_slot])
                fail(GKRGPU_ERR_INVALID, "unrecorded marker slot");
            a = ctx->markers[from_slot];
            b = ctx->markers[to_slot];
        }
        DeviceGuard dg(ctx->device);
        ck(cudaEventSynchronize(b), "cudaEventSynchronize");
        float t = 0.f;
        ck(cudaEventElapsedTime(&t, a, b), "cudaEventElapsedTime");
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

int gkrgpu_proof_write(const char* path, const uint8_t* proof, uint64_t proof_len) {
    return guarded([&] {
        if (!path || (!proof && proof_len)) fail(GKRGPU_ERR_INVALID, "null argument");
        // the length field is 32 bits (transcript.hpp:56-59 writes bytes.size() as uint32)
        if (proof_len > 0xffffffffull) fail(GKRGPU_ERR_INVALID, "proof of %llu bytes does not fit the 4-byte length",
                                            (unsigned long long)proof_len);
        FILE* f = fopen(path, "wb");
        if (!f) fail(GKRGPU_ERR_IO, "cannot open %s for writing", path);
        const uint32_t n = (uint32_t)proof_len;
        const uint8_t len[4] = {(uint8_t)n, (uint8_t)(n >> 8), (uint8_t)(n >> 16), (uint8_t)(n >> 24)};
        const bool ok = fwrite(len, 1, 4, f) == 4 && (n == 0 || fwrite(proof, 1, n, f) == n);
        if (fclose(f) != 0 || !ok) fail(GKRGPU_ERR_IO, "write to %s failed", path);
    });
}

int gkrgpu_proof_read(const char* path, uint8_t* buf, uint64_t cap, uint64_t* proof_len) {
    return guarded([&] {
        if (!path || !proof_len) fail(GKRGPU_ERR_INVALID, "null argument");
        FILE* f = fopen(path, "rb");
        if (!f) fail(GKRGPU_ERR_IO, "cannot open %s", path);
        struct Closer {
            FILE* f;
            ~Closer() { fclose(f); }
        } closer{f};
        uint8_t len[4];
        if (fread(len, 1, 4, f) != 4) fail(GKRGPU_ERR_IO, "%s: no 4-byte length", path);
        const uint64_t n = (uint64_t)len[0] | ((uint64_t)len[1] << 8) | ((uint64_t)len[2] << 16) | ((uint64_t)len[3] << 24);
        *proof_len = n;
        if (!buf) return;  // size query
        if (cap < n) fail(GKRGPU_ERR_CAPACITY, "proof needs %llu bytes, buffer has %llu", (unsigned long long)n,
                          (unsigned long long)cap);
        if (n && fread(buf, 1, n, f) != n) fail(GKRGPU_ERR_IO, "%s: truncated (length field says %llu bytes)", path,
                                                (unsigned long long)n);
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
        if (b < 32 || b > 256 || b % 32) fail(GKRGPU_ERR_INVALID, "block must be a multiple of 32 in [32, 256]");
        if (threads_per_row > b) fail(GKRGPU_ERR_INVALID, "threads_per_row must be in [1, block]");
        ctx->block = b;
        for (auto& t : ctx->tiles) {
            if (threads_per_row) t.tpr = threads_per_row;
            if (ctas) t.ctas = ctas;
        }
    });
}

int gkrgpu_autotune(gkrgpu_ctx* ctx, const gkrgpu_circuit* circuit, uint32_t n_copies, int grinding_bits,
                    const uint32_t* input, int input_on_device, gkrgpu_tile_choice* out, int cap) {
    return guarded([&] {
        check_run(ctx, circuit, n_copies);
        if (!input) fail(GKRGPU_ERR_INVALID, "null input");
        ctx->drain();
        const bool bn = circuit->field == GKRGPU_FIELD_BN254;
        const int R = reps_for_field(circuit->field, grinding_bits);
        if (R < 1 || R > 3) fail(GKRGPU_ERR_INVALID, "unsupported grinding_bits");
        std::vector<uint8_t> proof(proof_bytes(circuit, n_copies, R));
        std::vector<uint32_t> cv((size_t)R * n_copies * elem_bytes(circuit->field) / 4);
        // effective threads per row slice of kind k for this circuit's field
        auto tile_tpr = [&](int k) { return k >= K_BN_LOAD ? geo_bn(*ctx, n_copies, k).tpr : ctx->geo(n_copies, k).tpr; };
        const bool saved_timing = ctx->timing;
        const auto saved_tiles = std::vector<gkrgpu_ctx::Tile>(std::begin(ctx->tiles), std::end(ctx->tiles));
        ctx->timing = true;
        auto snapshot = [&](double* ms) {
            std::lock_guard<std::mutex> lk(ctx->stats_m);
            for (int k = 0; k < K_NUM_KERNELS; k++) ms[k] = ctx->ms[k];
        };
        // One proof with the current tiles; returns the device ms of each kernel kind.
        auto run = [&](double* ms) {
            double a[K_NUM_KERNELS], b[K_NUM_KERNELS];
            snapshot(a);
            uint64_t len = 0;
            const int rc = prove_entry(ctx, circuit, n_copies, grinding_bits, input_on_device ? nullptr : input,
                                       input_on_device ? input : nullptr, proof.data(), proof.size(), &len, cv.data());
            if (rc != GKRGPU_OK) throw Error(rc, g_last_error);
            snapshot(b);
            for (int k = 0; k < K_NUM_KERNELS; k++) ms[k] = b[k] - a[k];
        };
        const std::vector<int> kinds =
            bn ? std::vector<int>{K_BN_EVALUATE, K_BN_HG_ROUND0, K_BN_ROUND_LANE, K_BN_ROUND_SCALAR, K_BN_WSUM}
               : std::vector<int>{K_EVALUATE, K_HG_ROUND0, K_HG_ROUND1, K_ROUND_LANE, K_ROUND_SCALAR, K_P2_ROUND0,
                                  K_WSUM};
        try {
            double ms[K_NUM_KERNELS];
            run(ms);  // warm-up: pool growth, first-launch costs
            // stage 1: threads per row (distinct effective tiles only), default CTA budgets
            double best_ms[K_NUM_KERNELS];
            uint32_t best_tpr[K_NUM_KERNELS], best_ctas[K_NUM_KERNELS];
            for (int k = 0; k < K_NUM_KERNELS; k++) {
                best_ms[k] = 1e300;
                best_tpr[k] = saved_tiles[k].tpr;
                best_ctas[k] = 0;
            }
            std::vector<uint32_t> seen;
            for (uint32_t t : {8u, 16u, 32u, 64u, 128u}) {
                for (auto& tl : ctx->tiles) tl = gkrgpu_ctx::Tile{t, 0};
                const uint32_t eff = tile_tpr(bn ? K_BN_ROUND_LANE : K_ROUND_LANE);
                if (std::find(seen.begin(), seen.end(), eff) != seen.end()) continue;
                seen.push_back(eff);
                run(ms);
                for (int k : kinds)
                    if (ms[k] > 0 && ms[k] < best_ms[k]) {
                        best_ms[k] = ms[k];
                        best_tpr[k] = t;
                    }
            }
            // stage 2: CTA budgets with each kind's best tile
            for (uint32_t m : {2u, 8u, 16u}) {
                for (int k = 0; k < K_NUM_KERNELS; k++) ctx->tiles[k] = gkrgpu_ctx::Tile{best_tpr[k], m * ctx->sm_count};
                run(ms);
                for (int k : kinds)
                    if (ms[k] > 0 && ms[k] < best_ms[k]) {
                        best_ms[k] = ms[k];
                        best_ctas[k] = m * ctx->sm_count;
                    }
            }
            for (int k = 0; k < K_NUM_KERNELS; k++) ctx->tiles[k] = gkrgpu_ctx::Tile{best_tpr[k], best_ctas[k]};
            if (out)
                for (int k = 0; k < K_NUM_KERNELS && k < cap; k++) {
                    out[k].threads_per_row = tile_tpr(k);
                    out[k].ctas = ctx->cta_budget(k);
                    out[k].ms = best_ms[k] < 1e300 ? best_ms[k] : 0.0;
                }
        } catch (...) {
            for (int k = 0; k < K_NUM_KERNELS; k++) ctx->tiles[k] = saved_tiles[k];
            ctx->timing = saved_timing;
            throw;
        }
        ctx->timing = saved_timing;
    });
}

}  // extern "C"
