// gkrgpu_eval_multilinear_noalloc: eval_multilinear of a device table for callers that
// cannot allocate device memory.
//
// Typical such callers are a verifier embedded in a host process whose device memory is
// already carved up by another framework's caching allocator (a cudaMalloc from outside
// that allocator can fail or fragment it), and latency-critical code where cudaMalloc and
// cudaFree are not allowed because they can synchronize the whole device.  This entry point
// therefore uses one fixed scratch region that is part of the library image: a file-scope
// __device__ array, which every GPU that loads the library holds until the process exits.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "../../include/gkrgpu.h"
#include "kernels.cuh"
#include "m31.cuh"

namespace gkrgpu {
void set_last_error(const char* msg);
}

namespace {

constexpr uint32_t kMaxVars = 18;       // tables of up to 2^18 rows
constexpr uint32_t kMaxCopies = 4096;   // up to 4096 copies per row
constexpr int kMaxPoints = 3;           // up to 3 evaluation points per call
constexpr size_t kEqBytes = (size_t)kMaxPoints * (1u << kMaxVars) * 4;  // 3 MiB of eq tables
constexpr size_t kAccBytes = (size_t)kMaxPoints * kMaxCopies * 8;       // 96 KiB of 64-bit sums
// One arrival ticket per lane group of the reduction: a group covers 4 * tpr copies, so
// 4096 copies at one thread per row slice (tpr = 1, when n_copies / 4 has no larger
// divisor up to 32) give the most groups, 1024.
constexpr uint32_t kMaxLaneGroups = kMaxCopies / 4;
constexpr size_t kTicketBytes = (size_t)kMaxLaneGroups * 4;
constexpr size_t kScratchBytes = kEqBytes + kAccBytes + kTicketBytes;

// The scratch.  Host code must not use this name as an address (it is a host-side stand-in
// for the symbol); the device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char* g_scratch_ptr[kMaxDevices] = {};
int g_sm_count[kMaxDevices] = {};

// Once per device, with that device current: the device address of the scratch and the
// SM count that sizes the grids.
int setup_device(int dev) {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (g_scratch_ptr[dev]) return GKRGPU_OK;
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
        gkrgpu::set_last_error(cudaGetErrorString(e));
        return GKRGPU_ERR_CUDA;
    }
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) {
        gkrgpu::set_last_error(cudaGetErrorString(e));
        return GKRGPU_ERR_CUDA;
    }
    g_sm_count[dev] = sms;
    g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
    return GKRGPU_OK;
}

int fail(int code, const char* msg) {
    gkrgpu::set_last_error(msg);
    return code;
}

}  // namespace

extern "C" int gkrgpu_eval_multilinear_noalloc(const uint32_t* d_evals, uint32_t nb_vars, uint32_t n_copies,
                                               const uint32_t* r, int n_points, uint32_t* d_out, void* stream) {
    if (!d_evals || !r || !d_out) return fail(GKRGPU_ERR_INVALID, "null buffer");
    if (((uintptr_t)d_evals & 15) || ((uintptr_t)d_out & 3)) return fail(GKRGPU_ERR_INVALID, "misaligned buffer");
    if (n_points < 1 || n_points > kMaxPoints) return fail(GKRGPU_ERR_INVALID, "n_points must be in [1, 3]");
    if (nb_vars > kMaxVars) return fail(GKRGPU_ERR_INVALID, "nb_vars exceeds the no-alloc limit of 18 (2^18 rows)");
    if (n_copies < 4 || n_copies % 4 || n_copies > kMaxCopies)
        return fail(GKRGPU_ERR_INVALID, "n_copies must be a multiple of 4 in [4, 4096] for the no-alloc variant");
    for (int j = 0; j < n_points; j++)
        for (uint32_t t = 0; t < nb_vars; t++)
            if (r[(size_t)j * nb_vars + t] >= m31::P) return fail(GKRGPU_ERR_INVALID, "point coordinate >= p");

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(GKRGPU_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(GKRGPU_ERR_INVALID, "device index out of range");
    const int rc = setup_device(dev);
    if (rc != GKRGPU_OK) return rc;

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned char* base = g_scratch_ptr[dev];
    uint32_t* eq = reinterpret_cast<uint32_t*>(base);
    gkrgpu::RedScratch red{reinterpret_cast<unsigned long long*>(base + kEqBytes),
                           reinterpret_cast<unsigned int*>(base + kEqBytes + kAccBytes)};

    // The scratch keeps the previous call's contents: zero the sums and the ticket.
    e = cudaMemsetAsync(base + kEqBytes, 0, kAccBytes + kTicketBytes, s);
    if (e != cudaSuccess) return fail(GKRGPU_ERR_CUDA, cudaGetErrorString(e));

    gkrgpu::EqArgs a;
    memset(&a, 0, sizeof(a));
    for (int j = 0; j < n_points; j++) memcpy(a.r1[j], r + (size_t)j * nb_vars, 4 * nb_vars);
    a.f1 = 1u;
    a.nvars = nb_vars;
    a.reps = (uint32_t)n_points;
    e = gkrgpu::launch_eq(eq, a, s);
    if (e != cudaSuccess) return fail(GKRGPU_ERR_CUDA, cudaGetErrorString(e));

    gkrgpu::Geo g;
    g.N = n_copies;
    const uint32_t Q = n_copies / 4;
    g.tpr = Q <= 32 ? Q : 32;
    while (Q % g.tpr) g.tpr--;
    g.rps = 256 / g.tpr;
    if (Q % g.tpr || Q / g.tpr > kMaxLaneGroups)
        return fail(GKRGPU_ERR_INVALID, "no row tile with at most 1024 lane groups for this copy count");
    e = gkrgpu::launch_wsum(n_points, d_evals, 1ull << nb_vars, eq, g, 256, (uint32_t)g_sm_count[dev] * 4, red, d_out, s);
    if (e != cudaSuccess) return fail(GKRGPU_ERR_CUDA, cudaGetErrorString(e));
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(GKRGPU_ERR_CUDA, cudaGetErrorString(e));
    return GKRGPU_OK;
}
