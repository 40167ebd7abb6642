/* gkrgpu: GB300-native GKR prover for data-parallel layered circuits over M31 and BN254.
 *
 * C ABI of the drop-in boundary.  Each entry point replaces one piece of the reference
 * prove path of PolyhedraZK/Expander-cpp (file:line below are paths in that project).
 * Plain pointers and sizes only; every call returns a status code (GKRGPU_OK = 0) and
 * the message of the last failure on the calling thread is gkrgpu_last_error().
 * No C++ exception crosses this boundary.  Device waits inside the library are bounded.
 *
 * Value layout: a table of R rows for N data-parallel circuit copies is R*N uint32
 * values, row-major (row i, copy k at i*N + k), each canonical in [0, 2^31 - 1).  One row
 * is the byte image of the reference's vector field element (VectorizedM31::to_bytes,
 * include/field/M31.hpp:420-426) for N copies.
 *
 * BN254 circuits (gkrgpu_circuit_load_field with GKRGPU_FIELD_BN254): an element is 8
 * uint32 words, the canonical integer in [0, r) as 32 little-endian bytes, so a row is
 * 8*N words and every uint32_t* table argument below holds 8 words per value.  R = 1.
 */
#ifndef GKRGPU_H
#define GKRGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GKRGPU_OK 0
#define GKRGPU_ERR_INVALID 1   /* bad argument (shape, id out of range, non-canonical value) */
#define GKRGPU_ERR_CUDA 2      /* CUDA runtime failure */
#define GKRGPU_ERR_NOMEM 3     /* device or pinned host allocation failed */
#define GKRGPU_ERR_CAPACITY 4  /* caller buffer too small (required size still reported) */
#define GKRGPU_ERR_TIMEOUT 5   /* a bounded wait expired */
#define GKRGPU_ERR_STATE 6     /* object used in the wrong state */
#define GKRGPU_ERR_IO 7        /* file could not be opened, read or written */

/* Field_type, include/configuration/config.hpp:12-16 (same numbering).  BabyBear is
 * declared there without a prover and is rejected here too. */
#define GKRGPU_FIELD_M31 0
#define GKRGPU_FIELD_BABYBEAR 1
#define GKRGPU_FIELD_BN254 2

typedef struct gkrgpu_ctx gkrgpu_ctx;
typedef struct gkrgpu_circuit gkrgpu_circuit;

/* Gate<M31,2> and Gate<M31,1>, include/circuit/circuit.hpp:13-30 (16 and 12 bytes). */
typedef struct { uint32_t o_id, i0, i1, coef; } gkrgpu_mul_gate;
typedef struct { uint32_t o_id, i0, coef; } gkrgpu_add_gate;

/* CircuitLayer, include/circuit/circuit.hpp:68-116.  nb_output_vars of layer l must equal
 * nb_input_vars of layer l+1; layer 0 reads the circuit input. */
typedef struct {
    uint32_t nb_output_vars, nb_input_vars;
    uint64_t n_mul, n_add;
    const gkrgpu_mul_gate* mul;
    const gkrgpu_add_gate* add;
} gkrgpu_layer_desc;

/* Per-kernel launch accounting (see gkrgpu_kernel_stats). */
typedef struct {
    const char* name;
    uint64_t launches;
    double total_ms;          /* CUDA-event time, only while timing is enabled */
    double algorithmic_bytes; /* compulsory HBM bytes summed over the launches */
} gkrgpu_kernel_stat;

/* Message of the last failure on this thread ("" if none). */
const char* gkrgpu_last_error(void);

/* Library version string. */
const char* gkrgpu_version(void);

/* Config::get_num_repetitions for M31 with 100-bit security,
 * include/configuration/config.hpp:61-65 (3 for the default grinding_bits = 10). */
int gkrgpu_num_repetitions(int grinding_bits);

/* The same for any supported field: ceil((100 - grinding_bits) / field_size), field_size 31
 * (M31) or 254 (BN254), config.hpp:40-65.  Negative for an unsupported field. */
int gkrgpu_num_repetitions_field(int field, int grinding_bits);

/* Bytes of one element of `field` in every table and in the proof (4 or 32; 0 if unsupported). */
uint32_t gkrgpu_field_bytes(int field);

/* A context owns one CUDA device, a stream and a reusable device workspace.
 * Replaces the reference's per-prover scratch (GKRScratchPad,
 * include/LinearGKR/scratch_pad.hpp:8-65; Prover::prepare_mem, LinearGKR.hpp:49-56). */
int gkrgpu_create(int device, gkrgpu_ctx** out);
void gkrgpu_destroy(gkrgpu_ctx* ctx);

/* Uploads a circuit's wiring (the gate lists of every layer) to the device and builds
 * the per-layer gate indexes the kernels use.  Replaces building Circuit<F,F_primitive>
 * (include/circuit/circuit.hpp:118-251).  Ids and coefficients are checked. */
int gkrgpu_circuit_load(gkrgpu_ctx* ctx, const gkrgpu_layer_desc* layers, int n_layers, gkrgpu_circuit** out);
void gkrgpu_circuit_free(gkrgpu_circuit* circuit);

/* As gkrgpu_circuit_load for the field Config::field_type names (GKRGPU_FIELD_*).  Every
 * later call on the circuit works in that field: BN254 tables hold 8 words per value,
 * coefficients are any uint32 (canonical in BN254), R = 1 and n_copies may be any count
 * in [1, 65536].  gkrgpu_circuit_load is this call with GKRGPU_FIELD_M31. */
int gkrgpu_circuit_load_field(gkrgpu_ctx* ctx, const gkrgpu_layer_desc* layers, int n_layers, int field,
                              gkrgpu_circuit** out);

/* Field of a loaded circuit (GKRGPU_FIELD_*), negative for a null circuit. */
int gkrgpu_circuit_field(const gkrgpu_circuit* circuit);

/* Circuit files of the reference, parsed on the host into layers ready for
 * gkrgpu_circuit_load(_field).  The handle owns the gate arrays the layer descriptors point
 * to; free it with gkrgpu_parsed_free after loading.
 *
 * gkrgpu_circuit2_parse: the binary CIRCUIT2 segment format (CircuitRaw::operator>>,
 *   include/circuit/circuit_raw.hpp:511-568) flattened as Circuit::from_circuit_raw does
 *   (include/circuit/circuit.hpp:217-251): segment trees expanded with their allocation
 *   offsets, const gates dropped, layer sizes from the largest gate ids
 *   (_compute_nb_vars, circuit.hpp:124-150), and every coefficient 1, because the
 *   reference's M31 reader discards the 32 bytes it reads (include/field/M31.hpp:124-135).
 * gkrgpu_extracted_parse: the text gate lists of Circuit::load_extracted_gates
 *   (circuit.hpp:152-215), line i of each file being layer (lines - 1 - i).
 * A malformed file gives GKRGPU_ERR_INVALID (the reference exits the process). */
typedef struct gkrgpu_parsed gkrgpu_parsed;
int gkrgpu_circuit2_parse(const uint8_t* bytes, uint64_t len, gkrgpu_parsed** out);
int gkrgpu_extracted_parse(const char* mul_text, uint64_t mul_len, const char* add_text, uint64_t add_len,
                           gkrgpu_parsed** out);
int gkrgpu_parsed_layers(const gkrgpu_parsed* parsed);
int gkrgpu_parsed_layer(const gkrgpu_parsed* parsed, int layer, gkrgpu_layer_desc* out);
void gkrgpu_parsed_free(gkrgpu_parsed* parsed);

/* Proof bytes of Prover::prove for this circuit: RAW commitment (2^nb_input_vars(0) rows
 * of 4N bytes) + 32 grinding bytes + per layer R*(6*nb_input_vars + 2) rows of 4N bytes. */
uint64_t gkrgpu_proof_size(const gkrgpu_circuit* circuit, uint32_t n_copies, int grinding_bits);

/* Rows of the value tables gkrgpu_evaluate writes with all_layers = 1. */
uint64_t gkrgpu_value_rows(const gkrgpu_circuit* circuit, int all_layers);

/* Circuit::evaluate (include/circuit/circuit.hpp:92-105,273-280) on the device.
 * input: host table of 2^nb_input_vars(0) rows.  out: host table of the last layer's
 * output rows (all_layers = 0) or of every layer's input rows followed by the output
 * rows (all_layers = 1). */
int gkrgpu_evaluate(gkrgpu_ctx* ctx, const gkrgpu_circuit* circuit, uint32_t n_copies, const uint32_t* input,
                    uint32_t* out, int all_layers);

/* Prover::prove (include/LinearGKR/LinearGKR.hpp:58-90): RAW commitment, grinding,
 * gkr_prove (include/LinearGKR/gkr.hpp:24-73) and the empty RAW openings, after
 * Circuit::evaluate.  input: host table (2^nb_input_vars(0) rows, n_copies lanes, a
 * multiple of 4).  proof_out receives the transcript bytes (proof_len set even when the
 * capacity is short); claimed_v receives R rows of n_copies lanes (gkr.hpp:52-55).
 * The bytes are identical to the reference prover's for the same circuit and input. */
int gkrgpu_prove(gkrgpu_ctx* ctx, const gkrgpu_circuit* circuit, uint32_t n_copies, int grinding_bits,
                 const uint32_t* input, uint8_t* proof_out, uint64_t proof_cap, uint64_t* proof_len,
                 uint32_t* claimed_v);

/* As gkrgpu_prove with the input table already resident in device memory (d_input, on
 * this context's device).  The commitment bytes are read back from the device. */
int gkrgpu_prove_device(gkrgpu_ctx* ctx, const gkrgpu_circuit* circuit, uint32_t n_copies, int grinding_bits,
                        const uint32_t* d_input, uint8_t* proof_out, uint64_t proof_cap, uint64_t* proof_len,
                        uint32_t* claimed_v);

/* Transcript hash of the proofs submitted on this context from now on and of
 * gkrgpu_verify (FiatShamir_hash_type numbering, include/configuration/config.hpp:18-24):
 * GKRGPU_FS_SHA256 (default; the only hash the reference's transcript implements, so the
 * only one with byte parity against it) or GKRGPU_FS_KECCAK256 (the same transcript schedule
 * with Keccak-256 wherever SHA-256 is used; the reference has no Keccak code).  Waits for
 * queued proofs first. */
#define GKRGPU_FS_SHA256 0
#define GKRGPU_FS_KECCAK256 1
int gkrgpu_set_fs_hash(gkrgpu_ctx* ctx, int fs_hash_type);

/* The Keccak-256 transcript hash (original Keccak padding, domain byte 0x01, rate 136
 * bytes) and SHA3-256 (the same sponge with the FIPS 202 domain byte 0x06), host-side;
 * out receives 32 bytes. */
void gkrgpu_keccak256(const uint8_t* in, uint64_t len, uint8_t* out);
void gkrgpu_sha3_256(const uint8_t* in, uint64_t len, uint8_t* out);

/* Verifier::verify (include/LinearGKR/LinearGKR.hpp:105-149: gkr_verify, gkr.hpp:75-122, and
 * RawPC::verify, raw.hpp:75-78), GPU-assisted, for M31 and BN254 circuits: the host replays the
 * transcript and checks every round; the device computes each layer's
 * eval_sparse_circuit_connect_poly (eq tables and gate sums,
 * sumcheck_verifier_utils.hpp:22-56) and the multilinear evaluations of the committed input
 * (the proof's first 2^nb_input_vars(0) rows).  claimed_v: R rows of n_copies lanes.
 * *accepted is 1 when the reference verifier would accept, else 0 (the status is
 * GKRGPU_OK either way; errors are bad arguments or device failures). */
int gkrgpu_verify(gkrgpu_ctx* ctx, const gkrgpu_circuit* circuit, uint32_t n_copies, int grinding_bits,
                  const uint8_t* proof, uint64_t proof_len, const uint32_t* claimed_v, int* accepted);

/* Pipelined Prover::prove.  gkrgpu_prove_submit queues one proof and returns at once; its
 * host stage (RAW commitment bytes, their SHA-256, grinding) runs on a host worker while
 * earlier proofs' device stages run on the GPU, and device stages run one at a time in
 * submission order.  The input (host memory, or device memory with input_on_device = 1),
 * proof_out and claimed_v must stay valid until gkrgpu_prove_wait returns.  With
 * marker_slot in [0, 64) the device stage's end is recorded as timing marker
 * `marker_slot` and its beginning (when a lane takes the proof, once that lane's stream has
 * finished its previous proof) as marker 64 + marker_slot (gkrgpu_elapsed_ms).  gkrgpu_prove_wait blocks until the job is finished, frees it and
 * returns its status; proof_len receives the proof length.  gkrgpu_prove and
 * gkrgpu_prove_device are submit + wait.  No counterpart in the reference (one proof per
 * thread there, bench_keccak.cpp:82-93). */
typedef struct gkrgpu_job gkrgpu_job;

/* Continuous batching.  A context runs the device stages of up to `lanes` proofs at once,
 * each on its own stream (default 1); a queued proof starts when a lane is free and its
 * device workspace (gkrgpu_workspace_bytes) fits in `hbm_budget_bytes` next to the proofs
 * already running (a proof larger than the budget runs alone).  Workspaces come from a
 * stream-ordered pool and are returned when the proof ends.  Waits for queued proofs
 * first; 0 keeps the current value (default budget: 90% of the free memory at creation).
 * Host stages (the commitment's SHA-256 and grinding) run on max(4, min(lanes, 8)) host
 * threads, so the sequential hashes of several queued proofs overlap.
 * No counterpart in the reference, which proves one circuit per thread. */
int gkrgpu_set_concurrency(gkrgpu_ctx* ctx, int lanes, uint64_t hbm_budget_bytes);
/* Host threads that run host stages (the SHA-256 of the RAW commitment, grinding): the
 * hashes of queued proofs' commitments are sequential each, so this many run at once.  0
 * restores the default, max(4, min(lanes, 8)).  Waits for queued proofs first. */
int gkrgpu_set_host_threads(gkrgpu_ctx* ctx, int threads);
/* Device bytes one proof of this circuit holds while it runs. */
uint64_t gkrgpu_workspace_bytes(const gkrgpu_circuit* circuit, uint32_t n_copies, int grinding_bits,
                                int input_on_device);
/* Workspace bytes held now, the peak since creation, and the budget. */
int gkrgpu_memory_stats(gkrgpu_ctx* ctx, uint64_t* in_use, uint64_t* peak, uint64_t* budget);

int gkrgpu_prove_submit(gkrgpu_ctx* ctx, const gkrgpu_circuit* circuit, uint32_t n_copies, int grinding_bits,
                        const uint32_t* input, int input_on_device, uint8_t* proof_out, uint64_t proof_cap,
                        uint32_t* claimed_v, int marker_slot, gkrgpu_job** job);
int gkrgpu_prove_wait(gkrgpu_job* job, uint64_t* proof_len);

/* gkrgpu_prove_submit for an input held both in host memory and, resident, in device
 * memory (16-byte aligned; the same values): the host stage copies and hashes the RAW
 * commitment from h_input and the device stage computes from d_input, so nothing is copied
 * between host and device for the input.  For request loops that upload each witness once,
 * when it is admitted, and keep it on the device.  No counterpart in the reference. */
int gkrgpu_prove_submit_resident(gkrgpu_ctx* ctx, const gkrgpu_circuit* circuit, uint32_t n_copies,
                                 int grinding_bits, const uint32_t* h_input, const uint32_t* d_input,
                                 uint8_t* proof_out, uint64_t proof_cap, uint32_t* claimed_v, int marker_slot,
                                 gkrgpu_job** job);

/* eval_multilinear (include/poly_commit/poly.hpp:88-104) of a device table d_evals of
 * 2^nb_vars rows at n_points (1..3) points: r is a host array of n_points x nb_vars
 * canonical values, out (host) receives n_points rows of n_copies lanes, row j being
 * sum_z eq(r_j, z) * evals[z].  This is RawPC::verify's check value
 * (include/poly_commit/raw.hpp:75-78) and gkr_prove's output claim
 * (include/LinearGKR/gkr.hpp:52-55).  The eq tables and the reduction scratch live in
 * the context's workspace. */
int gkrgpu_eval_multilinear(gkrgpu_ctx* ctx, const uint32_t* d_evals, uint32_t nb_vars, uint32_t n_copies,
                            const uint32_t* r, int n_points, uint32_t* out);

/* gkrgpu_eval_multilinear without any allocation, for callers that cannot allocate device
 * memory: e.g. a verifier living in a process whose device memory is already reserved by
 * another framework's caching allocator, or code where cudaMalloc/cudaFree (which can
 * synchronize the whole device) are not allowed.  No counterpart in the reference.
 * Same result as gkrgpu_eval_multilinear, but the output d_out is a caller-owned device
 * buffer of n_points x n_copies u32 and no context is needed: the work runs on `stream`
 * (a cudaStream_t; NULL = the legacy default stream) of the current device and the call
 * returns when it has finished.  Its scratch is a fixed 3.1 MiB region inside the library
 * (held by every GPU that loads the library until the process exits), so the limits are
 * nb_vars <= 18, n_copies <= 4096 (a multiple of 4) and n_points <= 3; larger sizes are
 * rejected with GKRGPU_ERR_INVALID.  The first call on a device looks up the scratch
 * address; make that first call before any stream capture begins.  Every call waits for
 * its own work on `stream` before it returns.  All calls share the one scratch region:
 * calls that overlap on the GPU (from several host threads or streams) race and must be
 * serialized by the caller. */
int gkrgpu_eval_multilinear_noalloc(const uint32_t* d_evals, uint32_t nb_vars, uint32_t n_copies,
                                    const uint32_t* r, int n_points, uint32_t* d_out, void* stream);

/* Persistent phase tails.  When the tables of a phase's last rounds are small, those rounds
 * run in one launch (k_tail) that waits on the device for each round's challenges, which
 * the host writes into host-mapped memory after hashing the round's evaluations, instead of
 * one kernel launch per round.  On by default; gkrgpu_set_round_tail(ctx, 0) runs every
 * round as its own launch (the proof bytes are the same).  A context created under a CUDA
 * injection tool (CUDA_INJECTION64_PATH set, as profilers do) starts with the tails off:
 * such tools may run each kernel to completion before the launching thread goes on, and a
 * tail waits for that thread.  No counterpart in the reference, whose sumcheck runs on the
 * CPU (sumcheck.hpp:72-97). */
int gkrgpu_set_round_tail(gkrgpu_ctx* ctx, int enabled);
/* Checks the bounded device wait of the phase tails: runs a two-round tail whose second
 * challenge is never written, with a wait limit of timeout_us, and reports whether the wait
 * expired and the kernel returned (expired = 1) and how many rounds it published (1).  The
 * context stays usable.  A diagnostic with no counterpart in the reference. */
int gkrgpu_check_device_wait(gkrgpu_ctx* ctx, uint32_t timeout_us, int* expired, int* rounds_published);

/* Device / pinned host buffers for callers without a CUDA allocator of their own. */
int gkrgpu_device_alloc(gkrgpu_ctx* ctx, uint64_t bytes, void** out);
int gkrgpu_device_free(gkrgpu_ctx* ctx, void* p);
int gkrgpu_host_alloc(uint64_t bytes, void** out);
int gkrgpu_host_free(void* p);
int gkrgpu_memcpy_h2d(gkrgpu_ctx* ctx, void* dst, const void* src, uint64_t bytes);
int gkrgpu_memcpy_d2h(gkrgpu_ctx* ctx, void* dst, const void* src, uint64_t bytes);
/* Host -> device copy on the context's own transfer stream: unlike gkrgpu_memcpy_h2d it
 * does not wait for queued proofs, which keep running while it copies; it returns when the
 * copy is done.  For request loops that upload witnesses as requests are admitted. */
int gkrgpu_upload(gkrgpu_ctx* ctx, void* d_dst, const void* h_src, uint64_t bytes);

/* Launch accounting.  With timing on, every kernel launch is bracketed by CUDA events on
 * the context's stream.  Counts and times are added to the totals when each proof (or
 * other call) finishes, so gkrgpu_kernel_stats, which may be called while proofs are in
 * flight, always reads whole proofs; it fills up to cap entries (one per kernel kind) and
 * returns how many kinds exist.  gkrgpu_set_timing and gkrgpu_reset_stats first wait for
 * queued proofs to finish.  When the environment variable GKRGPU_TRACE names a file at
 * gkrgpu_create, every timed launch also appends a CSV line to it: kernel kind, lane,
 * layer, phase (0 evaluate, 1, 2), round, algorithmic bytes, milliseconds, and the launch's
 * device start and host launch-call time in milliseconds after the context's creation
 * (plus a host_stage_wait line per proof: how long its device stage waited for the host
 * stage). */
int gkrgpu_set_timing(gkrgpu_ctx* ctx, int enabled);
int gkrgpu_reset_stats(gkrgpu_ctx* ctx);
int gkrgpu_kernel_stats(gkrgpu_ctx* ctx, gkrgpu_kernel_stat* out, int cap);

/* Tuning of the row tile: threads per row slice (each covers 4 copies), CTA size and the
 * CTA budget of the reducing kernels.  0 keeps the current value. */
int gkrgpu_set_tile(gkrgpu_ctx* ctx, uint32_t threads_per_row, uint32_t block, uint32_t ctas);

/* Autotuner.  Times whole proofs of `circuit` on `input` (host memory, or device memory with
 * input_on_device = 1) with candidate row tiles - threads per row slice 8..128 (copies per
 * CTA row tile = 4x that), then CTA budgets 2..16 x the SM count - and keeps, for each kernel
 * kind, the tile with the least device time; tiles never change the proof bytes.  out
 * (optional, up to cap entries, one per kernel kind in gkrgpu_kernel_stats order) receives
 * the chosen tiles and their device ms per proof.  About 9 proofs of work. */
typedef struct {
    uint32_t threads_per_row, ctas;
    double ms;
} gkrgpu_tile_choice;
int gkrgpu_autotune(gkrgpu_ctx* ctx, const gkrgpu_circuit* circuit, uint32_t n_copies, int grinding_bits,
                    const uint32_t* input, int input_on_device, gkrgpu_tile_choice* out, int cap);

/* Timing markers: gkrgpu_mark records CUDA event `slot` (0..127) on the context's stream
 * once every queued proof has finished; gkrgpu_elapsed_ms waits for `to_slot` and returns
 * the device time between the two.  Slots 0..63 and 64..127 are also written by proofs
 * submitted with a marker slot (their device-stage end and beginning). */
int gkrgpu_mark(gkrgpu_ctx* ctx, int slot);
int gkrgpu_elapsed_ms(gkrgpu_ctx* ctx, int from_slot, int to_slot, double* ms);

/* Bytes the library copied host->device and device->host since the last reset. */
int gkrgpu_transfer_stats(gkrgpu_ctx* ctx, uint64_t* h2d_bytes, uint64_t* d2h_bytes);

/* Proof files in the reference's format, Proof::write_and_compress / read_proof
 * (include/fiat_shamir/transcript.hpp:54-84): a 4-byte little-endian length, then the proof
 * bytes.  The reference also tars the file (a shell call); that step is left to the caller.
 * gkrgpu_proof_write rejects proofs of 2^32 bytes or more (the reference would truncate the
 * length).  gkrgpu_proof_read with buf = NULL returns the length only; a buffer smaller than
 * the length gives GKRGPU_ERR_CAPACITY with proof_len set; a short file GKRGPU_ERR_IO. */
int gkrgpu_proof_write(const char* path, const uint8_t* proof, uint64_t proof_len);
int gkrgpu_proof_read(const char* path, uint8_t* buf, uint64_t cap, uint64_t* proof_len);

#ifdef __cplusplus
}
#endif
#endif
