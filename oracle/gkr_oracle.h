/* Test infrastructure only: the CPU oracle for the GKR prove path.
 *
 * A plain-C restatement of the reference prover and verifier of PolyhedraZK/Expander-cpp
 * (M31 field, SHA-256 Fiat-Shamir transcript, RAW commitment) for any number N of
 * data-parallel circuit copies.  It is pinned against the compiled reference
 * (oracle/ref_driver.cpp, built into oracle/_ref/ where the reference tree is present)
 * and against the golden fixtures in tests/golden/.  Only tests, the smoke check and
 * bench.py's CPU-baseline arm may load it; the product never links it.
 *
 * Field elements of one layer are stored row-major: value (row i, copy k) sits at
 * index i * N + k, i.e. each row is the N-lane vector the reference serialises with
 * VectorizedM31::to_bytes (include/field/M31.hpp:420-426).
 */
#ifndef GKR_ORACLE_H
#define GKR_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One circuit layer.  mul = n_mul gates of {o_id, i0, i1, coef}; add = n_add gates of
 * {o_id, i0, coef} (include/circuit/circuit.hpp:13-30, Gate<F,2> and Gate<F,1>). */
typedef struct {
    uint32_t nb_output_vars, nb_input_vars;
    uint64_t n_mul, n_add;
    const uint32_t* mul;
    const uint32_t* add;
} oracle_layer;

/* Number of parallel repetitions, include/configuration/config.hpp:61-65 (M31, 100-bit). */
int oracle_num_repetitions(int grinding_bits);

/* Proof length in bytes for this circuit, copy count and repetition count. */
uint64_t oracle_proof_size(const oracle_layer* layers, int nlayers, uint32_t n_copies, int reps);

/* Circuit::evaluate.  out receives every layer's input rows followed by the last layer's
 * output rows (sum of 2^nb_input_vars over layers plus 2^nb_output_vars(last), times N). */
int oracle_evaluate(const oracle_layer* layers, int nlayers, uint32_t n_copies, const uint32_t* input, uint32_t* out);

/* Prover::prove after Circuit::evaluate.  claimed_v receives reps x N lanes.
 * Returns 0 on success, 2 if proof_cap is too small, negative on bad input. */
int oracle_prove(const oracle_layer* layers, int nlayers, uint32_t n_copies, const uint32_t* input,
                 int grinding_bits, uint8_t* proof_out, uint64_t proof_cap, uint64_t* proof_len, uint32_t* claimed_v);

/* Verifier::verify.  Returns 1 accept, 0 reject, negative on bad input. */
int oracle_verify(const oracle_layer* layers, int nlayers, uint32_t n_copies, const uint32_t* input,
                  int grinding_bits, const uint8_t* proof, uint64_t proof_len, const uint32_t* claimed_v);

/* eval_multilinear (include/poly_commit/poly.hpp:88-104) of rows x N values at point r. */
void oracle_eval_multilinear(const uint32_t* evals, uint32_t nb_vars, uint32_t n_copies, const uint32_t* r, uint32_t* out);

/* SHA256Hasher::hash (include/hash/hashes.hpp:22-33). */
void oracle_sha256(const uint8_t* in, uint64_t len, uint8_t out[32]);

/* Transcript hash selection (fs_hash.c): 0 = SHA-256 (default), 1 = Keccak-256; process-wide,
 * for single-threaded test use.  oracle_fs_hash hashes with the selected function. */
void oracle_set_fs_hash(int h);
int oracle_get_fs_hash(void);
void oracle_fs_hash(const uint8_t* in, uint64_t len, uint8_t out[32]);
void oracle_keccak256(const uint8_t* in, uint64_t len, uint8_t out[32]);
void oracle_sha3_256(const uint8_t* in, uint64_t len, uint8_t out[32]);

/* Throughput harness in the manner of benchmarks/bench_keccak.cpp:32-42,82-93: n_threads
 * threads each run proofs_per_thread proofs (evaluate + prove) of the same circuit.
 * Returns wall seconds, or a negative value on failure. */
double oracle_bench(const oracle_layer* layers, int nlayers, uint32_t n_copies, const uint32_t* input,
                    int grinding_bits, int n_threads, int proofs_per_thread);

/* BN254 (gkr_oracle_bn254.c): the same calls with one repetition.  Tables hold 4 uint64
 * limbs per element (its 32 canonical little-endian bytes); coefficients are any uint32;
 * claimed_v is N elements.  prove/evaluate return -1 on an input element >= r. */
int oracle_bn254_num_repetitions(int grinding_bits);
uint64_t oracle_bn254_proof_size(const oracle_layer* layers, int nlayers, uint32_t n_copies);
int oracle_bn254_evaluate(const oracle_layer* layers, int nlayers, uint32_t n_copies, const uint64_t* input,
                          uint64_t* out);
int oracle_bn254_prove(const oracle_layer* layers, int nlayers, uint32_t n_copies, const uint64_t* input,
                       int grinding_bits, uint8_t* proof_out, uint64_t proof_cap, uint64_t* proof_len,
                       uint64_t* claimed_v);
int oracle_bn254_verify(const oracle_layer* layers, int nlayers, uint32_t n_copies, const uint64_t* input,
                        int grinding_bits, const uint8_t* proof, uint64_t proof_len, const uint64_t* claimed_v);
double oracle_bn254_bench(const oracle_layer* layers, int nlayers, uint32_t n_copies, const uint64_t* input,
                          int grinding_bits, int n_threads, int proofs_per_thread);

#ifdef __cplusplus
}
#endif
#endif
