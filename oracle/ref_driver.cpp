// Test infrastructure only: a thin extern "C" driver around the UNMODIFIED reference
// prover and verifier (PolyhedraZK/Expander-cpp, header-only templates).  It is compiled
// from the reference's own headers by oracle/build_ref.sh into oracle/_ref/ and is used
// by the CPU tests to pin the C restatement (oracle/gkr_oracle.c) and to generate the
// golden fixtures under tests/golden/.  Nothing in the product links or calls it.
//
// The reference packs 8 circuit copies per field element on x86 (VectorizedM31,
// include/field/M31.hpp:240-449).  To run its templates with other copy counts this
// driver supplies LaneVec<E, N>, an N-lane element whose arithmetic calls the scalar type
// E's operators: the reference's own M31 (include/field/M31.hpp:64-93), or Bn254 below.
// At N=8 the proofs of LaneVec<M31, 8> and of VectorizedM31 are compared byte for byte by
// the tests.
//
// BN254: the reference declares the field (include/configuration/config.hpp:12-16,53-55)
// but its implementation header is missing, so Bn254 here is this project's definition
// (oracle/bn254.h: canonical 32-byte little-endian encoding, from_bytes reduces mod r).
// Instantiating the reference templates with it pins the protocol (transcript schedule,
// grinding with one 32-byte challenge, R = 1) for the BN254 prover.  The reference's
// Prover constructor asserts M31 (include/LinearGKR/LinearGKR.hpp:44), so this driver is
// compiled with NDEBUG.
//
// Everything the reference headers define must live in exactly one translation unit
// (include/field/M31.hpp:451-452 and include/utils/myutil.hpp define non-inline symbols).

#include "field/M31.hpp"
#include "LinearGKR/LinearGKR.hpp"

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fcntl.h>
#include <sstream>
#include <string>
#include <unistd.h>

#include "bn254.h"

namespace refdrv {

using gkr::M31_field::M31;
static const uint32_t P = 2147483647u;

// BN254 scalar with the interface the reference templates use for F_primitive.
struct Bn254 {
    bn_t a;
    static Bn254 INV_2;
    Bn254() { memset(a.v, 0, 32); }
    Bn254(uint32_t x) { a = bn_from_u32(x); }
    static Bn254 mk(bn_t v) { Bn254 r; r.a = v; return r; }
    static Bn254 zero() { return Bn254(); }
    static Bn254 one() { return Bn254(1u); }
    Bn254 operator+(const Bn254& o) const { return mk(bn_add(a, o.a)); }
    Bn254 operator-(const Bn254& o) const { return mk(bn_sub(a, o.a)); }
    Bn254 operator-() const { return mk(bn_neg(a)); }
    Bn254 operator*(const Bn254& o) const { return mk(bn_mul(a, o.a)); }
    void operator+=(const Bn254& o) { a = bn_add(a, o.a); }
    void operator-=(const Bn254& o) { a = bn_sub(a, o.a); }
    void operator*=(const Bn254& o) { a = bn_mul(a, o.a); }
    bool operator==(const Bn254& o) const { return bn_eq(a, o.a); }
    void to_bytes(uint8_t* out) const { bn_to_bytes(a, out); }
    void from_bytes(const uint8_t* in) { a = bn_from_bytes(in); }
    static int byte_length() { return 32; }
};
Bn254 Bn254::INV_2 = Bn254::mk(bn_t{{0xa1f0fac9f8000001ull, 0x9419f4243cdcb848ull, 0xdc2822db40c0ac2eull,
                                      0x183227397098d014ull}});

template <class E> struct Elem;
template <> struct Elem<M31> {
    static constexpr int bytes = 4;
    static M31 make(uint32_t x) { M31 m(x); if (m.x >= P) m.x -= P; return m; }
    static M31 inv2() { return M31::new_unchecked(1u << 30); }
};
template <> struct Elem<Bn254> {
    static constexpr int bytes = 32;
    static Bn254 make(uint32_t x) { return Bn254(x); }
    static Bn254 inv2() { return Bn254::INV_2; }
};

template <class E, int N>
struct Lanes {
    E v[N];
    Lanes operator+(const Lanes& o) const { Lanes r; for (int i = 0; i < N; i++) r.v[i] = v[i] + o.v[i]; return r; }
    Lanes operator-(const Lanes& o) const { Lanes r; for (int i = 0; i < N; i++) r.v[i] = v[i] - o.v[i]; return r; }
    Lanes operator*(const Lanes& o) const { Lanes r; for (int i = 0; i < N; i++) r.v[i] = v[i] * o.v[i]; return r; }
    Lanes operator*(const E& s) const { Lanes r; for (int i = 0; i < N; i++) r.v[i] = v[i] * s; return r; }
    void operator+=(const Lanes& o) { *this = *this + o; }
    bool operator==(const Lanes& o) const { for (int i = 0; i < N; i++) if (!(v[i] == o.v[i])) return false; return true; }
};

// N-lane stand-in for VectorizedM31: one Lanes "packed" element, because the reference
// indexes .elements[j] for j < vectorize_size (== 1 on x86),
// include/LinearGKR/sumcheck_helper.hpp:82-97,113-126.
template <class E, int N>
struct LaneVec {
    typedef E primitive_type;
    Lanes<E, N> elements[1];
    static LaneVec INV_2;

    LaneVec() { for (int i = 0; i < N; i++) elements[0].v[i] = E(); }
    LaneVec(uint32_t x) { const E e = Elem<E>::make(x); for (int i = 0; i < N; i++) elements[0].v[i] = e; }
    static LaneVec bcast(const E& e) { LaneVec r; for (int i = 0; i < N; i++) r.elements[0].v[i] = e; return r; }
    static LaneVec zero() { return LaneVec(); }
    static LaneVec one() { return LaneVec(1u); }
    static size_t pack_size() { return N; }

    LaneVec operator+(const LaneVec& o) const { LaneVec r; r.elements[0] = elements[0] + o.elements[0]; return r; }
    LaneVec operator-(const LaneVec& o) const { LaneVec r; r.elements[0] = elements[0] - o.elements[0]; return r; }
    LaneVec operator-() const { return LaneVec() - *this; }
    LaneVec operator*(const LaneVec& o) const { LaneVec r; r.elements[0] = elements[0] * o.elements[0]; return r; }
    LaneVec operator*(const E& s) const { LaneVec r; r.elements[0] = elements[0] * s; return r; }
    LaneVec operator*(const int& s) const { return *this * LaneVec((uint32_t)s); }
    LaneVec operator+(const E& s) const { return *this + bcast(s); }
    void operator+=(const LaneVec& o) { *this = *this + o; }
    void operator-=(const LaneVec& o) { *this = *this - o; }
    void operator*=(const LaneVec& o) { *this = *this * o; }
    bool operator==(const LaneVec& o) const { return elements[0] == o.elements[0]; }

    // Same byte layout as VectorizedM31::to_bytes/from_bytes (M31.hpp:420-434,
    // M31_avx.tcc:62-67): N elements in lane order, each reduced on read.
    void to_bytes(uint8_t* out) const { for (int i = 0; i < N; i++) elements[0].v[i].to_bytes(out + i * Elem<E>::bytes); }
    void from_bytes(const uint8_t* in) { for (int i = 0; i < N; i++) elements[0].v[i].from_bytes(in + i * Elem<E>::bytes); }
};
template <class E, int N> LaneVec<E, N> LaneVec<E, N>::INV_2 = LaneVec<E, N>::bcast(Elem<E>::inv2());

}  // namespace refdrv

extern "C" {

// One layer, gates as flat u32 arrays: mul = {o, i0, i1, coef} x n_mul, add = {o, i0, coef} x n_add.
struct ref_layer {
    uint32_t nb_output_vars, nb_input_vars;
    uint64_t n_mul, n_add;
    const uint32_t* mul;
    const uint32_t* add;
};

}

namespace refdrv {

template <class F, class Fp>
static gkr::Circuit<F, Fp> build_circuit(const ref_layer* layers, int nlayers, const uint8_t* input, size_t row_bytes) {
    gkr::Circuit<F, Fp> c;
    c.layers.resize(nlayers);
    for (int l = 0; l < nlayers; l++) {
        auto& L = c.layers[l];
        L.nb_output_vars = layers[l].nb_output_vars;
        L.nb_input_vars = layers[l].nb_input_vars;
        L.input_layer_vals.nb_vars = L.nb_input_vars;
        L.mul.nb_output_vars = L.add.nb_output_vars = L.nb_output_vars;
        L.mul.nb_input_vars = L.add.nb_input_vars = L.nb_input_vars;
        L.mul.sparse_evals.resize(layers[l].n_mul);
        for (uint64_t g = 0; g < layers[l].n_mul; g++) {
            const uint32_t* s = layers[l].mul + 4 * g;
            auto& G = L.mul.sparse_evals[g];
            G.o_id = s[0]; G.i_ids[0] = s[1]; G.i_ids[1] = s[2]; G.coef = Fp(s[3]);
        }
        L.add.sparse_evals.resize(layers[l].n_add);
        for (uint64_t g = 0; g < layers[l].n_add; g++) {
            const uint32_t* s = layers[l].add + 3 * g;
            auto& G = L.add.sparse_evals[g];
            G.o_id = s[0]; G.i_ids[0] = s[1]; G.coef = Fp(s[2]);
        }
    }
    uint64_t I0 = 1ull << layers[0].nb_input_vars;
    auto& ev = c.layers[0].input_layer_vals.evals;
    ev.resize(I0);
    for (uint64_t i = 0; i < I0; i++) ev[i].from_bytes(input + i * row_bytes);
    c.evaluate();
    return c;
}

static ::Config make_config(int grinding_bits, bool bn254 = false) {
    ::Config cfg;
    cfg.grinding_bits = grinding_bits;
    if (bn254) cfg.field_type = Field_type::BN254;
    cfg.initialize_config();
    return cfg;
}

// Silences the verifier's progress prints (include/LinearGKR/LinearGKR.hpp:143-144).
struct Mute {
    int saved;
    Mute() { fflush(stdout); std::cout.flush(); saved = dup(1); int dn = open("/dev/null", O_WRONLY); dup2(dn, 1); close(dn); }
    ~Mute() { fflush(stdout); std::cout.flush(); dup2(saved, 1); close(saved); }
};

template <class F, class Fp>
static int prove_t(const ref_layer* layers, int nlayers, const uint8_t* input, size_t row_bytes, int grinding_bits,
                   bool bn254, uint8_t* proof_out, uint64_t proof_cap, uint64_t* proof_len, uint8_t* claimed_v) {
    auto circuit = build_circuit<F, Fp>(layers, nlayers, input, row_bytes);
    ::Config cfg = make_config(grinding_bits, bn254);
    gkr::Prover<F, Fp> prover(cfg);
    prover.prepare_mem(circuit);
    auto t = prover.prove(circuit);
    auto& cv = std::get<0>(t);
    auto& proof = std::get<1>(t);
    *proof_len = proof.bytes.size();
    if (proof.bytes.size() > proof_cap) return 2;
    memcpy(proof_out, proof.bytes.data(), proof.bytes.size());
    for (size_t j = 0; j < cv.size(); j++) cv[j].to_bytes(claimed_v + j * row_bytes);
    return 0;
}

template <class F, class Fp>
static int verify_t(const ref_layer* layers, int nlayers, const uint8_t* input, size_t row_bytes, int grinding_bits,
                    bool bn254, const uint8_t* proof_bytes, uint64_t proof_len, const uint8_t* claimed_v) {
    auto circuit = build_circuit<F, Fp>(layers, nlayers, input, row_bytes);
    ::Config cfg = make_config(grinding_bits, bn254);
    gkr::Proof<F> proof;
    proof.bytes.assign(proof_bytes, proof_bytes + proof_len);
    std::vector<F> cv(cfg.get_num_repetitions());
    for (int j = 0; j < cfg.get_num_repetitions(); j++) cv[j].from_bytes(claimed_v + (size_t)j * row_bytes);
    gkr::Verifier verifier(cfg);
    bool ok;
    {
        Mute m;
        ok = verifier.verify(circuit, cv, proof);
    }
    return ok ? 1 : 0;
}

template <class F, class Fp>
static int evaluate_t(const ref_layer* layers, int nlayers, const uint8_t* input, size_t row_bytes, uint8_t* out) {
    auto circuit = build_circuit<F, Fp>(layers, nlayers, input, row_bytes);
    uint64_t off = 0;
    for (int l = 0; l < nlayers; l++) {
        for (auto& e : circuit.layers[l].input_layer_vals.evals) { e.to_bytes(out + off); off += row_bytes; }
    }
    for (auto& e : circuit.layers.back().output_layer_vals.evals) { e.to_bytes(out + off); off += row_bytes; }
    return 0;
}

template <int N> using M31L = LaneVec<M31, N>;
template <int N> using BnL = LaneVec<Bn254, N>;

}  // namespace refdrv

#define REF_M31(FN, ...)                                                                          \
    switch (lanes) {                                                                              \
        case 4: return refdrv::FN<refdrv::M31L<4>, refdrv::M31>(__VA_ARGS__);                     \
        case 8: return native ? refdrv::FN<gkr::M31_field::VectorizedM31, refdrv::M31>(__VA_ARGS__) \
                              : refdrv::FN<refdrv::M31L<8>, refdrv::M31>(__VA_ARGS__);            \
        case 16: return refdrv::FN<refdrv::M31L<16>, refdrv::M31>(__VA_ARGS__);                   \
        case 32: return refdrv::FN<refdrv::M31L<32>, refdrv::M31>(__VA_ARGS__);                   \
        case 48: return refdrv::FN<refdrv::M31L<48>, refdrv::M31>(__VA_ARGS__);                   \
        case 64: return refdrv::FN<refdrv::M31L<64>, refdrv::M31>(__VA_ARGS__);                   \
        case 128: return refdrv::FN<refdrv::M31L<128>, refdrv::M31>(__VA_ARGS__);                 \
        case 256: return refdrv::FN<refdrv::M31L<256>, refdrv::M31>(__VA_ARGS__);                 \
        case 1024: return refdrv::FN<refdrv::M31L<1024>, refdrv::M31>(__VA_ARGS__);               \
        default: return -1;                                                                       \
    }

#define REF_BN(FN, ...)                                                        \
    switch (lanes) {                                                           \
        case 4: return refdrv::FN<refdrv::BnL<4>, refdrv::Bn254>(__VA_ARGS__);   \
        case 8: return refdrv::FN<refdrv::BnL<8>, refdrv::Bn254>(__VA_ARGS__);   \
        case 16: return refdrv::FN<refdrv::BnL<16>, refdrv::Bn254>(__VA_ARGS__); \
        case 64: return refdrv::FN<refdrv::BnL<64>, refdrv::Bn254>(__VA_ARGS__); \
        default: return -1;                                                    \
    }

extern "C" {

// Lane counts this driver was instantiated for (0-terminated).
extern const int ref_supported_lanes[] = {4, 8, 16, 32, 48, 64, 128, 256, 1024, 0};
extern const int ref_supported_lanes_bn254[] = {4, 8, 16, 64, 0};

int ref_num_repetitions(int grinding_bits) { return refdrv::make_config(grinding_bits).get_num_repetitions(); }

// Prover::prove (include/LinearGKR/LinearGKR.hpp:58-90) on a circuit evaluated by
// Circuit::evaluate (include/circuit/circuit.hpp:273-280).  native=1 at lanes=8 uses the
// reference's own VectorizedM31 SIMD type.  Returns 0 on success, -1 for an
// unsupported lane count, 2 if proof_cap is too small (proof_len is still set).
int ref_prove(int lanes, int native, const ref_layer* layers, int nlayers, const uint32_t* input, int grinding_bits,
              uint8_t* proof_out, uint64_t proof_cap, uint64_t* proof_len, uint32_t* claimed_v) {
    REF_M31(prove_t, layers, nlayers, (const uint8_t*)input, (size_t)lanes * 4, grinding_bits, false, proof_out,
            proof_cap, proof_len, (uint8_t*)claimed_v)
}

// Verifier::verify (include/LinearGKR/LinearGKR.hpp:105-149).  Returns 1 accept, 0 reject.
int ref_verify(int lanes, int native, const ref_layer* layers, int nlayers, const uint32_t* input, int grinding_bits,
               const uint8_t* proof, uint64_t proof_len, const uint32_t* claimed_v) {
    REF_M31(verify_t, layers, nlayers, (const uint8_t*)input, (size_t)lanes * 4, grinding_bits, false, proof,
            proof_len, (const uint8_t*)claimed_v)
}

// Circuit::evaluate: writes every layer's input values followed by the last layer's output.
int ref_evaluate(int lanes, int native, const ref_layer* layers, int nlayers, const uint32_t* input, uint32_t* out) {
    REF_M31(evaluate_t, layers, nlayers, (const uint8_t*)input, (size_t)lanes * 4, (uint8_t*)out)
}

// The same three entry points over BN254 (Config::field_type = BN254: R = 1): values are
// rows of `lanes` 32-byte little-endian canonical elements.
int ref_prove_bn254(int lanes, const ref_layer* layers, int nlayers, const uint8_t* input, int grinding_bits,
                    uint8_t* proof_out, uint64_t proof_cap, uint64_t* proof_len, uint8_t* claimed_v) {
    REF_BN(prove_t, layers, nlayers, input, (size_t)lanes * 32, grinding_bits, true, proof_out, proof_cap, proof_len,
           claimed_v)
}
int ref_verify_bn254(int lanes, const ref_layer* layers, int nlayers, const uint8_t* input, int grinding_bits,
                     const uint8_t* proof, uint64_t proof_len, const uint8_t* claimed_v) {
    REF_BN(verify_t, layers, nlayers, input, (size_t)lanes * 32, grinding_bits, true, proof, proof_len, claimed_v)
}
int ref_evaluate_bn254(int lanes, const ref_layer* layers, int nlayers, const uint8_t* input, uint8_t* out) {
    REF_BN(evaluate_t, layers, nlayers, input, (size_t)lanes * 32, out)
}
int ref_num_repetitions_bn254(int grinding_bits) {
    return refdrv::make_config(grinding_bits, true).get_num_repetitions();
}

// BN254 field helpers for the tests (canonical 32-byte little-endian values).
void ref_bn254_mul(const uint8_t* a, const uint8_t* b, uint8_t* out) {
    bn_to_bytes(bn_mul(bn_from_bytes(a), bn_from_bytes(b)), out);
}
void ref_bn254_add(const uint8_t* a, const uint8_t* b, uint8_t* out) {
    bn_to_bytes(bn_add(bn_from_bytes(a), bn_from_bytes(b)), out);
}
void ref_bn254_sub(const uint8_t* a, const uint8_t* b, uint8_t* out) {
    bn_to_bytes(bn_sub(bn_from_bytes(a), bn_from_bytes(b)), out);
}
void ref_bn254_reduce(const uint8_t* a, uint8_t* out) { bn_to_bytes(bn_from_bytes(a), out); }

// SHA256Hasher::hash (include/hash/hashes.hpp:22-33) -> CSHA256.
void ref_sha256(const uint8_t* in, uint64_t len, uint8_t* out) {
    gkr::SHA256Hasher h;
    h.hash(out, in, (gkr::uint32)len);
}

// Circuit files through the reference's own loaders: CircuitRaw::operator>> and
// Circuit::from_circuit_raw (CIRCUIT2), or Circuit::load_extracted_gates (text files).
// The flattened layers stay in a static circuit read back with ref_loaded_layer.  Inputs
// must be well formed (the reference exits the process on a bad magic number).
static gkr::Circuit<refdrv::M31L<8>, refdrv::M31> g_loaded;

int ref_circuit2_load(const uint8_t* bytes, uint64_t len) {
    std::istringstream is(std::string((const char*)bytes, len), std::ios::binary);
    CircuitRaw<refdrv::M31> raw;
    is >> raw;
    g_loaded = gkr::Circuit<refdrv::M31L<8>, refdrv::M31>::from_circuit_raw(raw);
    return (int)g_loaded.layers.size();
}
int ref_extracted_load(const char* mul_path, const char* add_path) {
    g_loaded = gkr::Circuit<refdrv::M31L<8>, refdrv::M31>::load_extracted_gates(mul_path, add_path);
    return (int)g_loaded.layers.size();
}
// Sizes of layer l (counts, then the gates into mul: n_mul x {o, i0, i1, coef}, add:
// n_add x {o, i0, coef} when those are non-null).
void ref_loaded_layer(int l, uint32_t* nb_in, uint32_t* nb_out, uint64_t* n_mul, uint64_t* n_add, uint32_t* mul,
                      uint32_t* add) {
    const auto& L = g_loaded.layers[l];
    *nb_in = L.nb_input_vars;
    *nb_out = L.nb_output_vars;
    *n_mul = L.mul.sparse_evals.size();
    *n_add = L.add.sparse_evals.size();
    if (mul)
        for (size_t k = 0; k < L.mul.sparse_evals.size(); k++) {
            const auto& g = L.mul.sparse_evals[k];
            mul[4 * k] = g.o_id;
            mul[4 * k + 1] = g.i_ids[0];
            mul[4 * k + 2] = g.i_ids[1];
            mul[4 * k + 3] = g.coef.x;
        }
    if (add)
        for (size_t k = 0; k < L.add.sparse_evals.size(); k++) {
            const auto& g = L.add.sparse_evals[k];
            add[3 * k] = g.o_id;
            add[3 * k + 1] = g.i_ids[0];
            add[3 * k + 2] = g.coef.x;
        }
}

}
