// Test infrastructure only: a thin extern "C" driver around the UNMODIFIED reference
// prover and verifier (PolyhedraZK/Expander-cpp, header-only templates).  It is compiled
// from the reference's own headers by oracle/build_ref.sh into oracle/_ref/ and is used
// by the CPU tests to pin the C restatement (oracle/gkr_oracle.c) and to generate the
// golden fixtures under tests/golden/.  Nothing in the product links or calls it.
//
// The reference packs 8 circuit copies per field element on x86 (VectorizedM31,
// include/field/M31.hpp:240-449).  To run its templates with other copy counts this
// driver supplies LaneVec<N>, an N-lane element whose arithmetic calls the reference's
// own scalar M31 operators (include/field/M31.hpp:64-93).  At N=8 the proofs of
// LaneVec<8> and of VectorizedM31 are compared byte for byte by the tests.
//
// Everything the reference headers define must live in exactly one translation unit
// (include/field/M31.hpp:451-452 and include/utils/myutil.hpp define non-inline symbols).

#include "field/M31.hpp"
#include "LinearGKR/LinearGKR.hpp"

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <unistd.h>
#include <fcntl.h>

namespace refdrv {

using gkr::M31_field::M31;
static const uint32_t P = 2147483647u;

template <int N>
struct Lanes {
    uint32_t v[N];
    static uint32_t ladd(uint32_t a, uint32_t b) { return (M31::new_unchecked(a) + M31::new_unchecked(b)).x; }
    static uint32_t lsub(uint32_t a, uint32_t b) { return (M31::new_unchecked(a) - M31::new_unchecked(b)).x; }
    static uint32_t lmul(uint32_t a, uint32_t b) { return (M31::new_unchecked(a) * M31::new_unchecked(b)).x; }
    Lanes operator+(const Lanes& o) const { Lanes r; for (int i = 0; i < N; i++) r.v[i] = ladd(v[i], o.v[i]); return r; }
    Lanes operator-(const Lanes& o) const { Lanes r; for (int i = 0; i < N; i++) r.v[i] = lsub(v[i], o.v[i]); return r; }
    Lanes operator*(const Lanes& o) const { Lanes r; for (int i = 0; i < N; i++) r.v[i] = lmul(v[i], o.v[i]); return r; }
    Lanes operator*(const M31& s) const { Lanes r; for (int i = 0; i < N; i++) r.v[i] = lmul(v[i], s.x); return r; }
    void operator+=(const Lanes& o) { *this = *this + o; }
    bool operator==(const Lanes& o) const { return memcmp(v, o.v, sizeof(v)) == 0; }
};

// N-lane stand-in for VectorizedM31: one Lanes<N> "packed" element, because the
// reference indexes .elements[j] for j < vectorize_size (== 1 on x86),
// include/LinearGKR/sumcheck_helper.hpp:82-97,113-126.
template <int N>
struct LaneVec {
    typedef M31 primitive_type;
    Lanes<N> elements[1];
    static LaneVec INV_2;

    LaneVec() { memset(elements[0].v, 0, sizeof(elements[0].v)); }
    LaneVec(uint32_t x) { M31 m(x); if (m.x >= P) m.x -= P; for (int i = 0; i < N; i++) elements[0].v[i] = m.x; }
    static LaneVec zero() { return LaneVec(); }
    static LaneVec one() { return LaneVec(1u); }
    static size_t pack_size() { return N; }

    LaneVec operator+(const LaneVec& o) const { LaneVec r; r.elements[0] = elements[0] + o.elements[0]; return r; }
    LaneVec operator-(const LaneVec& o) const { LaneVec r; r.elements[0] = elements[0] - o.elements[0]; return r; }
    LaneVec operator-() const { return LaneVec() - *this; }
    LaneVec operator*(const LaneVec& o) const { LaneVec r; r.elements[0] = elements[0] * o.elements[0]; return r; }
    LaneVec operator*(const M31& s) const { LaneVec r; r.elements[0] = elements[0] * s; return r; }
    LaneVec operator*(const int& s) const { return *this * LaneVec((uint32_t)s); }
    LaneVec operator+(const M31& s) const { return *this + LaneVec(s.x); }
    void operator+=(const LaneVec& o) { *this = *this + o; }
    void operator-=(const LaneVec& o) { *this = *this - o; }
    void operator*=(const LaneVec& o) { *this = *this * o; }
    bool operator==(const LaneVec& o) const { return elements[0] == o.elements[0]; }

    // Same byte layout as VectorizedM31::to_bytes/from_bytes (M31.hpp:420-434,
    // M31_avx.tcc:62-67): N little-endian u32 lanes, reduced on read.
    void to_bytes(uint8_t* out) const { memcpy(out, elements[0].v, 4 * N); }
    void from_bytes(const uint8_t* in) {
        memcpy(elements[0].v, in, 4 * N);
        for (int i = 0; i < N; i++) {
            uint32_t x = elements[0].v[i];
            x = (x & P) + (x >> 31);
            if (x >= P) x -= P;
            elements[0].v[i] = x;
        }
    }
};
template <int N> LaneVec<N> LaneVec<N>::INV_2 = LaneVec<N>(1u << 30);

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

template <class F>
static gkr::Circuit<F, M31> build_circuit(const ref_layer* layers, int nlayers, const uint32_t* input, int lanes) {
    gkr::Circuit<F, M31> c;
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
            G.o_id = s[0]; G.i_ids[0] = s[1]; G.i_ids[1] = s[2]; G.coef = M31(s[3]);
        }
        L.add.sparse_evals.resize(layers[l].n_add);
        for (uint64_t g = 0; g < layers[l].n_add; g++) {
            const uint32_t* s = layers[l].add + 3 * g;
            auto& G = L.add.sparse_evals[g];
            G.o_id = s[0]; G.i_ids[0] = s[1]; G.coef = M31(s[2]);
        }
    }
    uint64_t I0 = 1ull << layers[0].nb_input_vars;
    auto& ev = c.layers[0].input_layer_vals.evals;
    ev.resize(I0);
    for (uint64_t i = 0; i < I0; i++) ev[i].from_bytes((const uint8_t*)(input + i * lanes));
    c.evaluate();
    return c;
}

static ::Config make_config(int grinding_bits) {
    ::Config cfg;
    cfg.grinding_bits = grinding_bits;
    cfg.initialize_config();
    return cfg;
}

// Silences the verifier's progress prints (include/LinearGKR/LinearGKR.hpp:143-144).
struct Mute {
    int saved;
    Mute() { fflush(stdout); std::cout.flush(); saved = dup(1); int dn = open("/dev/null", O_WRONLY); dup2(dn, 1); close(dn); }
    ~Mute() { fflush(stdout); std::cout.flush(); dup2(saved, 1); close(saved); }
};

template <class F>
static int prove_t(const ref_layer* layers, int nlayers, int lanes, const uint32_t* input, int grinding_bits,
                   uint8_t* proof_out, uint64_t proof_cap, uint64_t* proof_len, uint32_t* claimed_v) {
    auto circuit = build_circuit<F>(layers, nlayers, input, lanes);
    ::Config cfg = make_config(grinding_bits);
    gkr::Prover<F, M31> prover(cfg);
    prover.prepare_mem(circuit);
    auto t = prover.prove(circuit);
    auto& cv = std::get<0>(t);
    auto& proof = std::get<1>(t);
    *proof_len = proof.bytes.size();
    if (proof.bytes.size() > proof_cap) return 2;
    memcpy(proof_out, proof.bytes.data(), proof.bytes.size());
    for (size_t j = 0; j < cv.size(); j++) cv[j].to_bytes((uint8_t*)(claimed_v + j * lanes));
    return 0;
}

template <class F>
static int verify_t(const ref_layer* layers, int nlayers, int lanes, const uint32_t* input, int grinding_bits,
                    const uint8_t* proof_bytes, uint64_t proof_len, const uint32_t* claimed_v) {
    auto circuit = build_circuit<F>(layers, nlayers, input, lanes);
    ::Config cfg = make_config(grinding_bits);
    gkr::Proof<F> proof;
    proof.bytes.assign(proof_bytes, proof_bytes + proof_len);
    std::vector<F> cv(cfg.get_num_repetitions());
    for (int j = 0; j < cfg.get_num_repetitions(); j++) cv[j].from_bytes((const uint8_t*)(claimed_v + (size_t)j * lanes));
    gkr::Verifier verifier(cfg);
    bool ok;
    {
        Mute m;
        ok = verifier.verify(circuit, cv, proof);
    }
    return ok ? 1 : 0;
}

template <class F>
static int evaluate_t(const ref_layer* layers, int nlayers, int lanes, const uint32_t* input, uint32_t* out) {
    auto circuit = build_circuit<F>(layers, nlayers, input, lanes);
    uint64_t off = 0;
    for (int l = 0; l < nlayers; l++) {
        for (auto& e : circuit.layers[l].input_layer_vals.evals) { e.to_bytes((uint8_t*)(out + off)); off += lanes; }
    }
    for (auto& e : circuit.layers.back().output_layer_vals.evals) { e.to_bytes((uint8_t*)(out + off)); off += lanes; }
    return 0;
}

}  // namespace refdrv

#define REF_DISPATCH(FN, ...)                                                              \
    switch (lanes) {                                                                       \
        case 4: return refdrv::FN<refdrv::LaneVec<4>>(__VA_ARGS__);                        \
        case 8: return native ? refdrv::FN<gkr::M31_field::VectorizedM31>(__VA_ARGS__)     \
                              : refdrv::FN<refdrv::LaneVec<8>>(__VA_ARGS__);               \
        case 16: return refdrv::FN<refdrv::LaneVec<16>>(__VA_ARGS__);                      \
        case 32: return refdrv::FN<refdrv::LaneVec<32>>(__VA_ARGS__);                      \
        case 48: return refdrv::FN<refdrv::LaneVec<48>>(__VA_ARGS__);                      \
        case 64: return refdrv::FN<refdrv::LaneVec<64>>(__VA_ARGS__);                      \
        case 128: return refdrv::FN<refdrv::LaneVec<128>>(__VA_ARGS__);                    \
        case 256: return refdrv::FN<refdrv::LaneVec<256>>(__VA_ARGS__);                    \
        case 1024: return refdrv::FN<refdrv::LaneVec<1024>>(__VA_ARGS__);                  \
        default: return -1;                                                                \
    }

extern "C" {

// Lane counts this driver was instantiated for (0-terminated).
extern const int ref_supported_lanes[] = {4, 8, 16, 32, 48, 64, 128, 256, 1024, 0};

int ref_num_repetitions(int grinding_bits) { return refdrv::make_config(grinding_bits).get_num_repetitions(); }

// Prover::prove (include/LinearGKR/LinearGKR.hpp:58-90) on a circuit evaluated by
// Circuit::evaluate (include/circuit/circuit.hpp:273-280).  native=1 at lanes=8 uses the
// reference's own VectorizedM31 SIMD type.  Returns 0 on success, -1 for an
// unsupported lane count, 2 if proof_cap is too small (proof_len is still set).
int ref_prove(int lanes, int native, const ref_layer* layers, int nlayers, const uint32_t* input, int grinding_bits,
              uint8_t* proof_out, uint64_t proof_cap, uint64_t* proof_len, uint32_t* claimed_v) {
    REF_DISPATCH(prove_t, layers, nlayers, lanes, input, grinding_bits, proof_out, proof_cap, proof_len, claimed_v)
}

// Verifier::verify (include/LinearGKR/LinearGKR.hpp:105-149).  Returns 1 accept, 0 reject.
int ref_verify(int lanes, int native, const ref_layer* layers, int nlayers, const uint32_t* input, int grinding_bits,
               const uint8_t* proof, uint64_t proof_len, const uint32_t* claimed_v) {
    REF_DISPATCH(verify_t, layers, nlayers, lanes, input, grinding_bits, proof, proof_len, claimed_v)
}

// Circuit::evaluate: writes every layer's input values followed by the last layer's output.
int ref_evaluate(int lanes, int native, const ref_layer* layers, int nlayers, const uint32_t* input, uint32_t* out) {
    REF_DISPATCH(evaluate_t, layers, nlayers, lanes, input, out)
}

// SHA256Hasher::hash (include/hash/hashes.hpp:22-33) -> CSHA256.
void ref_sha256(const uint8_t* in, uint64_t len, uint8_t* out) {
    gkr::SHA256Hasher h;
    h.hash(out, in, (gkr::uint32)len);
}

}
