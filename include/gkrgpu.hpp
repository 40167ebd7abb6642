// C++ drop-in adapter over the gkrgpu C ABI with the interface of the reference's
// gkr::Prover (PolyhedraZK/Expander-cpp, include/LinearGKR/LinearGKR.hpp:34-91):
//
//     gkrgpu::Prover<F, F_primitive> prover(config);     // was gkr::Prover<F, F_primitive>
//     prover.prepare_mem(circuit);
//     auto [claimed_v, proof] = prover.prove(circuit);   // tuple<vector<F>, gkr::Proof<F>>
//
// Include it after the reference's "LinearGKR/LinearGKR.hpp".  F is any vector field type
// whose to_bytes/from_bytes write N little-endian u32 lanes (VectorizedM31: N = 8 on x86);
// the proof bytes are the reference prover's bytes for the same circuit and input.
// Errors from the library are thrown as std::runtime_error (the reference asserts).
#pragma once

#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "gkrgpu.h"

namespace gkrgpu {

template <typename F, typename F_primitive, typename ConfigT = ::Config>
class Prover {
   public:
    const ConfigT& config;

    explicit Prover(const ConfigT& config_, int device = 0) : config(config_) {
        check(gkrgpu_create(device, &ctx_), "gkrgpu_create");
    }
    ~Prover() {
        if (circuit_) gkrgpu_circuit_free(circuit_);
        if (ctx_) gkrgpu_destroy(ctx_);
    }
    Prover(const Prover&) = delete;
    Prover& operator=(const Prover&) = delete;

    // Uploads the circuit's wiring once (the reference allocates its scratch pads here,
    // LinearGKR.hpp:49-56).  Re-uploads when called with another circuit.
    void prepare_mem(const gkr::Circuit<F, F_primitive>& circuit) {
        if (loaded_from_ == &circuit) return;
        std::vector<gkrgpu_layer_desc> descs(circuit.layers.size());
        std::vector<std::vector<gkrgpu_mul_gate>> muls(circuit.layers.size());
        std::vector<std::vector<gkrgpu_add_gate>> adds(circuit.layers.size());
        for (size_t l = 0; l < circuit.layers.size(); l++) {
            const auto& L = circuit.layers[l];
            for (const auto& g : L.mul.sparse_evals) muls[l].push_back({g.o_id, g.i_ids[0], g.i_ids[1], coef(g.coef)});
            for (const auto& g : L.add.sparse_evals) adds[l].push_back({g.o_id, g.i_ids[0], coef(g.coef)});
            descs[l] = {L.nb_output_vars, L.nb_input_vars, muls[l].size(), adds[l].size(), muls[l].data(),
                        adds[l].data()};
        }
        if (circuit_) gkrgpu_circuit_free(circuit_);
        circuit_ = nullptr;
        check(gkrgpu_circuit_load(ctx_, descs.data(), (int)descs.size(), &circuit_), "gkrgpu_circuit_load");
        loaded_from_ = &circuit;
    }

    // Prover::prove (LinearGKR.hpp:58-90): RAW commitment of layers[0]'s input values,
    // grinding, gkr_prove, empty openings.  Returns (claimed_v, proof).
    std::tuple<std::vector<F>, gkr::Proof<F>> prove(const gkr::Circuit<F, F_primitive>& circuit) {
        prepare_mem(circuit);
        const uint32_t lanes = sizeof(F) / 4;
        const auto& in = circuit.layers[0].input_layer_vals.evals;
        std::vector<uint32_t> input(in.size() * lanes);
        for (size_t i = 0; i < in.size(); i++) in[i].to_bytes(reinterpret_cast<uint8_t*>(input.data() + i * lanes));
        const int grinding = config.grinding_bits;
        const uint64_t need = gkrgpu_proof_size(circuit_, lanes, grinding);
        gkr::Proof<F> proof;
        proof.bytes.resize(need);
        const int reps = gkrgpu_num_repetitions(grinding);
        std::vector<uint32_t> cv((size_t)reps * lanes);
        uint64_t len = 0;
        check(gkrgpu_prove(ctx_, circuit_, lanes, grinding, input.data(), proof.bytes.data(), need, &len, cv.data()),
              "gkrgpu_prove");
        proof.bytes.resize(len);
        std::vector<F> claimed_v(reps);
        for (int j = 0; j < reps; j++) claimed_v[j].from_bytes(reinterpret_cast<const uint8_t*>(cv.data() + (size_t)j * lanes));
        return {claimed_v, proof};
    }

   private:
    gkrgpu_ctx* ctx_ = nullptr;
    gkrgpu_circuit* circuit_ = nullptr;
    const void* loaded_from_ = nullptr;

    static uint32_t coef(const F_primitive& c) {
        uint32_t x = 0;
        c.to_bytes(reinterpret_cast<uint8_t*>(&x));
        return x;
    }
    static void check(int rc, const char* what) {
        if (rc != GKRGPU_OK) throw std::runtime_error(std::string(what) + ": " + gkrgpu_last_error());
    }
};

}  // namespace gkrgpu
