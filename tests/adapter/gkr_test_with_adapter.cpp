// The body of the reference's GKR_WITH_PC_TEST (tests/GKR_Test.cpp:8-32) with the one-line
// prover swap of the drop-in adapter: gkr::Prover -> gkrgpu::Prover.  Compiled against the
// reference headers by tests/test_adapter.py; on a GPU machine the binary also runs it.
#include "field/M31.hpp"
#include "LinearGKR/LinearGKR.hpp"
#include "gkrgpu.hpp"

#include <cstdio>

int main() {
    using namespace gkr;
    using F = gkr::M31_field::VectorizedM31;
    using F_primitive = gkr::M31_field::M31;

    uint32 n_layers = 4;
    Circuit<F, F_primitive> circuit;
    for (int i = n_layers - 1; i >= 0; --i)
        circuit.layers.emplace_back(CircuitLayer<F, F_primitive>::random(1 << i, 1 << (i + 1)));
    circuit.evaluate();

    Config default_config{};
    try {
        gkrgpu::Prover<F, F_primitive> prover(default_config);
        prover.prepare_mem(circuit);
        auto t = prover.prove(circuit);
        auto claimed_v = std::get<0>(t);
        Proof<F> proof = std::get<1>(t);

        Prover<F, F_primitive> ref_prover(default_config);
        ref_prover.prepare_mem(circuit);
        auto rt = ref_prover.prove(circuit);
        const bool same = std::get<1>(rt).bytes == proof.bytes;

        Verifier verifier(default_config);
        bool verified = verifier.verify(circuit, claimed_v, proof);
        printf("adapter proof: %zu bytes, identical to reference: %d, verified: %d\n", proof.bytes.size(), same,
               verified);
        return (same && verified) ? 0 : 1;
    } catch (const std::exception& e) {
        printf("no GPU run: %s\n", e.what());
        return 77;
    }
}
