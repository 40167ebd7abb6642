"""gkr_gb300: GB300-native GKR prover for data-parallel layered circuits (M31).

A drop-in for the prove path of PolyhedraZK/Expander-cpp: circuit load and evaluate,
gkr_prove, the SHA-256 Fiat-Shamir transcript and the RAW commitment, with the hot path
in hand-written sm_103a kernels behind the C ABI of include/gkrgpu.h (libgkrgpu.so).
"""
from .circuit import (P, Circuit, CircuitLayer, config1_circuit, config2_circuit, random_circuit, random_layer,
                      random_witness)

__all__ = ["P", "Circuit", "CircuitLayer", "config1_circuit", "config2_circuit", "random_circuit", "random_layer",
           "random_witness", "Config", "Context", "Prover", "Proof"]


def __getattr__(name):
    # The device-facing classes load libgkrgpu.so on first use, so the circuit model and
    # generators stay importable on machines without the built library.
    if name in ("Config", "Context", "Prover", "Proof", "DeviceCircuit"):
        from . import prover
        return getattr(prover, name)
    raise AttributeError(name)
