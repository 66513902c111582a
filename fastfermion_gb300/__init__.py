"""fastfermion_gb300: truncated Heisenberg-picture propagation of Pauli and
Majorana polynomials on NVIDIA GB300 (sm_103a).

Drop-in for fastfermion's propagation path: the same ``propagate`` signature,
gate types (H, S, CNOT, SWAP, CZ, ROT, MROT), polynomial types and product
states, backed by hand-written CUDA kernels in libffg (C ABI: include/ffg.h).
"""
from . import workloads
from .autotune import autotune
from .majorana import FockState, MajoranaPolynomial, MajoranaString, MROT, jw, majoranas
from .parse import poly
from .pauli import CNOT, CZ, H, MAX_QUBITS, ROT, S, SWAP, PauliPolynomial, PauliString, QubitProductState, paulis
from .propagation import (encode_majorana_circuit, encode_pauli_circuit, has_openmp, last_profile,
                          profile_disable, profile_get, profile_reset, propagate)

__version__ = "0.1.0"


def build_circuit(specs):
    """Instantiates the gate tuples of ``fastfermion_gb300.workloads``."""
    out = []
    for s in specs:
        if s[0] == "ROT":
            out.append(ROT(s[1], list(s[2]), s[3]))
        elif s[0] == "MROT":
            out.append(MROT(MajoranaString(list(s[1])), s[2], s[3]))
        else:
            out.append({"H": H, "S": S, "CNOT": CNOT, "SWAP": SWAP, "CZ": CZ}[s[0]](*s[1:]))
    return out


__all__ = ["PauliString", "PauliPolynomial", "MajoranaString", "MajoranaPolynomial", "H", "S",
           "CNOT", "SWAP", "CZ", "ROT", "MROT", "QubitProductState", "FockState", "propagate",
           "poly", "paulis", "majoranas", "profile_reset", "profile_disable", "profile_get",
           "last_profile", "has_openmp", "MAX_QUBITS", "build_circuit", "workloads",
           "encode_pauli_circuit", "encode_majorana_circuit", "jw", "autotune"]
