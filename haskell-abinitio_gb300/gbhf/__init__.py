"""gbhf: GB300-native restricted Hartree-Fock hot path (libgbhf + host mirror).

``gbhf.hartree_fock`` mirrors the reference's Science.QuantumChemistry
functions; ``gbhf._lib`` is the ctypes binding of the C ABI in
include/gbhf.h; ``gbhf.basis`` and ``gbhf.molecules`` build inputs.
"""
from ._lib import GBHFError, NotConverged  # noqa: F401
