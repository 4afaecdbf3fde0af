"""CPU oracle for the selected-CI / CASCI hot path (test infrastructure only).

`macis_oracle.cpp` restates MACIS's sorted-double-loop Hamiltonian build,
Davidson eigensolver and spin-resolved RDMs (external/macis in
microsoft/qdk-chemistry) in plain C++/OpenMP.  Only `tests/`, the smoke check
in `__graft_entry__` and the CPU-baseline legs of `bench.py` use it, as the
checker; the GPU library never calls it.
"""
from .oracle import *  # noqa: F401,F403
