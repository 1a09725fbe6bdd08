"""CPU oracle for the Kronecker-free eigensolver hot path -- TEST INFRASTRUCTURE ONLY.

This package is a NumPy restatement of the reference's algorithms (KronFreeCircuits.jl):
single-mode bases and their port operators, the circuit term expansion, the
`KronFreeOperator` application, and the Dense / LOBPCG / Chebyshev-filter / Lanczos
solver policies.  It is the checker the GPU library is compared against.

Only `tests/`, `__graft_entry__.smoke()` and the CPU-baseline leg of `bench.py` may import
it.  The product (`libkfgpu.so` and its Python mirror `kfgpu`) never imports, links or runs
anything here; there is no CPU fallback through this package.

Parity pins: `tests/test_oracle_golden.py` checks this oracle against the reference's
committed scqubits golden energies (test/fixtures/scqubits_reference.json) and against the
reference's own known-answer constructions (test/test_materialize.jl:117-157).
"""
