"""CPU oracle for the Curvami Gauss-point hot path — test infrastructure only.

This package builds and loads ``curvami_oracle.cpp`` (a C++17 restatement of the
reference's FRNN, crease indicator, RKPM solve, sparsity pattern, face assembly,
elastic hinge and energies). Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline / reference arm of ``bench.py`` may import it, and only as the checker
or as the timed CPU baseline; the GPU library never calls it.

Parity status: the reference cannot be compiled (its hot-path headers need Eigen,
absent on both machines) and ships no golden vectors for this path, so bit-level
parity with the reference binary is unpinned. The oracle is pinned by the reference's
own invariants: RKPM reproducing conditions, central-difference consistency of the
tangent with the residual (the reference's TangentCheck, main.cpp:651-710) and of the
residual with the strain energy, and K symmetry — see tests/test_oracle_*.py.
"""
from .binding import Oracle, build_oracle, load_oracle  # noqa: F401
