"""CPU oracle for the Curvami Gauss-point hot path — test infrastructure only.

This package builds and loads ``curvami_oracle.cpp`` (a C++17 restatement of the
reference's FRNN, crease indicator, RKPM solve, sparsity pattern, face assembly,
elastic hinge and energies). Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline / reference arm of ``bench.py`` may import it, and only as the checker
or as the timed CPU baseline; the GPU library never calls it.

Parity status: the reference cannot be compiled (its hot-path headers need Eigen,
absent on both machines) and ships no golden Phi, K or neighbour vectors, so parity
with the reference binary at the bit level is unpinned. End to end the oracle is pinned
to the reference's one published result: driven through progressive creasing and
LineSearch on the smoke example (examples/smoke_centre_crease/README.md:14-20), it
reproduces the published last-step row (E_mem, E_ben, E_hin, mean fold angle) to every
printed digit with the published Newton counts (tests/test_creasing.py). Below that pin
it is held to the reference's own invariants: RKPM reproducing conditions,
central-difference consistency of the tangent with the residual (the reference's
TangentCheck, main.cpp:651-710) and of the residual with the strain energy, and K
symmetry (tests/test_oracle.py).
"""
from .binding import Oracle, build_oracle, load_oracle  # noqa: F401
