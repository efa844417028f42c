"""CPU oracle of the HEXA TopOpt FE-solve path.

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline leg, always as what results are compared
against, never as the thing measured or shipped.  Parity status: parity
unpinned — the reference ships no tests, golden vectors or fixtures, and
Julia is not available to run it, so the oracle is
pinned by exact rational-arithmetic known answers (tests/golden) for the
element matrices and by first-principles properties (symmetry, rigid-body
null space, assembled-matrix direct solves) for the operators.
"""
