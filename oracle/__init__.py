"""ORACLE -- CPU restatement of helios's closed-shell PPP CCSD path.

Test infrastructure only: the tests, the smoke check and the CPU-baseline leg of
the benchmark import it as the checker. The product (``helios_gb300``) never
imports, links or calls anything here.

Parity unpinned: the reference's own tests hold no golden vectors for this
path, and the reference (Fortran with compiler-specific extensions and no
build files) cannot be built or run here. The restatement is pinned instead
by the agreement of independent codes (literal, factorised and textbook
spin-orbital CCSD; the reference's spin-orbital (T) loop and the published
(T); the reference's LR-CCSD sigma equations and the exact determinant-space
similarity-transformed Hamiltonian) and by exact invariants, in
tests/test_oracle.py, tests/test_oracle_triples.py and
tests/test_oracle_lrccsd.py.
"""
