"""ORACLE -- CPU restatement of helios's closed-shell PPP CCSD path.

Test infrastructure only: the tests, the smoke check and the CPU-baseline leg of
the benchmark import it as the checker. The product (``helios_gb300``) never
imports, links or calls anything here.
"""
