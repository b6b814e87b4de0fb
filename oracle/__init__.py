"""ORACLE — test infrastructure only.

CPU restatement of the reference's (hpi-epic/gpucsl) skeleton-discovery path, used as
the checker by tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py.
The product package (gpucsl_gb300) never imports anything from here.

Parity is pinned against the reference's own golden vectors (tests/golden/) and, where
the reference sources are present, against the reference's host-compilable helpers
compiled in place into oracle/_ref/ (see oracle/build.py).
"""
