"""ORACLE: test infrastructure only.

A CPU restatement of the reference RREA kinetic step (oracle_core.cpp) plus
the builder for the reference-compiled golden generator (Makefile.ref).
Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU baseline.
"""
