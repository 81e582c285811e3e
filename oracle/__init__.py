"""Parity oracle (TEST INFRASTRUCTURE ONLY): a CPU restatement of the
reference's hot path (psph_oracle.c) and the recipe that builds the unmodified
reference as oracle/_ref. Only tests/, __graft_entry__.smoke() and bench.py's
CPU legs may use it."""
