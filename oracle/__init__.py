"""CPU oracles for the EllipsesInFlows time-step hot path.

TEST INFRASTRUCTURE ONLY. Nothing in the product package imports this package;
only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it,
and only as the checker.

Two oracles live here:

* ``oracle.ref`` -- the reference solver's own unmodified C sources compiled
  with single-rank MPI/FFTW shims (oracle/ref/Makefile -> oracle/_ref/). It can
  be built only where the reference sources are present.
* ``oracle.port`` -- a plain-C restatement of the same algorithm
  (oracle/port/eif_port.c), compiled on any machine. It is pinned against
  ``oracle.ref`` and against the committed golden vectors in tests/golden/.
"""
