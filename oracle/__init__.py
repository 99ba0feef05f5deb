"""Test oracle for the halo-finding hot path (test infrastructure only).

Two checkers live here, and only tests/, the smoke check and the CPU-baseline
leg of bench.py may use them:
  * refcall      - the reference's own hot-path C sources compiled as-is
                   (oracle/ref/Makefile -> oracle/_ref/libref_rockstar.so);
                   available where the reference checkout is present.
  * restatement  - oracle/rockstar_oracle.c, a C restatement of the same
                   algorithm written for this project (built into
                   oracle/_build/liboracle.so), which travels with the
                   repository and runs anywhere.
"""
