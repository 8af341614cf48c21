"""CPU oracle for the GB300 CSEM solver - TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
package, and only as the checker. The product (demo_matrixfree_csem_gb300) never
imports, links or calls anything here.

  build_oracle()   compile csem_oracle.c + fft2d.c -> oracle/_build/libcsemoracle.so
  build_ref()      compile the unmodified reference sources (when present) with the
                   stubs in ref_stubs/ -> oracle/_ref/libcsemref.so
  Oracle           ctypes wrapper over libcsemoracle.so
  Ref              ctypes wrapper over libcsemref.so (reference built from its sources)
"""
from .pyoracle import (Oracle, Ref, build_oracle, build_ref, ref_available,  # noqa: F401
                       ORACLE_LIB, REF_LIB)
