"""Test oracle for focss_gb300 (test infrastructure only).

``oracle.cpu`` wraps the FP64 C restatement (``focss_oracle.c``);
``oracle.ref`` wraps the reference's own sources compiled against the FFTW-API
shim (available only where the reference tree was present at build time).
Only tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this package.
"""
