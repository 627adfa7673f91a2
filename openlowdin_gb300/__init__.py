"""GB300-native direct-SCF / MP2 integral path for openLOWDIN.

The package holds the CUDA library (liblowdin_gb300.so, built from csrc/ by
build.py) behind the reference's LibintInterface_* C ABI, its ctypes binding
(lint), the SCF drivers that call it (scf, batch_scf) and the synthetic
workload generators (systems).
"""
import os

# The SCF drivers diagonalise many small Fock matrices concurrently on a host
# thread pool; one BLAS thread per pool worker avoids oversubscribing the cores
# (measured on the 16-core Grace host: 11.8 ms -> 2.1 ms for 4 x 136^2 + 32 x 7^2).
# Takes effect when this package is imported before numpy.
os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
