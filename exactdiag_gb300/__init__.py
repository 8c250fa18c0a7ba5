"""GB300-native exact diagonalisation of the symmetry-adapted spin-1/2 t-J two-leg ladder.

Drop-in for exactdiag's t-J ladder path: ``exactdiag_gb300.tJ_spin_half_ladder``
mirrors ``exactdiag.tJ_spin_half_ladder`` (configs, api, matrix_setup) and
``exactdiag_gb300.general`` mirrors ``exactdiag.general`` (lanczos_diagonalization,
sparse_matrices).  Basis construction, H.v, the Lanczos recursions, the
excitation operators and the continued fraction run as CUDA kernels for sm_103a
in libexactdiag_gb300.so (C ABI: include/exactdiag_gb300.h).
"""

__version__ = "0.1.0"
