"""GB300-native kinetic Monte Carlo engine for dopant networks.

The hop loop of the reference's ``kmc_dn`` (numba ``_simulate_discrete_record``
and the Go ``simulate``) runs here as hand-written sm_103a CUDA kernels behind
a C ABI (``include/kmc_dn_gb300.h``); this package is the Python host side:
set-up numerics, the ``kmc_dn``-compatible class with ``cuda_simulation``,
the batched engine and the serving loop.
"""
__version__ = "0.1.0"
