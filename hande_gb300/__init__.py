"""GB300-native FCIQMC walker-propagation engine with HANDE's calc interface.

    sys = hande_gb300.hubbard_k(lattice=[[4, 0], [0, 4]], electrons=10, U=4)
    out = hande_gb300.fciqmc(sys=sys, qmc=dict(tau=0.005, init_pop=10, mc_cycles=10,
                                               nreports=100, target_population=5e4, rng_seed=7))

The walker propagation runs in hand-written CUDA kernels (libhande_gpu.so,
C ABI in include/hande_gpu.h); this package holds the host-side system set-up
and the driver loop."""

from .systems import System, hubbard_k, read_in, synthetic_molecule, write_fcidump  # noqa: F401
from .calc import fciqmc  # noqa: F401
