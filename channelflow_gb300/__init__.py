"""GB300-native (sm_103a) channelflow DNS time step.

The compute path is libcfgpu.so (hand-written CUDA, C ABI in include/cfgpu.h);
this package holds its in-tree build script and a Python mirror of the
reference's DNS/DNSFlags API used by the tests and the benchmark.
"""

from .dns import DNS, DNSFlags, Ensemble, Grid, tau_solve_batched  # noqa: F401
