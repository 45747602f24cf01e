"""flexi_gb300: FLEXI's DGSEM Navier-Stokes right-hand side and LSERK stepper on GB300 (sm_103a).

The compute path is libflexigpu.so (hand-written CUDA, C ABI in include/flexi_gpu.h); this package
holds the in-tree build (build.py), its ctypes binding (_lib.py), the host-side mirror of FLEXI's
module interface (solver.py), the synthetic HOPR-style mesh generator (mesh.py) and the benchmark
initial states (testcases.py).
"""
from .solver import Flexi, FlexiError, config_dict, config_from_ini, make_config, probe_fp64_tflops  # noqa: F401
