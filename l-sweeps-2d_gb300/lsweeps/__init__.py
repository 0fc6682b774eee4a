"""Python side of the GB300 L-sweeps library: problem specs, synthetic media and
ctypes bindings to the C ABI declared in include/lsweeps.h."""
from .problems import ProblemSpec, config, small, omega_for_ppw  # noqa: F401
