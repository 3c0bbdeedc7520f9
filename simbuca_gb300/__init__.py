"""simbuca_gb300 -- the Simbuca integration hot path on GB300 (sm_103a).

Direct-sum Coulomb interaction, per-ion trap-field terms and the Dormand-Prince
5(4) stage / error-norm / step-control loop as hand-written CUDA kernels behind a
C ABI (include/simgb.h, libsimgb.so).  This package holds the build script, the
ctypes binding, the host mirror of the reference's IonCloud/force()/step()
interface and the benchmark workloads.
"""
from . import abi, constants  # noqa: F401

__all__ = ["abi", "constants", "api", "ode", "configs", "build"]
