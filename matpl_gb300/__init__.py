"""matpl_gb300 — GB300-native (sm_103a) DP / NEP evaluation path of MatPL.

Public surface:
  matpl_gb300.ops      CalcOps_cuda drop-ins (calculateForce, calculateVirial), GPU neighbor
                       search (find_neighbore) and environment matrix (env_mat)
  matpl_gb300.dp       DP: the reference DP.forward interface, fused on the GPU
  matpl_gb300.params   DPConfig, reference-named parameter init, davg/dstd statistics
  matpl_gb300.structures  seeded synthetic structures for tests and benchmarks
The native library (include/matpl_gb300.h) is built by matpl_gb300.build.build().
"""
from .params import DPConfig  # noqa: F401

__all__ = ["DPConfig"]
