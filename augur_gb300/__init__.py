"""augur_gb300 — GB300-native (sm_103a) particle-mesh gravity step and scatter-field CNN.

The compute path is hand-written CUDA in augur_gb300/csrc, exported as the C ABI of
include/augur_pm.h and loaded here with ctypes. There is no CPU implementation in this
package: calls on CPU tensors raise.
"""
from .pm import PMPlan, direct_sum_fp64, energy_fp64
from .scatter_field import ScatterField, pm_acc
from .field2d import ChunkedTick2D, UNetScatterField

__all__ = ["PMPlan", "ScatterField", "UNetScatterField", "ChunkedTick2D", "pm_acc", "direct_sum_fp64", "energy_fp64"]
