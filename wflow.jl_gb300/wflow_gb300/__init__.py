"""GB300-native SBM + kinematic-wave step for Wflow.jl: Python host mirror of the C ABI.

`Model` mirrors the parts of Wflow's model API that sit on the hot path
(`update_model!`, `run_timestep!`, BMI `update`/`get_value`/`set_value`); the compute runs in
the in-tree CUDA library through its C ABI.
"""

from . import abi, synthetic  # noqa: F401
