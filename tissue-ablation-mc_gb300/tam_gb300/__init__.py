"""tam_gb300 -- GB300-native (sm_103a) hot paths of Tissue-Ablation-MC.

The product is the C ABI library ``libtam.so`` (include/tam.h): photon
transport and the fused heat / damage / ablation step as hand-written CUDA
kernels, with the reference's set-up and driver loop in host C++.  This
package is its Python binding and build recipe.
"""
from . import _abi
from ._abi import (TAM_F_ALPHA, TAM_F_COEFF, TAM_F_DENSITY, TAM_F_HEATCAP, TAM_F_JMEAN, TAM_F_JMEAN_GLOBAL,
                   TAM_F_KAPPA, TAM_F_MATERIAL, TAM_F_Q, TAM_F_RHOKAP, TAM_F_TEMP, TAM_F_THRESTIME, TAM_F_TISSUE,
                   TAM_F_WATER, Config, Params, State)
from .api import (Context, TamError, batch_autotune, batch_heat_steps, batch_mc_pass, batch_run, batch_step_coupled, default_config, default_params, read_config, kernel_launches, tally_atomics_per_second,
                  read_input_params, selftest_philox, set_material)

__all__ = [
    "Context", "TamError", "Config", "Params", "State", "default_params", "default_config", "read_input_params",
    "selftest_philox", "set_material", "read_config", "kernel_launches", "batch_run", "batch_step_coupled", "batch_heat_steps", "batch_mc_pass", "batch_autotune", "_abi",
    "TAM_F_TEMP", "TAM_F_RHOKAP", "TAM_F_JMEAN", "TAM_F_JMEAN_GLOBAL", "TAM_F_TISSUE", "TAM_F_THRESTIME",
    "TAM_F_KAPPA", "TAM_F_DENSITY", "TAM_F_HEATCAP", "TAM_F_COEFF", "TAM_F_ALPHA", "TAM_F_Q", "TAM_F_WATER",
    "TAM_F_MATERIAL",
]
