from .common_density import DensityMethod, DensityMethodConfig, DensityMethod_OC_Config
from .logmoc import LogMOC_Config, LogMOC_Optimizer
from .oc import OC_Config, OC_Optimizer

__all__ = ["DensityMethod", "DensityMethodConfig", "DensityMethod_OC_Config", "OC_Config",
           "OC_Optimizer", "LogMOC_Config", "LogMOC_Optimizer"]
