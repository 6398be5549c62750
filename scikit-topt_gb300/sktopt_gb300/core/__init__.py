from .batch import BatchedDesigns
from .optimizers import (DensityMethod, DensityMethodConfig, DensityMethod_OC_Config,
                         LogMOC_Config, LogMOC_Optimizer, OC_Config, OC_Optimizer)

__all__ = ["BatchedDesigns", "DensityMethod", "DensityMethodConfig", "DensityMethod_OC_Config", "OC_Config",
           "OC_Optimizer", "LogMOC_Config", "LogMOC_Optimizer"]
