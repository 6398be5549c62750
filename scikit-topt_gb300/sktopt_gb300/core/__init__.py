from . import autotune
from .batch import BatchedDesigns, gather_design_results, partition_designs, run_sharded
from .optimizers import (DensityMethod, DensityMethodConfig, DensityMethod_OC_Config,
                         LogMOC_Config, LogMOC_Optimizer, OC_Config, OC_Optimizer)

__all__ = ["autotune", "BatchedDesigns", "partition_designs", "gather_design_results", "run_sharded",
           "DensityMethod", "DensityMethodConfig", "DensityMethod_OC_Config", "OC_Config",
           "OC_Optimizer", "LogMOC_Config", "LogMOC_Optimizer"]
