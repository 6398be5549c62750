from .solver_elastic import (FEM_SimpLinearElasticity, LinearSolverConfig,
                             normalize_linear_solver_config)

__all__ = ["FEM_SimpLinearElasticity", "LinearSolverConfig", "normalize_linear_solver_config"]
