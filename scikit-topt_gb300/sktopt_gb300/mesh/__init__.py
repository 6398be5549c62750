from .grid import (GridMesh, create_box_hex, create_box_hex_len, create_box_tet,
                   elements_volume, element_centers, get_elements_by_nodes)
from .task import FEMDomain, LinearElasticity, LinearHeatConduction
from . import toy_problem

__all__ = ["GridMesh", "create_box_hex", "create_box_hex_len", "create_box_tet",
           "elements_volume", "element_centers", "get_elements_by_nodes", "FEMDomain",
           "LinearElasticity", "LinearHeatConduction", "toy_problem"]
