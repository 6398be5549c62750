from .grid import (GridMesh, boundary_faces, create_box_hex, create_box_hex_len,
                   create_box_tet, elements_volume, element_centers, face_nodes,
                   get_elements_by_nodes, get_points_in_range)
from .task import FEMDomain, LinearElasticity, LinearHeatConduction
from . import toy_problem

__all__ = ["GridMesh", "create_box_hex", "create_box_hex_len", "create_box_tet",
           "elements_volume", "element_centers", "get_elements_by_nodes", "FEMDomain",
           "boundary_faces", "face_nodes", "get_points_in_range",
           "LinearElasticity", "LinearHeatConduction", "toy_problem"]
