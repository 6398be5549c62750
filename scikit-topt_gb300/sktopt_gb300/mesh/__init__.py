from .grid import (GridMesh, all_facets, boundary_faces, boundary_facets, create_box_hex,
                   create_box_hex_len, create_box_tet, elements_satisfying, elements_volume,
                   element_centers, face_nodes, facet_nodes_of, facets_satisfying,
                   get_elements_by_nodes, get_points_in_range, with_boundaries,
                   with_subdomains)
from .loader import basis_from_file, read_msh, write_msh
from .task import FEMDomain, LinearElasticity, LinearHeatConduction, assemble_surface_forces
from . import toy_problem

__all__ = ["GridMesh", "create_box_hex", "create_box_hex_len", "create_box_tet",
           "elements_volume", "element_centers", "get_elements_by_nodes", "FEMDomain",
           "boundary_faces", "face_nodes", "get_points_in_range", "boundary_facets",
           "facet_nodes_of", "read_msh", "write_msh", "basis_from_file", "all_facets",
           "facets_satisfying", "elements_satisfying", "with_boundaries", "with_subdomains",
           "assemble_surface_forces",
           "LinearElasticity", "LinearHeatConduction", "toy_problem"]
