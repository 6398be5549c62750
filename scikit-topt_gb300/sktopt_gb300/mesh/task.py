"""Problem definitions: boundary sets, design sets and loads.

Mirrors ``FEMDomain.from_nodes`` (sktopt/mesh/task_common.py:105-270),
``exlude_dirichlet_from_design`` (task_common.py:398-401), ``LinearElasticity``
(sktopt/mesh/task_elastic.py:85-147) and ``LinearHeatConduction``
(sktopt/mesh/task_heat.py:142-321): elements touching load nodes leave the
design set, elements touching Dirichlet nodes leave it when the optimizer's
``design_dirichlet`` is False, and DOFs are interleaved ``bs*node + comp``.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .grid import (GridMesh, boundary_faces, elements_volume, face_nodes,
                   get_elements_by_nodes, setdiff1d)

_COMP = {"u^1": 0, "u^2": 1, "u^3": 2}


@dataclass
class FEMDomain:
    mesh: GridMesh
    dirichlet_nodes: np.ndarray
    dirichlet_dofs: np.ndarray
    dirichlet_elements: np.ndarray
    neumann_nodes: np.ndarray | list | None
    neumann_elements: np.ndarray
    design_elements: np.ndarray
    free_dofs: np.ndarray
    all_elements: np.ndarray
    fixed_elements: np.ndarray
    dirichlet_neumann_elements: np.ndarray
    elements_volume: np.ndarray
    bs: int = 3

    @property
    def design_mask(self) -> np.ndarray:
        return np.isin(self.all_elements, self.design_elements)

    @property
    def n_dof(self) -> int:
        return self.bs * self.mesh.nnodes

    @property
    def dirichlet_mask(self) -> np.ndarray:
        m = np.zeros(self.n_dof, dtype=np.uint8)
        m[self.dirichlet_dofs] = 1
        return m

    def exlude_dirichlet_from_design(self):
        """task_common.py:398-401."""
        self.design_elements = setdiff1d(self.design_elements, self.dirichlet_elements)

    @staticmethod
    def _sets(mesh, bs, dirichlet_nodes, dirichlet_dir, neumann_nodes, design_elements):
        """task_common.py:105-270.  ``dirichlet_nodes`` may be a list of node
        sets with a list of directions (one per set, task_common.py:140-160)."""
        if isinstance(dirichlet_nodes, list):
            dirs = dirichlet_dir if isinstance(dirichlet_dir, list) else \
                [dirichlet_dir] * len(dirichlet_nodes)
            parts = [FEMDomain._dofs(bs, n, d) for n, d in zip(dirichlet_nodes, dirs)]
            ddofs = np.unique(np.concatenate(parts)) if parts else np.array([], np.int64)
            dn = np.unique(np.concatenate([np.asarray(n, dtype=np.int64).ravel()
                                           for n in dirichlet_nodes])) \
                if dirichlet_nodes else np.array([], np.int64)
        else:
            dn = np.unique(np.asarray(dirichlet_nodes, dtype=np.int64))
            ddofs = FEMDomain._dofs(bs, dn, dirichlet_dir)
        dir_el = get_elements_by_nodes(mesh, [dn]) if dn.size else np.array([], np.int32)
        if neumann_nodes is not None:
            nn = neumann_nodes if isinstance(neumann_nodes, list) else [neumann_nodes]
            neu_el = get_elements_by_nodes(mesh, nn)
            if neu_el.size == 0:
                raise ValueError("neumann_elements has not been set.")
        else:
            neu_el = np.array([], dtype=np.int32)
        design = setdiff1d(np.asarray(design_elements), neu_el)
        if design.size == 0:
            raise ValueError("design_elements is empty")
        all_el = np.arange(mesh.nelements)
        fixed = setdiff1d(all_el, design)
        dn_el = np.concatenate([v for v in (dir_el, neu_el) if v.size > 0]) \
            if (dir_el.size + neu_el.size) else np.array([], dtype=np.int64)
        free = setdiff1d(np.arange(bs * mesh.nnodes), ddofs)
        return dict(dirichlet_nodes=dn, dirichlet_dofs=ddofs, dirichlet_elements=dir_el,
                    neumann_elements=neu_el, design_elements=design, free_dofs=free,
                    all_elements=all_el, fixed_elements=fixed,
                    dirichlet_neumann_elements=dn_el,
                    elements_volume=elements_volume(mesh))


    @staticmethod
    def _dofs(bs, nodes, direction):
        nodes = np.unique(np.asarray(nodes, dtype=np.int64))
        comps = np.arange(bs) if (direction in (None, "all") or bs == 1) else \
            np.array([_COMP[direction]])
        return np.sort((bs * nodes[:, None] + comps[None, :]).ravel())


def _group_list(x):
    return x if isinstance(x, list) else [x]


def _tag_groups(tags: dict, prefix: str):
    """Facet groups named ``prefix_<k>`` in k order, else ``prefix``
    (the key rules of from_mesh_tags, task_elastic.py:266-317)."""
    import re
    keys = sorted([k for k in tags if re.match(rf"{prefix}_\d+$", k)],
                  key=lambda x: int(re.search(r"\d+$", x).group()))
    if keys:
        return [tags[k] for k in keys]
    if prefix in tags:
        return [tags[prefix]]
    return None


def _facet_integrals(mesh, facets):
    """Area and int N_a over each facet (rows (element, local face)): 2x2
    Gauss on the bilinear map of a hexahedron face, exact for a triangle."""
    from .grid import HEX_OFFSETS, element_faces
    faces = element_faces(mesh.kind)
    facets = np.asarray(facets, dtype=np.int64).reshape(-1, 2)
    k = len(faces[0])
    nodes = np.zeros((facets.shape[0], k), dtype=np.int64)
    area = np.zeros(facets.shape[0])
    integ = np.zeros((facets.shape[0], k))
    g = 0.5 / np.sqrt(3.0)
    gp = (0.5 - g, 0.5 + g)
    for i, (e, f) in enumerate(facets):
        loc = faces[f]
        nodes[i] = mesh.t[loc, e]
        X = mesh.p[:, nodes[i]]
        if mesh.kind == "hex":
            ax = [d for d in range(3) if d != f // 2]
            uv = HEX_OFFSETS[loc][:, ax]
            for s_ in gp:
                for t_ in gp:
                    Nf = np.array([(s_ if o[0] else 1 - s_) * (t_ if o[1] else 1 - t_)
                                   for o in uv])
                    dS = np.array([(1.0 if o[0] else -1.0) * (t_ if o[1] else 1 - t_)
                                   for o in uv])
                    dT = np.array([(s_ if o[0] else 1 - s_) * (1.0 if o[1] else -1.0)
                                   for o in uv])
                    jac = np.linalg.norm(np.cross(X @ dS, X @ dT))
                    area[i] += 0.25 * jac
                    integ[i] += 0.25 * jac * Nf
        else:
            a = 0.5 * np.linalg.norm(np.cross(X[:, 1] - X[:, 0], X[:, 2] - X[:, 0]))
            area[i] = a
            integ[i] = a / 3.0
    return nodes, area, integ


def assemble_surface_forces(mesh, force_facets, force_dir_type, force_value) -> list:
    """task_elastic.py:15-81: for each facet group, a uniform traction of
    value / (group area) along component u^1..u^3, integrated against the
    shape functions; one load vector (3 n_nodes) per group."""
    facets_list = _group_list(force_facets)
    dirs = _group_list(force_dir_type)
    vals = _group_list(force_value)
    if not (len(facets_list) == len(dirs) == len(vals)):
        raise ValueError("Lengths of force_facets_ids, force_dir_type, and force_value "
                         "must match when lists.")
    out = []
    for fac, d, v in zip(facets_list, dirs, vals):
        if not (isinstance(d, str) and d.startswith("u^") and d[2:].isdigit()):
            raise ValueError(f"force_dir_type must be like 'u^1','u^2','u^3', got: {d}")
        comp = int(d[2:]) - 1
        nodes, area, integ = _facet_integrals(mesh, fac)
        pressure = float(v) / float(np.sum(area))
        F = np.zeros(3 * mesh.nnodes)
        np.add.at(F, 3 * nodes.ravel() + comp, (pressure * integ).ravel())
        out.append(F)
    return out


@dataclass
class LinearElasticity(FEMDomain):
    E: float = 1.0
    nu: float = 0.3
    neumann_linear: list = field(default_factory=list)

    @property
    def material_coef(self) -> float:
        return self.E

    @property
    def n_tasks(self) -> int:
        return len(self.neumann_linear)

    @classmethod
    def from_nodes(cls, mesh, dirichlet_nodes, dirichlet_dir, neumann_nodes,
                   neumann_linear, design_elements, E, nu):
        """task_common.py:105-270 with nodal load vectors (one per load case)."""
        s = FEMDomain._sets(mesh, 3, dirichlet_nodes, dirichlet_dir, neumann_nodes,
                            design_elements)
        loads = neumann_linear if isinstance(neumann_linear, list) else [neumann_linear]
        loads = [np.ascontiguousarray(f, dtype=np.float64) for f in loads]
        return cls(mesh=mesh, neumann_nodes=neumann_nodes, bs=3, E=float(E), nu=float(nu),
                   neumann_linear=loads, **s)

    @classmethod
    def from_facets(cls, mesh, dirichlet_facets, dirichlet_dir, force_facets, force_dir_type,
                    force_value, design_elements, E, nu):
        """task_elastic.py:152-258 and task_common.py:273-347: Dirichlet nodes
        from the facets (one node set per facet group), force nodes from the
        force facets (their elements leave the design set), and one surface
        load vector per force group (assemble_surface_forces)."""
        from .grid import facet_nodes_of
        if isinstance(dirichlet_facets, list):
            dn = [np.unique(facet_nodes_of(mesh, f)) for f in dirichlet_facets]
        else:
            dn = np.unique(facet_nodes_of(mesh, dirichlet_facets))
        ff = np.concatenate([np.asarray(f, dtype=np.int64).reshape(-1, 2)
                             for f in _group_list(force_facets)])
        nn = np.unique(facet_nodes_of(mesh, ff))
        loads = assemble_surface_forces(mesh, force_facets, force_dir_type, force_value)
        return cls.from_nodes(mesh, dn, dirichlet_dir, nn, loads, design_elements, E, nu)

    @classmethod
    def from_mesh_tags(cls, mesh, dirichlet_dir, neumann_dir_type, neumann_values, E, nu):
        """task_elastic.py:266-317: facet groups ``dirichlete_<k>`` (the
        reference's spelling) or ``dirichlet``, ``neumann_<k>`` or ``neumann``,
        design elements from the ``design`` subdomain."""
        design = mesh.subdomains["design"]
        dir_f = _tag_groups(mesh.boundaries, "dirichlete")
        if dir_f is None:
            dir_f = [mesh.boundaries["dirichlet"]] if "dirichlet" in mesh.boundaries else []
        if len(dir_f) == 1 and not isinstance(dirichlet_dir, list):
            dir_f = dir_f[0]
        neu_f = _tag_groups(mesh.boundaries, "neumann") or []
        if len(neu_f) == 1 and not isinstance(neumann_dir_type, list):
            neu_f = neu_f[0]
        return cls.from_facets(mesh, dir_f, dirichlet_dir, neu_f, neumann_dir_type,
                               neumann_values, design, E, nu)


@dataclass
class LinearHeatConduction(FEMDomain):
    """task_heat.py:142-321.

    ``dirichlet_values``: one temperature, or a list (one load case per
    value on the same Dirichlet nodes).  ``emit``: optional volumetric
    source (nodal load; the reference has none).  Robin data
    (task_common.py:76-81): ``robin_faces`` -- an (n, 3) array of hexahedron
    faces (element, axis, side), on tetrahedra an (n, 2) array of faces
    (element, local face), or a list of such groups -- with
    ``robin_coefficient`` h and ``robin_bc_value`` T_env (scalars, or one per
    group for the surface terms).  ``objective``: "compliance",
    "heat_exchange" or "averaged_temp"."""
    k: float = 1.0
    dirichlet_values: float | list = 0.0
    emit: np.ndarray | None = None
    objective: str = "compliance"
    robin_faces: np.ndarray | list | None = None
    robin_coefficient: float | list | None = None
    robin_bc_value: float | list | None = None
    design_robin_boundary: bool | None = None
    robin_elements: np.ndarray | None = None
    avg_temp_weight: float = 0.0

    @property
    def material_coef(self) -> float:
        return self.k

    @property
    def dirichlet_value_list(self) -> list:
        v = self.dirichlet_values
        return [float(x) for x in v] if isinstance(v, (list, tuple)) else [float(v)]

    @property
    def n_tasks(self) -> int:
        return len(self.dirichlet_value_list)

    @property
    def robin_groups(self) -> list:
        if self.robin_faces is None:
            return []
        g = self.robin_faces if isinstance(self.robin_faces, list) else [self.robin_faces]
        w = 3 if self.mesh.kind == "hex" else 2
        return [np.asarray(x, dtype=np.int64).reshape(-1, w) for x in g]

    @classmethod
    def from_nodes(cls, mesh, dirichlet_nodes, emit, design_elements, k=1.0,
                   dirichlet_values=0.0, robin_faces=None, robin_coefficient=None,
                   robin_bc_value=None, design_robin_boundary=None,
                   objective="compliance", avg_temp_weight=0.0):
        """task_heat.py:172-250 and task_common.py:105-270: elements touching
        Robin facets leave the design set when design_robin_boundary is False."""
        if objective not in ("compliance", "heat_exchange", "averaged_temp"):
            raise ValueError("objective must be one of 'compliance', 'heat_exchange', "
                             "or 'averaged_temp'")
        s = FEMDomain._sets(mesh, 1, dirichlet_nodes, "all", None, design_elements)
        rob_el = None
        if robin_faces is not None:
            groups = robin_faces if isinstance(robin_faces, list) else [robin_faces]
            w = 3 if mesh.kind == "hex" else 2
            allf = np.concatenate([np.asarray(g, dtype=np.int64).reshape(-1, w)
                                   for g in groups])
            rob_el = np.unique(allf[:, 0])
            if design_robin_boundary is False:
                s["design_elements"] = setdiff1d(s["design_elements"], rob_el)
                s["fixed_elements"] = setdiff1d(s["all_elements"], s["design_elements"])
        if emit is None:
            emit = np.zeros(mesh.nnodes)
        return cls(mesh=mesh, neumann_nodes=None, bs=1, k=float(k),
                   dirichlet_values=dirichlet_values,
                   emit=np.ascontiguousarray(emit, dtype=np.float64), objective=objective,
                   robin_faces=robin_faces, robin_coefficient=robin_coefficient,
                   robin_bc_value=robin_bc_value, design_robin_boundary=design_robin_boundary,
                   robin_elements=rob_el, avg_temp_weight=float(avg_temp_weight), **s)

    @classmethod
    def from_facets(cls, mesh, dirichlet_facets, dirichlet_values, robin_facets,
                    robin_coefficient, robin_bc_value, design_robin_boundary, design_elements,
                    k, objective="compliance", avg_temp_weight=0.0, emit=None):
        """task_heat.py:172-250 with facets as rows (element, local face)."""
        from .grid import facet_nodes_of, facets_to_faces
        groups = _group_list(dirichlet_facets)
        dn = np.unique(np.concatenate([facet_nodes_of(mesh, f).ravel() for f in groups]))
        rob = None
        if robin_facets is not None:
            rob = [facets_to_faces(f) if mesh.kind == "hex" else
                   np.asarray(f, dtype=np.int64).reshape(-1, 2)
                   for f in _group_list(robin_facets)]
        return cls.from_nodes(mesh, dn, emit, design_elements, k=k,
                              dirichlet_values=dirichlet_values, robin_faces=rob,
                              robin_coefficient=robin_coefficient,
                              robin_bc_value=robin_bc_value,
                              design_robin_boundary=design_robin_boundary,
                              objective=objective, avg_temp_weight=avg_temp_weight)

    @classmethod
    def from_mesh_tags(cls, mesh, dirichlet_values, robin_coefficient, robin_bc_value,
                       design_robin_boundary, k, objective="compliance", avg_temp_weight=0.0):
        """task_heat.py:252-321: ``dirichlet_<k>`` / ``dirichlet`` and
        ``robin_<k>`` / ``robin`` facet groups, the ``design`` subdomain."""
        dir_f = _tag_groups(mesh.boundaries, "dirichlet")
        rob_f = _tag_groups(mesh.boundaries, "robin")
        return cls.from_facets(mesh, dir_f, dirichlet_values, rob_f, robin_coefficient,
                               robin_bc_value, design_robin_boundary,
                               mesh.subdomains["design"], k, objective=objective,
                               avg_temp_weight=avg_temp_weight)

    @classmethod
    def from_boundaries(cls, mesh, dirichlet, dirichlet_values, robin, robin_coefficient,
                        robin_bc_value, design_robin_boundary, k,
                        objective="compliance", avg_temp_weight=0.0, design_elements=None,
                        emit=None):
        """task_heat.py:252-321 with boundary predicates in place of mesh tags:
        ``dirichlet`` / ``robin`` are point predicates (get_points_in_range)
        or lists of them, applied to boundary-facet midpoints."""
        dl = dirichlet if isinstance(dirichlet, list) else [dirichlet]
        if mesh.kind == "hex":
            faces_of, nodes_of = boundary_faces, face_nodes
        else:   # tetrahedra: facets as rows (element, local face)
            from .grid import boundary_facets, facet_nodes_of
            faces_of, nodes_of = boundary_facets, facet_nodes_of
        dn = np.unique(np.concatenate([np.ravel(nodes_of(mesh, faces_of(mesh, f)))
                                       for f in dl]))
        rob = None
        if robin is not None:
            rl = robin if isinstance(robin, list) else [robin]
            rob = [faces_of(mesh, f) for f in rl]
        if design_elements is None:
            design_elements = np.arange(mesh.nelements)
        return cls.from_nodes(mesh, dn, emit, design_elements, k=k,
                              dirichlet_values=dirichlet_values, robin_faces=rob,
                              robin_coefficient=robin_coefficient,
                              robin_bc_value=robin_bc_value,
                              design_robin_boundary=design_robin_boundary,
                              objective=objective, avg_temp_weight=avg_temp_weight)
