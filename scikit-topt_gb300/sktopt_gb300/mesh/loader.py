"""Mesh files: gmsh MSH 2.2 and 4.1 (ASCII) with physical groups.

The reference reads meshes with meshio and scikit-fem
(``basis_from_file`` sktopt/mesh/loader.py:9-33, ``MeshHex.load`` /
``MeshTet.load``): hexahedral or tetrahedral volume cells, and the physical
groups as named boundaries (facet sets) and subdomains (element sets) that
``from_mesh_tags`` consumes (task_elastic.py:266-317, task_heat.py:252-321).
Neither library is a dependency here, so this module parses the two gmsh
ASCII formats itself:

* nodes in file order (node tags compacted to 0..n-1);
* volume cells (gmsh type 5, 8-node hexahedron; type 4, 4-node tetrahedron)
  in file order, re-ordered to the MeshHex local order (offsets (0,0,0)
  (0,1,0) (1,0,0) (0,0,1) (1,1,0) (0,1,1) (1,0,1) (1,1,1)) and oriented to a
  positive volume as ``fix_hexahedron_orientation`` / ``fix_tetrahedron_
  orientation`` (utils.py:18-91) do;
* boundary cells (type 3 quadrangle, type 2 triangle) of a named physical
  group become ``mesh.boundaries[name]``: the matching element facets, rows
  (element, local face); volume cells of a named group become
  ``mesh.subdomains[name]``.

The mesh carries no logical grid, so its linear systems are solved with
block-Jacobi preconditioning (the multigrid needs a grid).
"""
from __future__ import annotations

import pathlib

import numpy as np

from .grid import GridMesh, _orient_hex, _orient_tet, element_faces

# gmsh hexahedron order (bottom face counter-clockwise, then top) -> MeshHex
_GMSH_HEX_TO_LOCAL = [0, 3, 1, 4, 2, 7, 5, 6]
_NODES_PER_TYPE = {2: 3, 3: 4, 4: 4, 5: 8}
_VOLUME_TYPES = {4: "tet", 5: "hex"}


def _sections(text: str) -> dict:
    out = {}
    lines = text.splitlines()
    i = 0
    while i < len(lines):
        ln = lines[i].strip()
        if ln.startswith("$") and not ln.startswith("$End"):
            name = ln[1:]
            j = i + 1
            while j < len(lines) and lines[j].strip() != f"$End{name}":
                j += 1
            out[name] = lines[i + 1:j]
            i = j + 1
        else:
            i += 1
    return out


def _physical_names(sec) -> dict:
    names = {}
    if sec is None:
        return names
    for ln in sec[1:1 + int(sec[0])]:
        parts = ln.split(maxsplit=2)
        names[(int(parts[0]), int(parts[1]))] = parts[2].strip().strip('"')
    return names


def _read_v2(sec):
    nodes = sec["Nodes"]
    n = int(nodes[0])
    tags = np.empty(n, dtype=np.int64)
    xyz = np.empty((n, 3))
    for k, ln in enumerate(nodes[1:1 + n]):
        v = ln.split()
        tags[k] = int(v[0])
        xyz[k] = [float(v[1]), float(v[2]), float(v[3])]
    cells = []            # (type, physical tag, node tags)
    els = sec["Elements"]
    for ln in els[1:1 + int(els[0])]:
        v = [int(x) for x in ln.split()]
        typ, ntag = v[1], v[2]
        if typ not in _NODES_PER_TYPE:
            continue
        phys = v[3] if ntag > 0 else 0
        cells.append((typ, phys, v[3 + ntag:3 + ntag + _NODES_PER_TYPE[typ]]))
    return tags, xyz, cells


def _read_v4(sec):
    ent = sec.get("Entities")
    phys_of = {}
    if ent is not None:
        counts = [int(x) for x in ent[0].split()]
        row = 1
        for dim, cnt in enumerate(counts):
            for _ in range(cnt):
                v = ent[row].split()
                row += 1
                tag = int(v[0])
                k = 4 if dim == 0 else 7
                nph = int(v[k])
                phys_of[(dim, tag)] = [int(x) for x in v[k + 1:k + 1 + nph]]
    nodes = sec["Nodes"]
    nblocks, n = (int(x) for x in nodes[0].split()[:2])
    tags = np.empty(n, dtype=np.int64)
    xyz = np.empty((n, 3))
    row, k = 1, 0
    for _ in range(nblocks):
        _, _, param, cnt = (int(x) for x in nodes[row].split())
        row += 1
        if param:
            raise ValueError("parametric node blocks are not supported")
        for i in range(cnt):
            tags[k + i] = int(nodes[row + i])
        for i in range(cnt):
            xyz[k + i] = [float(x) for x in nodes[row + cnt + i].split()[:3]]
        row += 2 * cnt
        k += cnt
    cells = []
    els = sec["Elements"]
    nblocks = int(els[0].split()[0])
    row = 1
    for _ in range(nblocks):
        dim, etag, typ, cnt = (int(x) for x in els[row].split())
        row += 1
        phys = phys_of.get((dim, etag), [0])
        for i in range(cnt):
            if typ in _NODES_PER_TYPE:
                v = [int(x) for x in els[row + i].split()]
                for ph in (phys or [0]):
                    cells.append((typ, ph, v[1:1 + _NODES_PER_TYPE[typ]]))
        row += cnt
    return tags, xyz, cells


def _match_faces(t, faces, query):
    """(element, local face) of every query face (rows of node indices), the
    first element in (face, element) order holding it; (-1, -1) if none."""
    ne = t.shape[1]
    keys = np.concatenate([np.sort(t[loc].T, axis=1) for loc in faces])
    owner = np.concatenate([np.stack([np.arange(ne), np.full(ne, f)], 1)
                            for f in range(len(faces))])
    q = np.sort(query, axis=1)
    k = keys.shape[1]
    dt = np.dtype((np.void, 8 * k))
    kv = np.ascontiguousarray(keys).view(dt).ravel()
    qv = np.ascontiguousarray(q).view(dt).ravel()
    order = np.argsort(kv, kind="stable")
    pos = np.searchsorted(kv[order], qv)
    pos = np.minimum(pos, kv.size - 1)
    hit = kv[order][pos] == qv
    out = np.full((q.shape[0], 2), -1, dtype=np.int64)
    out[hit] = owner[order[pos[hit]]]
    return out


def read_msh(path) -> GridMesh:
    """Read a gmsh MSH 2.2 or 4.1 ASCII file (see the module docstring)."""
    text = pathlib.Path(path).read_text()
    sec = _sections(text)
    if "MeshFormat" not in sec:
        raise ValueError(f"{path}: not a gmsh mesh file")
    version, ftype = sec["MeshFormat"][0].split()[:2]
    if int(ftype) != 0:
        raise ValueError(f"{path}: binary gmsh files are not supported")
    names = _physical_names(sec.get("PhysicalNames"))
    if version.startswith("2"):
        tags, xyz, cells = _read_v2(sec)
    elif version.startswith("4"):
        tags, xyz, cells = _read_v4(sec)
    else:
        raise ValueError(f"{path}: unsupported MSH version {version}")
    index = {int(t): i for i, t in enumerate(tags)}
    vol = [(typ, ph, nd) for typ, ph, nd in cells if typ in _VOLUME_TYPES]
    kinds = {_VOLUME_TYPES[typ] for typ, _, _ in vol}
    if len(kinds) != 1:
        raise ValueError(f"{path}: need hexahedra or tetrahedra only, got {kinds}")
    kind = kinds.pop()
    # one volume cell per node tuple (a cell in several groups appears once
    # per group in MSH 4); first occurrence order
    seen, conn, groups = {}, [], {}
    for typ, ph, nd in vol:
        key = tuple(nd)
        if key not in seen:
            seen[key] = len(conn)
            conn.append([index[x] for x in nd])
        if ph:
            groups.setdefault(ph, []).append(seen[key])
    t = np.asarray(conn, dtype=np.int64).T
    if kind == "hex":
        t = t[_GMSH_HEX_TO_LOCAL]
    p = xyz.T.copy()
    t = _orient_hex(t, p) if kind == "hex" else _orient_tet(t, p)
    subdomains = {names.get((3, ph), str(ph)): np.unique(np.asarray(el, dtype=np.int64))
                  for ph, el in groups.items()}
    # boundary groups: match facet cells to element faces
    ftype = 3 if kind == "hex" else 2
    bcells = [(ph, [index[x] for x in nd]) for typ, ph, nd in cells if typ == ftype and ph]
    boundaries = {}
    if bcells:
        found = _match_faces(t, element_faces(kind),
                             np.asarray([nd for _, nd in bcells], dtype=np.int64))
        if np.any(found[:, 0] < 0):
            bad = bcells[int(np.nonzero(found[:, 0] < 0)[0][0])][1]
            raise ValueError(f"{path}: boundary cell {bad} is not a face of a volume cell")
        for (ph, _), row in zip(bcells, found):
            boundaries.setdefault(names.get((2, ph), str(ph)), []).append(row)
        boundaries = {k: np.unique(np.asarray(v, dtype=np.int64), axis=0)
                      for k, v in boundaries.items()}
    return GridMesh(p, t, kind, boundaries=boundaries, subdomains=subdomains)


def write_msh(path, mesh: GridMesh, boundaries=None, subdomains=None):
    """Write ``mesh`` as gmsh MSH 2.2 ASCII with named physical groups:
    ``boundaries`` name -> facets (element, local face), ``subdomains``
    name -> elements (default: the mesh's own tags)."""
    boundaries = mesh.boundaries if boundaries is None else boundaries
    subdomains = mesh.subdomains if subdomains is None else subdomains
    faces = element_faces(mesh.kind)
    vtype, ftype = (5, 3) if mesh.kind == "hex" else (4, 2)
    inv = np.argsort(_GMSH_HEX_TO_LOCAL) if mesh.kind == "hex" else np.arange(4)
    lines = ["$MeshFormat", "2.2 0 8", "$EndMeshFormat", "$PhysicalNames"]
    groups = [(2, name) for name in boundaries] + [(3, name) for name in subdomains]
    lines.append(str(len(groups)))
    tag_of = {}
    for k, (dim, name) in enumerate(groups, start=1):
        tag_of[(dim, name)] = k
        lines.append(f'{dim} {k} "{name}"')
    lines += ["$EndPhysicalNames", "$Nodes", str(mesh.nnodes)]
    lines += [f"{i + 1} {float(x)!r} {float(y)!r} {float(z)!r}"
              for i, (x, y, z) in enumerate(mesh.p.T)]
    lines += ["$EndNodes", "$Elements"]
    rows = []
    for name, fac in boundaries.items():
        for e, f in np.asarray(fac, dtype=np.int64).reshape(-1, 2):
            nd = mesh.t[faces[f], e] + 1
            rows.append((ftype, tag_of[(2, name)], nd))
    in_group = {}
    for name, el in subdomains.items():
        for e in np.asarray(el, dtype=np.int64):
            in_group.setdefault(int(e), []).append(tag_of[(3, name)])
    for e in range(mesh.nelements):
        nd = mesh.t[:, e][inv] + 1
        for ph in in_group.get(e, [0]):
            rows.append((vtype, ph, nd))
    lines.append(str(len(rows)))
    for k, (typ, ph, nd) in enumerate(rows, start=1):
        lines.append(f"{k} {typ} 2 {ph} {ph} " + " ".join(str(int(x)) for x in nd))
    lines.append("$EndElements")
    pathlib.Path(path).write_text("\n".join(lines) + "\n")


def basis_from_file(mesh_path):
    """loader.py:9-33: the mesh of a gmsh file (hexahedra or tetrahedra)."""
    return read_msh(mesh_path)
