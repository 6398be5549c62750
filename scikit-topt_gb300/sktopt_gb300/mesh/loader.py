"""Mesh files: gmsh MSH 2.2 and 4.1, ASCII and binary, with physical groups.

The reference reads meshes with meshio and scikit-fem
(``basis_from_file`` sktopt/mesh/loader.py:9-33, ``MeshHex.load`` /
``MeshTet.load``; its tutorial lists gmsh v2 and v4, ASCII and binary):
hexahedral or tetrahedral volume cells, and the physical groups as named
boundaries (facet sets) and subdomains (element sets) that
``from_mesh_tags`` consumes (task_elastic.py:266-317, task_heat.py:252-321).
Neither library is a dependency here, so this module parses the gmsh
formats itself:

* nodes in file order (node tags compacted to 0..n-1);
* volume cells (gmsh type 5, 8-node hexahedron; type 4, 4-node tetrahedron)
  in file order, re-ordered to the MeshHex local order (offsets (0,0,0)
  (0,1,0) (1,0,0) (0,0,1) (1,1,0) (0,1,1) (1,0,1) (1,1,1)) and oriented to a
  positive volume as ``fix_hexahedron_orientation`` / ``fix_tetrahedron_
  orientation`` (utils.py:18-91) do;
* boundary cells (type 3 quadrangle, type 2 triangle) of a named physical
  group become ``mesh.boundaries[name]``: the matching element facets, rows
  (element, local face); volume cells of a named group become
  ``mesh.subdomains[name]``;
* binary files (file type 1, data size 8): the section headers and
  ``$PhysicalNames`` are text, the rest little- or big-endian as the
  ``$MeshFormat`` integer 1 says.  MSH 2.2: nodes as (int tag, 3 doubles),
  elements in blocks headed by (type, count, number of tags), each element
  (int tag, int tags, int nodes).  MSH 4.1: counts and node / element tags
  as 8-byte unsigned integers, entity dimensions, tags and types as 4-byte
  integers, coordinates and bounding boxes as doubles.  Other sections are
  skipped.

The mesh carries no logical grid: its linear systems are solved with the
smoothed-aggregation multigrid built on the GPU (block Jacobi on request).
"""
from __future__ import annotations

import pathlib

import numpy as np

from .grid import GridMesh, _orient_hex, _orient_tet, element_faces

# gmsh hexahedron order (bottom face counter-clockwise, then top) -> MeshHex
_GMSH_HEX_TO_LOCAL = [0, 3, 1, 4, 2, 7, 5, 6]
_NODES_PER_TYPE = {2: 3, 3: 4, 4: 4, 5: 8}
_VOLUME_TYPES = {4: "tet", 5: "hex"}
# nodes of every gmsh element type a binary file may hold (to step over the
# types this module does not use): lines, triangles, quadrangles,
# tetrahedra, hexahedra, prisms, pyramids of order 1-2, points
_GMSH_TYPE_NODES = {1: 2, 2: 3, 3: 4, 4: 4, 5: 8, 6: 6, 7: 5, 8: 3, 9: 6, 10: 9, 11: 10,
                    12: 27, 13: 18, 14: 14, 15: 1, 16: 8, 17: 20, 18: 15, 19: 13}


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


class _Bytes:
    """Cursor over the bytes of a binary gmsh file."""

    def __init__(self, data: bytes):
        self.d = data
        self.i = 0
        self.order = "<"

    def skip_space(self):
        while self.i < len(self.d) and self.d[self.i] in b" \t\r\n":
            self.i += 1

    def line(self) -> str:
        j = self.d.find(b"\n", self.i)
        j = len(self.d) if j < 0 else j
        out = self.d[self.i:j].decode("ascii", errors="replace").strip()
        self.i = j + 1
        return out

    def arr(self, dtype, n):
        dt = np.dtype(dtype).newbyteorder(self.order)
        if self.i + dt.itemsize * int(n) > len(self.d):
            raise ValueError("truncated binary gmsh section")
        a = np.frombuffer(self.d, dtype=dt, count=int(n), offset=self.i)
        self.i += a.nbytes
        return a.astype(dt.newbyteorder("="))

    def size(self) -> int:
        return int(self.arr("u8", 1)[0])

    def end(self, name):
        self.skip_space()
        got = self.line()
        if got != f"$End{name}":
            raise ValueError(f"binary gmsh: expected $End{name}, found {got[:40]!r}")


def _type_nodes(typ: int) -> int:
    if typ not in _GMSH_TYPE_NODES:
        raise ValueError(f"binary gmsh: element type {typ} is not supported")
    return _GMSH_TYPE_NODES[typ]


def _read_binary(data: bytes, version: str):
    """Physical names, node tags, coordinates and cells of a binary file."""
    b = _Bytes(data)
    v4 = version.startswith("4")
    names, phys_of = {}, {}
    tags = xyz = None
    cells = []
    while True:
        b.skip_space()
        if b.i >= len(b.d):
            break
        hdr = b.line()
        if not hdr.startswith("$"):
            raise ValueError(f"binary gmsh: expected a section, found {hdr[:40]!r}")
        name = hdr[1:]
        if name == "MeshFormat":
            fmt = b.line().split()
            if len(fmt) < 3 or fmt[2] != "8":
                raise ValueError("binary gmsh: only data size 8 is supported")
            one = b.d[b.i:b.i + 4]
            b.i += 4
            if one == (1).to_bytes(4, "little"):
                b.order = "<"
            elif one == (1).to_bytes(4, "big"):
                b.order = ">"
            else:
                raise ValueError("binary gmsh: bad endianness mark")
        elif name == "PhysicalNames":
            n = int(b.line())
            names = _physical_names([str(n)] + [b.line() for _ in range(n)])
        elif name == "Entities" and v4:
            counts = b.arr("u8", 4)
            for dim, cnt in enumerate(counts):
                for _ in range(int(cnt)):
                    etag = int(b.arr("i4", 1)[0])
                    b.arr("f8", 3 if dim == 0 else 6)
                    phys_of[(dim, etag)] = [int(x) for x in b.arr("i4", b.size())]
                    if dim > 0:
                        b.arr("i4", b.size())
        elif name == "Nodes":
            if v4:
                nblocks, n = (int(x) for x in b.arr("u8", 4)[:2])
                tags = np.empty(n, dtype=np.int64)
                xyz = np.empty((n, 3))
                k = 0
                for _ in range(nblocks):
                    _, _, param = (int(x) for x in b.arr("i4", 3))
                    cnt = b.size()
                    if param:
                        raise ValueError("parametric node blocks are not supported")
                    tags[k:k + cnt] = b.arr("u8", cnt)
                    xyz[k:k + cnt] = b.arr("f8", 3 * cnt).reshape(cnt, 3)
                    k += cnt
            else:
                n = int(b.line())
                rec = b.arr(np.dtype([("tag", "i4"), ("xyz", "f8", (3,))]), n)
                tags = rec["tag"].astype(np.int64)
                xyz = np.array(rec["xyz"], dtype=np.float64)
        elif name == "Elements":
            if v4:
                nblocks = int(b.arr("u8", 4)[0])
                for _ in range(nblocks):
                    dim, etag, typ = (int(x) for x in b.arr("i4", 3))
                    cnt = b.size()
                    nn = _type_nodes(typ)
                    rows = b.arr("u8", cnt * (1 + nn)).reshape(cnt, 1 + nn)
                    if typ in _NODES_PER_TYPE:
                        phys = phys_of.get((dim, etag), [0]) or [0]
                        for r in rows:
                            nd = [int(x) for x in r[1:]]
                            for ph in phys:
                                cells.append((typ, ph, nd))
            else:
                total = int(b.line())
                got = 0
                while got < total:
                    typ, follow, ntag = (int(x) for x in b.arr("i4", 3))
                    nn = _type_nodes(typ)
                    rows = b.arr("i4", follow * (1 + ntag + nn)).reshape(follow, -1)
                    if typ in _NODES_PER_TYPE:
                        for r in rows:
                            cells.append((typ, int(r[1]) if ntag > 0 else 0,
                                          [int(x) for x in r[1 + ntag:]]))
                    got += follow
        else:
            j = b.d.find(f"$End{name}".encode(), b.i)
            if j < 0:
                raise ValueError(f"binary gmsh: section ${name} is not closed")
            b.i = j
        b.end(name)
    if tags is None:
        raise ValueError("binary gmsh: no $Nodes section")
    return names, tags, xyz, cells


def read_msh(path) -> GridMesh:
    """Read a gmsh MSH 2.2 or 4.1 file, ASCII or binary (see the module
    docstring)."""
    data = pathlib.Path(path).read_bytes()
    start = data.find(b"$MeshFormat")
    if start < 0:
        raise ValueError(f"{path}: not a gmsh mesh file")
    fmt_line = data[start:].split(b"\n", 2)[1].decode("ascii", errors="replace").split()
    if len(fmt_line) < 2:
        raise ValueError(f"{path}: not a gmsh mesh file")
    version, ftype = fmt_line[0], int(fmt_line[1])
    if not (version.startswith("2") or version.startswith("4")):
        raise ValueError(f"{path}: unsupported MSH version {version}")
    if ftype == 1:
        names, tags, xyz, cells = _read_binary(data, version)
    else:
        sec = _sections(data.decode("utf-8", errors="replace"))
        names = _physical_names(sec.get("PhysicalNames"))
        tags, xyz, cells = _read_v2(sec) if version.startswith("2") else _read_v4(sec)
    return _assemble(path, names, tags, xyz, cells)


def _assemble(path, names, tags, xyz, cells) -> GridMesh:
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


def write_msh(path, mesh: GridMesh, boundaries=None, subdomains=None, version="2.2",
              binary=False, byteorder="<"):
    """Write ``mesh`` as gmsh MSH ``version`` "2.2" or "4.1", ASCII or
    ``binary`` (``byteorder`` "<" or ">"), with named physical groups:
    ``boundaries`` name -> facets (element, local face), ``subdomains``
    name -> elements (default: the mesh's own tags).  MSH 4.1 puts every
    boundary group in a surface entity and the volume cells in one volume
    entity per distinct set of groups (element blocks follow the element
    order, one block per run of elements of the same entity)."""
    if version not in ("2.2", "4.1"):
        raise ValueError("version must be '2.2' or '4.1'")
    boundaries = mesh.boundaries if boundaries is None else boundaries
    subdomains = mesh.subdomains if subdomains is None else subdomains
    faces = element_faces(mesh.kind)
    vtype, ftype = (5, 3) if mesh.kind == "hex" else (4, 2)
    inv = np.argsort(_GMSH_HEX_TO_LOCAL) if mesh.kind == "hex" else np.arange(4)
    groups = [(2, name) for name in boundaries] + [(3, name) for name in subdomains]
    tag_of = {g: k for k, g in enumerate(groups, start=1)}
    out = _MshOut(binary, byteorder)
    out.text(f"$MeshFormat\n{version} {1 if binary else 0} 8\n")
    if binary:
        out.ints([1])
        out.text("\n")
    out.text("$EndMeshFormat\n$PhysicalNames\n" + f"{len(groups)}\n")
    for (dim, name), k in tag_of.items():
        out.text(f'{dim} {k} "{name}"\n')
    out.text("$EndPhysicalNames\n")
    # surface cells per boundary group; volume cells with their group tags
    surf = [(tag_of[(2, name)], [mesh.t[faces[f], e] + 1 for e, f in
                                 np.asarray(fac, dtype=np.int64).reshape(-1, 2)])
            for name, fac in boundaries.items()]
    in_group = {}
    for name, el in subdomains.items():
        for e in np.asarray(el, dtype=np.int64):
            in_group.setdefault(int(e), []).append(tag_of[(3, name)])
    vol_nodes = [mesh.t[:, e][inv] + 1 for e in range(mesh.nelements)]
    if version == "2.2":
        rows = [(ftype, ph, nd) for ph, cells in surf for nd in cells]
        for e in range(mesh.nelements):
            for ph in in_group.get(e, [0]):
                rows.append((vtype, ph, vol_nodes[e]))
        out.text(f"$Nodes\n{mesh.nnodes}\n")
        if binary:
            rec = np.empty(mesh.nnodes, dtype=np.dtype([("tag", "i4"), ("xyz", "f8", (3,))])
                           .newbyteorder(byteorder))
            rec["tag"] = np.arange(1, mesh.nnodes + 1)
            rec["xyz"] = mesh.p.T
            out.raw(rec.tobytes())
            out.text("\n")
        else:
            out.text("".join(f"{i + 1} {float(x)!r} {float(y)!r} {float(z)!r}\n"
                             for i, (x, y, z) in enumerate(mesh.p.T)))
        out.text(f"$EndNodes\n$Elements\n{len(rows)}\n")
        if binary:
            k = 0
            while k < len(rows):
                typ = rows[k][0]
                j2 = k
                while j2 < len(rows) and rows[j2][0] == typ:
                    j2 += 1
                out.ints([typ, j2 - k, 2])
                for n, (_, ph, nd) in enumerate(rows[k:j2], start=k + 1):
                    out.ints([n, ph, ph] + [int(x) for x in nd])
                k = j2
            out.text("\n")
        else:
            out.text("".join(f"{k} {typ} 2 {ph} {ph} " + " ".join(str(int(x)) for x in nd) + "\n"
                             for k, (typ, ph, nd) in enumerate(rows, start=1)))
        out.text("$EndElements\n")
    else:
        vsets = {}
        for e in range(mesh.nelements):
            vsets.setdefault(tuple(in_group.get(e, [])), []).append(e)
        lo, hi = mesh.p.min(axis=1), mesh.p.max(axis=1)
        box = [float(v) for v in np.concatenate([lo, hi])]
        out.text("$Entities\n")
        if binary:
            out.sizes([0, 0, len(surf), len(vsets)])
        else:
            out.text(f"0 0 {len(surf)} {len(vsets)}\n")
        ents = [(2, k + 1, [ph]) for k, (ph, _) in enumerate(surf)] + \
            [(3, k + 1, list(key)) for k, key in enumerate(vsets)]
        for _, etag, phys in ents:
            if binary:
                out.ints([etag])
                out.doubles(box)
                out.sizes([len(phys)])
                out.ints(phys)
                out.sizes([0])
            else:
                out.text(f"{etag} " + " ".join(repr(v) for v in box) + f" {len(phys)} " +
                         "".join(f"{ph} " for ph in phys) + "0\n")
        if binary:
            out.text("\n")
        out.text("$EndEntities\n$Nodes\n")
        n = mesh.nnodes
        if binary:
            out.sizes([1, n, 1, n])
            out.ints([3, 1, 0])
            out.sizes([n])
            out.sizes(list(range(1, n + 1)))
            out.doubles(mesh.p.T.ravel())
            out.text("\n")
        else:
            out.text(f"1 {n} 1 {n}\n3 1 0 {n}\n")
            out.text("".join(f"{i}\n" for i in range(1, n + 1)))
            out.text("".join(f"{float(x)!r} {float(y)!r} {float(z)!r}\n" for x, y, z in mesh.p.T))
        # volume cells in element order: one block per run of consecutive
        # elements of the same entity, so that a reader keeps the order
        etag_of = {key: k + 1 for k, key in enumerate(vsets)}
        blocks = [(2, k + 1, ftype, cells) for k, (_, cells) in enumerate(surf)]
        for e in range(mesh.nelements):
            et = etag_of[tuple(in_group.get(e, []))]
            if blocks and blocks[-1][0] == 3 and blocks[-1][1] == et:
                blocks[-1][3].append(vol_nodes[e])
            else:
                blocks.append((3, et, vtype, [vol_nodes[e]]))
        total = sum(len(c) for *_, c in blocks)
        out.text("$EndNodes\n$Elements\n")
        if binary:
            out.sizes([len(blocks), total, 1, total])
        else:
            out.text(f"{len(blocks)} {total} 1 {total}\n")
        tag = 1
        for dim, etag, typ, cells in blocks:
            if binary:
                out.ints([dim, etag, typ])
                out.sizes([len(cells)])
            else:
                out.text(f"{dim} {etag} {typ} {len(cells)}\n")
            for nd in cells:
                if binary:
                    out.sizes([tag] + [int(x) for x in nd])
                else:
                    out.text(f"{tag} " + " ".join(str(int(x)) for x in nd) + "\n")
                tag += 1
        if binary:
            out.text("\n")
        out.text("$EndElements\n")
    pathlib.Path(path).write_bytes(out.bytes())


class _MshOut:
    """Byte buffer of a gmsh file: text, and binary values in one byte order."""

    def __init__(self, binary, byteorder):
        self.parts = []
        self.binary = binary
        self.order = byteorder

    def text(self, s):
        self.parts.append(s.encode("ascii"))

    def raw(self, b):
        self.parts.append(b)

    def _vals(self, vals, dt):
        self.parts.append(np.asarray(vals, dtype=np.dtype(dt).newbyteorder(self.order))
                          .tobytes())

    def ints(self, vals):
        self._vals(vals, "i4")

    def sizes(self, vals):
        self._vals(vals, "u8")

    def doubles(self, vals):
        self._vals(vals, "f8")

    def bytes(self):
        return b"".join(self.parts)


def basis_from_file(mesh_path):
    """loader.py:9-33: the mesh of a gmsh file (hexahedra or tetrahedra)."""
    return read_msh(mesh_path)
