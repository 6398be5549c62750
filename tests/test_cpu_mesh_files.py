"""Mesh files, boundary facets and surface tractions (CPU).

* gmsh MSH 2.2 and 4.1 round trips, ASCII and binary (little- and
  big-endian), hexahedra and jittered tetrahedra: nodes, connectivity,
  named boundaries and subdomains come back unchanged;
* a hand-written MSH 4.1 file (two hexahedra, entity-level physical groups)
  parses to the MeshHex local order with the expected facets, and so do its
  binary MSH 4.1 and MSH 2.2 forms packed field by field with ``struct``;
* boundary facets and traction loads (task_elastic.py:15-81) against the
  oracle restatement (other quadrature rules): 1e-13 relative;
* ``from_mesh_tags`` (task_elastic.py:266-317, task_heat.py:252-321) builds
  the same Dirichlet sets, design sets and loads as the node-based set-up.
"""
import numpy as np
import pytest

from oracle import mesh as omesh
from oracle import surface as osurf


def _meshes():
    from sktopt_gb300.mesh import create_box_hex, create_box_tet
    return [create_box_hex(5, 3, 2, 0.5, 1.0, 1.5),
            create_box_tet(5, 3, 3, 2.0, 1.0, 1.0, jitter=0.25, seed=4)]


def _omesh(m):
    return omesh.GridMesh(m.p, m.t, m.kind, None, None, None)


@pytest.mark.parametrize("k", [0, 1])
def test_boundary_facets_and_tractions_match_oracle(k):
    from sktopt_gb300.mesh import assemble_surface_forces, boundary_facets
    from sktopt_gb300.mesh import get_points_in_range as rng
    m = _meshes()[k]
    om = _omesh(m)
    assert np.array_equal(boundary_facets(m), osurf.boundary_facets(om))
    xmax, ymax = m.p[0].max(), m.p[1].max()
    g1 = rng((xmax, xmax), (0, ymax), (0, 9))
    g2 = rng((0, xmax), (ymax, ymax), (0, 9))
    f1, f2 = boundary_facets(m, g1), boundary_facets(m, g2)
    assert np.array_equal(f1, osurf.boundary_facets(om, g1)) and len(f1) > 0
    assert np.array_equal(f2, osurf.boundary_facets(om, g2)) and len(f2) > 0
    F = assemble_surface_forces(m, [f1, f2], ["u^3", "u^1"], [-2.0, 0.5])
    R = osurf.surface_forces(om, [f1, f2], ["u^3", "u^1"], [-2.0, 0.5])
    for a, b, tot, comp in zip(F, R, (-2.0, 0.5), (2, 0)):
        np.testing.assert_allclose(a, b, rtol=1e-13, atol=1e-15)
        s = a.reshape(-1, 3).sum(axis=0)
        assert abs(s[comp] - tot) <= 1e-13 and np.abs(np.delete(s, comp)).max() == 0.0


@pytest.mark.parametrize("k", [0, 1])
@pytest.mark.parametrize("version,binary,order", [("2.2", False, "<"), ("2.2", True, "<"),
                                                  ("2.2", True, ">"), ("4.1", False, "<"),
                                                  ("4.1", True, "<"), ("4.1", True, ">")])
def test_msh_round_trip(tmp_path, k, version, binary, order):
    from sktopt_gb300.mesh import boundary_facets, read_msh, write_msh
    from sktopt_gb300.mesh import get_points_in_range as rng
    m = _meshes()[k]
    b = {"dirichlet": boundary_facets(m, rng((0, 0), (0, 9), (0, 9))),
         "neumann_1": boundary_facets(m, rng((m.p[0].max(), 9), (0, 9), (0, 9)))}
    # overlapping subdomains: an element in two groups
    sub = {"design": np.arange(m.nelements)[::2], "solid": np.arange(m.nelements)[1::2],
           "probe": np.arange(m.nelements)[:3]}
    path = tmp_path / "m.msh"
    write_msh(path, m, boundaries=b, subdomains=sub, version=version, binary=binary,
              byteorder=order)
    assert (b"\x00" in path.read_bytes()) == binary
    r = read_msh(path)
    assert r.kind == m.kind and not r.has_grid
    assert np.array_equal(r.t, m.t) and np.array_equal(r.p, m.p)
    for name, fac in b.items():
        assert np.array_equal(r.boundaries[name], np.unique(fac, axis=0))
    for name, el in sub.items():
        assert np.array_equal(r.subdomains[name], el)


_MSH41 = """$MeshFormat
4.1 0 8
$EndMeshFormat
$PhysicalNames
3
2 1 "dirichlet"
2 2 "neumann"
3 3 "design"
$EndPhysicalNames
$Entities
0 0 2 1
1 0 0 0 0 1 1 1 1 0
2 2 0 0 2 1 1 1 2 0
1 0 0 0 2 1 1 1 3 0
$EndEntities
$Nodes
1 12 1 12
3 1 0 12
{tags}
{xyz}
$EndNodes
$Elements
3 4 1 4
2 1 3 1
1 {q0}
2 2 3 1
2 {q1}
3 1 5 2
3 {h0}
4 {h1}
$EndElements
"""


def _two_hex_data():
    nid = lambda x, y, z: 1 + x + 3 * y + 6 * z          # noqa: E731
    xyz = [(x, y, z) for z in range(2) for y in range(2) for x in range(3)]
    gm = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    hexes = [[nid(x + o[0], o[1], o[2]) for o in gm] for x in (0, 1)]
    quads = [[nid(x, y, z) for y, z in ((0, 0), (1, 0), (1, 1), (0, 1))] for x in (0, 2)]
    return nid, xyz, hexes, quads


def _check_two_hex(m):
    assert m.kind == "hex" and m.nelements == 2 and m.nnodes == 12
    for e in range(2):
        for a, o in enumerate(omesh.HEX_OFFSETS):
            assert np.array_equal(m.p[:, m.t[a, e]], [e + o[0], o[1], o[2]])
    assert np.array_equal(m.boundaries["dirichlet"], [[0, 0]])
    assert np.array_equal(m.boundaries["neumann"], [[1, 1]])
    assert np.array_equal(m.subdomains["design"], [0, 1])


_NAMES = b'''$PhysicalNames
3
2 1 "dirichlet"
2 2 "neumann"
3 3 "design"
$EndPhysicalNames
'''


@pytest.mark.parametrize("order", ["<", ">"])
def test_msh41_binary_packed_by_hand(tmp_path, order):
    """The two-hexahedra file in binary MSH 4.1, each field packed with
    struct as the format lays it out: size_t counts and tags, int entity
    dimensions / tags / types, double coordinates and bounding boxes."""
    import struct
    nid, xyz, hexes, quads = _two_hex_data()
    o = order
    ent = struct.pack(o + "4Q", 0, 0, 2, 1)
    for tag, ph in ((1, 1), (2, 2)):
        ent += struct.pack(o + "i6dQiQ", tag, 0, 0, 0, 2, 1, 1, 1, ph, 0)
    ent += struct.pack(o + "i6dQiQ", 1, 0, 0, 0, 2, 1, 1, 1, 3, 0)
    nodes = struct.pack(o + "4Q", 1, 12, 1, 12) + struct.pack(o + "3iQ", 3, 1, 0, 12)
    nodes += struct.pack(o + "12Q", *[nid(*c) for c in xyz])
    nodes += struct.pack(o + "36d", *[float(v) for c in xyz for v in c])
    els = struct.pack(o + "4Q", 3, 4, 1, 4)
    els += struct.pack(o + "3iQ", 2, 1, 3, 1) + struct.pack(o + "5Q", 1, *quads[0])
    els += struct.pack(o + "3iQ", 2, 2, 3, 1) + struct.pack(o + "5Q", 2, *quads[1])
    els += struct.pack(o + "3iQ", 3, 1, 5, 2) + struct.pack(o + "9Q", 3, *hexes[0])
    els += struct.pack(o + "9Q", 4, *hexes[1])
    data = (b"$MeshFormat\n4.1 1 8\n" + struct.pack(o + "i", 1) + b"\n$EndMeshFormat\n" +
            _NAMES + b"$Entities\n" + ent + b"\n$EndEntities\n$Nodes\n" + nodes +
            b"\n$EndNodes\n$Elements\n" + els + b"\n$EndElements\n")
    from sktopt_gb300.mesh import read_msh
    (tmp_path / "b41.msh").write_bytes(data)
    _check_two_hex(read_msh(tmp_path / "b41.msh"))
    # an unknown section and a point-element block (type 15) are stepped over
    pts = struct.pack(o + "3iQ", 0, 1, 15, 1) + struct.pack(o + "2Q", 9, 1)
    els2 = struct.pack(o + "4Q", 4, 5, 1, 9) + els[32:] + pts
    data2 = data.replace(els, els2).replace(
        b"$Entities", b"$Comments\nwritten by hand\n$EndComments\n$Entities")
    (tmp_path / "b41x.msh").write_bytes(data2)
    _check_two_hex(read_msh(tmp_path / "b41x.msh"))
    # an element type this reader does not know
    bad = data.replace(struct.pack(o + "3iQ", 3, 1, 5, 2), struct.pack(o + "3iQ", 3, 1, 99, 2))
    (tmp_path / "b41bad.msh").write_bytes(bad)
    with pytest.raises(ValueError, match="element type 99"):
        read_msh(tmp_path / "b41bad.msh")


@pytest.mark.parametrize("order", ["<", ">"])
def test_msh22_binary_packed_by_hand(tmp_path, order):
    """The same mesh in binary MSH 2.2: nodes as (int tag, 3 doubles), the
    elements in blocks headed by (type, count, number of tags), each element
    (int number, int tags, int nodes); a point element (type 15) to step
    over."""
    import struct
    nid, xyz, hexes, quads = _two_hex_data()
    o = order
    nodes = b"".join(struct.pack(o + "i3d", nid(*c), *[float(v) for v in c]) for c in xyz)
    els = struct.pack(o + "3i", 15, 1, 2) + struct.pack(o + "4i", 1, 0, 0, 1)
    els += struct.pack(o + "3i", 3, 2, 2)
    els += struct.pack(o + "7i", 2, 1, 1, *quads[0]) + struct.pack(o + "7i", 3, 2, 2, *quads[1])
    els += struct.pack(o + "3i", 5, 2, 2)
    els += struct.pack(o + "11i", 4, 3, 3, *hexes[0]) + struct.pack(o + "11i", 5, 3, 3, *hexes[1])
    data = (b"$MeshFormat\n2.2 1 8\n" + struct.pack(o + "i", 1) + b"\n$EndMeshFormat\n" +
            _NAMES + b"$Nodes\n12\n" + nodes + b"\n$EndNodes\n$Elements\n5\n" + els +
            b"\n$EndElements\n")
    from sktopt_gb300.mesh import read_msh
    (tmp_path / "b22.msh").write_bytes(data)
    _check_two_hex(read_msh(tmp_path / "b22.msh"))


def test_msh41_two_hexahedra(tmp_path):
    from sktopt_gb300.mesh import read_msh
    nid = lambda x, y, z: 1 + x + 3 * y + 6 * z          # noqa: E731
    xyz = [(x, y, z) for z in range(2) for y in range(2) for x in range(3)]
    gm = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    hexes = [" ".join(str(nid(x + o[0], o[1], o[2])) for o in gm) for x in (0, 1)]
    text = _MSH41.format(
        tags="\n".join(str(nid(*c)) for c in xyz),
        xyz="\n".join(f"{c[0]}.0 {c[1]}.0 {c[2]}.0" for c in xyz),
        q0=" ".join(str(nid(0, y, z)) for y, z in ((0, 0), (1, 0), (1, 1), (0, 1))),
        q1=" ".join(str(nid(2, y, z)) for y, z in ((0, 0), (1, 0), (1, 1), (0, 1))),
        h0=hexes[0], h1=hexes[1])
    path = tmp_path / "two.msh"
    path.write_text(text)
    m = read_msh(path)
    assert m.kind == "hex" and m.nelements == 2 and m.nnodes == 12
    # MeshHex local order: node a of element e sits at offset HEX_OFFSETS[a]
    for e in range(2):
        for a, o in enumerate(omesh.HEX_OFFSETS):
            assert np.array_equal(m.p[:, m.t[a, e]], [e + o[0], o[1], o[2]])
    assert np.array_equal(m.boundaries["dirichlet"], [[0, 0]])
    assert np.array_equal(m.boundaries["neumann"], [[1, 1]])
    assert np.array_equal(m.subdomains["design"], [0, 1])


def test_elastic_from_mesh_tags_matches_node_setup(tmp_path):
    from sktopt_gb300.mesh import (LinearElasticity, boundary_facets, create_box_tet,
                                   read_msh, write_msh)
    from sktopt_gb300.mesh import get_points_in_range as rng
    m = create_box_tet(6, 3, 3, 2.0, 1.0, 1.0, jitter=0.2, seed=2)
    left = boundary_facets(m, rng((0, 0), (0, 9), (0, 9)))
    right = boundary_facets(m, rng((2.0, 2.0), (0, 9), (0, 9)))
    top = boundary_facets(m, rng((0, 9), (0, 9), (1.0, 1.0)))
    write_msh(tmp_path / "c.msh", m, boundaries={"dirichlet": left, "neumann_1": right,
                                                 "neumann_2": top},
              subdomains={"design": np.arange(m.nelements)})
    r = read_msh(tmp_path / "c.msh")
    t = LinearElasticity.from_mesh_tags(r, "all", ["u^3", "u^2"], [-1.0, 0.25], 1.0, 0.3)
    assert t.n_tasks == 2
    dn = np.nonzero(np.isclose(m.p[0], 0.0))[0]
    assert np.array_equal(t.dirichlet_nodes, dn)
    assert np.array_equal(t.dirichlet_dofs, np.sort((3 * dn[:, None] + np.arange(3)).ravel()))
    om = _omesh(m)
    R = osurf.surface_forces(om, [right, top], ["u^3", "u^2"], [-1.0, 0.25])
    for a, b in zip(t.neumann_linear, R):
        np.testing.assert_allclose(a, b, rtol=1e-13, atol=1e-15)
    # elements touching a loaded node leave the design set (task_common.py:208-227)
    loaded_nodes = np.unique(np.nonzero(np.abs(R[0]) + np.abs(R[1]))[0] // 3)
    touching = np.nonzero(np.isin(m.t, loaded_nodes).any(axis=0))[0]
    assert touching.size > 0 and not np.isin(touching, t.design_elements).any()


def test_heat_from_mesh_tags_matches_plate(tmp_path):
    from sktopt_gb300.mesh import LinearHeatConduction, read_msh, write_msh
    from sktopt_gb300.mesh import boundary_facets, toy_problem
    from sktopt_gb300.mesh import get_points_in_range as rng
    ref = toy_problem.heat_plate(12, 12, 3)
    m = ref.mesh
    b = {"dirichlet_0": boundary_facets(m, rng((7.6, 8.0), (0.0, 0.4), (0.0, 1.0))),
         "robin_0": boundary_facets(m, rng((0.0, 0.0), (0.0, 8.0), (0.0, 1.0))),
         "robin_1": boundary_facets(m, rng((0.0, 8.0), (8.0, 8.0), (0.0, 1.0)))}
    write_msh(tmp_path / "h.msh", m, boundaries=b,
              subdomains={"design": np.arange(m.nelements)})
    r = read_msh(tmp_path / "h.msh")
    t = LinearHeatConduction.from_mesh_tags(r, 600.0, 4e-5, 300.0, True, 10.0)
    assert np.array_equal(t.dirichlet_nodes, ref.dirichlet_nodes)
    for a, c in zip(t.robin_groups, ref.robin_groups):
        key = lambda x: np.lexsort(x.T[::-1])                 # noqa: E731
        assert np.array_equal(a[key(a)], c[key(c)])


def test_msh_rejects_unsupported_input(tmp_path):
    from sktopt_gb300.mesh import read_msh
    # binary without its endianness mark, and a truncated binary node block
    (tmp_path / "bin.msh").write_text("$MeshFormat\n4.1 1 8\n$EndMeshFormat\n")
    with pytest.raises(ValueError, match="endianness"):
        read_msh(tmp_path / "bin.msh")
    (tmp_path / "trunc.msh").write_bytes(b"$MeshFormat\n2.2 1 8\n\x01\x00\x00\x00\n"
                                         b"$EndMeshFormat\n$Nodes\n5\n\x01\x00")
    with pytest.raises(ValueError, match="truncated"):
        read_msh(tmp_path / "trunc.msh")
    (tmp_path / "none.msh").write_text("hello\n")
    with pytest.raises(ValueError, match="not a gmsh"):
        read_msh(tmp_path / "none.msh")
    # a hexahedron and a tetrahedron in one file
    mixed = """$MeshFormat
2.2 0 8
$EndMeshFormat
$Nodes
9
1 0 0 0
2 1 0 0
3 1 1 0
4 0 1 0
5 0 0 1
6 1 0 1
7 1 1 1
8 0 1 1
9 2 0 0
$EndNodes
$Elements
2
1 5 2 0 0 1 2 3 4 5 6 7 8
2 4 2 0 0 2 9 3 6
$EndElements
"""
    (tmp_path / "mixed.msh").write_text(mixed)
    with pytest.raises(ValueError, match="hexahedra or tetrahedra"):
        read_msh(tmp_path / "mixed.msh")


def test_traction_direction_and_length_checks():
    from sktopt_gb300.mesh import assemble_surface_forces, boundary_facets, create_box_hex
    m = create_box_hex(2, 2, 2)
    f = boundary_facets(m)[:3]
    with pytest.raises(ValueError):
        assemble_surface_forces(m, [f, f], ["u^1"], [1.0, 2.0])
    with pytest.raises(ValueError):
        assemble_surface_forces(m, f, "x", 1.0)


def test_msh41_cell_in_two_physical_groups(tmp_path):
    """A volume entity carrying two physical tags: its cells appear once in the
    mesh and in both subdomains."""
    from sktopt_gb300.mesh import read_msh
    text = _MSH41.replace('3\n2 1 "dirichlet"\n2 2 "neumann"\n3 3 "design"',
                          '4\n2 1 "dirichlet"\n2 2 "neumann"\n3 3 "design"\n3 4 "solid"')
    # volume entity 1: bounding box, 2 physical tags (3, 4), no bounding surfaces
    text = text.replace("1 0 0 0 2 1 1 1 3 0\n$EndEntities", "1 0 0 0 2 1 1 2 3 4 0\n$EndEntities")
    nid = lambda x, y, z: 1 + x + 3 * y + 6 * z          # noqa: E731
    xyz = [(x, y, z) for z in range(2) for y in range(2) for x in range(3)]
    gm = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    hexes = [" ".join(str(nid(x + o[0], o[1], o[2])) for o in gm) for x in (0, 1)]
    text = text.format(
        tags="\n".join(str(nid(*c)) for c in xyz),
        xyz="\n".join(f"{c[0]}.0 {c[1]}.0 {c[2]}.0" for c in xyz),
        q0=" ".join(str(nid(0, y, z)) for y, z in ((0, 0), (1, 0), (1, 1), (0, 1))),
        q1=" ".join(str(nid(2, y, z)) for y, z in ((0, 0), (1, 0), (1, 1), (0, 1))),
        h0=hexes[0], h1=hexes[1])
    (tmp_path / "g.msh").write_text(text)
    m = read_msh(tmp_path / "g.msh")
    assert m.nelements == 2
    assert np.array_equal(m.subdomains["design"], [0, 1])
    assert np.array_equal(m.subdomains["solid"], [0, 1])
