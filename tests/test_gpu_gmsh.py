"""Gmsh reader -> device mesh (GPU): the mesh built from a .msh file has the
oracle's numbering bit for bit (nodes, cells, pre-registered and created
edges, orientations), and physical groups select edges for the boundary-edge
providers exactly as on the oracle."""
import os

import numpy as np
import pytest

from parity import O, L, W, compare_triplets
from test_gmsh_reader import FIRST_ORDER, G, _path

pytestmark = pytest.mark.gpu


def _same_topology(mesh, r):
    om = O.Mesh(r["xy"], r["cells"], r["edges"] if len(r["edges"]) else None)
    assert (mesh.num_nodes, mesh.num_edges, mesh.num_cells) == (om.num_nodes, om.num_edges, om.num_cells)
    en, ce, co, nc = mesh.topology()
    oen, oce, oco, onc = om.topology()
    assert np.array_equal(en, oen)
    assert np.array_equal(ce, oce)
    assert np.array_equal(co, oco)
    assert np.array_equal(nc, onc)
    return om


@pytest.mark.parametrize("name", FIRST_ORDER)
def test_fixture_meshes_on_device(ctx, name):
    r = G.read(_path(name))
    rd = L.GmshReader(ctx, _path(name))
    _same_topology(rd.mesh, r)
    # edges beyond the segment elements carry no physical numbers
    ep = rd.physical_entity_nr(1)
    assert len(ep) == rd.mesh.num_edges
    assert ep[: len(r["phys"][1])] == r["phys"][1]
    assert all(p == [] for p in ep[len(r["phys"][1]):])


def test_piece_of_cake_counts(ctx):
    """checkPieceOfCake: 2 cells, 5 edges, 4 nodes; the arc edges are group 2."""
    rd = L.GmshReader(ctx, _path("piece_of_cake.msh"))
    m = rd.mesh
    assert (m.num_cells, m.num_edges, m.num_nodes) == (2, 5, 4)
    arc = rd.is_physical_entity(1, rd.physical_entity_name2nr("arc"))
    en, _, _, _ = m.topology()
    xy, _ = m.geometry()
    on_arc = np.array([all(abs(np.hypot(*xy[v]) - 1) < 1e-6 for v in e) for e in en])
    assert np.array_equal(arc.astype(bool), on_arc)


@pytest.mark.parametrize("version,binary", [(2, False), (2, True), (4, False), (4, True)])
def test_synthetic_file_pipeline(ctx, tmp_path, version, binary):
    """A hybrid mesh with two physical boundary groups: read, build on the
    device, select the 'right' group's edges and assemble the edge mass
    matrix there; the cell matrix of the whole mesh against the oracle."""
    xy, cells = W.hybrid_mesh(12, seed=9)
    bottom = np.where(np.abs(xy[:, 1]) < 1e-12)[0]
    bottom = bottom[np.argsort(xy[bottom, 0])]
    edges = np.stack([bottom[:-1], bottom[1:]], 1)
    ep = np.where(np.arange(len(edges)) < len(edges) // 2, 7, 8)
    p = str(tmp_path / "m.msh")
    W.write_msh(p, xy, cells, edges, edge_phys=ep, version=version, binary=binary,
                names=[(1, 7, "left"), (1, 8, "right"), (2, 1, "domain")])
    r = G.read(p)
    rd = L.GmshReader(ctx, p)
    om = _same_topology(rd.mesh, r)
    right = rd.is_physical_entity(1, rd.physical_entity_name2nr("right"))
    assert right.sum() == (ep == 8).sum()
    for degree in (1, 2):
        sp = L.Space.lagrange(rd.mesh, degree)
        osp = O.Space(om, degree)
        n = degree + 1
        active = int(right.sum())
        coo = L.COOMatrix(ctx, sp.num_dofs, sp.num_dofs, active * n * n)
        L.assemble_matrix_edge_mass(sp, L.edge_mass_provider(L.coeff(L.CONSTANT, 1.5), ctx.to_device(right)), coo)
        rr, cc, vv = O.assemble_edge_mass(osp, O.coeff(O.CONSTANT, 1.5), right).arrays()
        compare_triplets(coo.triplets(), rr, cc, vv, np.full(active, n * n))
        # the right group spans half the bottom side: its edge mass sums to its length
        assert abs(coo.triplets()["value"].sum() / 1.5 - np.ptp(xy[edges[ep == 8]][:, :, 0])) < 1e-12
