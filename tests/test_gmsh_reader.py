"""Gmsh reader (CPU): the oracle's restatement against the reference's own
reader tests (lib/lf/io/test/gmsh_reader_tests.cc) on the reference's .msh
fixtures (copied into tests/golden/msh/ by tests/golden/make_golden.py), and
the library's C++ reader (lfg_gmsh_*, host-only) against the oracle on those
fixtures and on synthetic MSH 2.2 / 4.1 ASCII / binary files."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
import gmsh as G  # noqa: E402
import oracle as O  # noqa: E402

MSH = os.path.join(HERE, "golden", "msh")
FIRST_ORDER = ["two_element_hybrid_2d.msh", "two_element_hybrid_2d_binary.msh", "two_element_hybrid_2d_v4.msh",
               "two_element_hybrid_2d_v4_binary.msh", "piece_of_cake.msh", "piece_of_cake_binary.msh",
               "circle_first_order.msh", "circle_first_order_v4.msh", "lecturedemomesh.msh"]
SECOND_ORDER = ["two_element_hybrid_2d_second_order.msh", "two_element_hybrid_2d_second_order_v4.msh",
                "circle_second_order.msh", "circle_second_order_v4.msh", "circle_second_order_quad.msh",
                "circle_second_order_quad_v4.msh", "curved_square_quads_2nd_order.msh",
                "curved_square_trias_2nd_order.msh", "curved_square_quads_2nd_order_v4.msh",
                "curved_square_trias_2nd_order_v4.msh"]


def _path(name):
    return os.path.join(MSH, name)


def _oracle_mesh(r):
    return O.Mesh(r["xy"], r["cells"], r["edges"] if len(r["edges"]) else None)


def _edge_phys(r, m):
    """Physical numbers of every mesh edge (edges beyond the preset list: none)."""
    return r["phys"][1] + [[] for _ in range(m.num_edges - len(r["phys"][1]))]


def _node_phys(r, m):
    return r["phys"][2] + [[] for _ in range(m.num_nodes - len(r["phys"][2]))]


@pytest.mark.parametrize("name", FIRST_ORDER[:4])
def test_oracle_two_element_mesh(name):
    """checkTwoElementMesh (gmsh_reader_tests.cc:22-140)."""
    r = G.read(_path(name))
    m = _oracle_mesh(r)
    assert (m.num_cells, m.num_edges, m.num_nodes) == (2, 6, 5)
    origin = int(np.argmin((r["xy"] ** 2).sum(1)))
    assert (r["xy"][origin] ** 2).sum() < 1e-10
    nphys = _node_phys(r, m)
    assert nphys[origin] == [1, 2]
    assert all(len(p) == 0 for i, p in enumerate(nphys) if i != origin)
    en, _, _, _ = m.topology()
    lens = np.hypot(*(r["xy"][en[:, 1]] - r["xy"][en[:, 0]]).T)
    diag = int(np.argmax(lens))
    assert lens[diag] > 1.1
    ephys = _edge_phys(r, m)
    assert ephys[diag] == [4]
    assert all(len(p) == 0 for i, p in enumerate(ephys) if i != diag)
    quad = [c for c in range(2) if r["cells"][c, 3] >= 0][0]
    tria = 1 - quad
    assert r["phys"][0][quad] == [5] and r["phys"][0][tria] == [1, 3]
    names = r["names"]
    assert G.nr_to_name(names, 1, 2) == "physicalEntity1"
    assert G.nr_to_name(names, 2) == "physicalEntity2"
    assert G.name_to_nr(names, "physicalEntity2") == 2
    assert G.name_to_nr(names, "physicalEntity1", 0) == 1
    assert G.name_to_nr(names, "physicalEntity3") == 3
    assert G.name_to_nr(names, "diagonal") == 4
    for bad in (lambda: G.nr_to_name(names, 1), lambda: G.name_to_nr(names, "physicalEntity1"),
                lambda: G.nr_to_name(names, 100), lambda: G.name_to_nr(names, "gugus"),
                lambda: G.nr_to_name(names, 3, 1)):
        with pytest.raises(G.GmshError):
            bad()


@pytest.mark.parametrize("name", ["piece_of_cake.msh", "piece_of_cake_binary.msh"])
def test_oracle_piece_of_cake(name):
    """checkPieceOfCake (gmsh_reader_tests.cc:229-296): a partitioned 4.1 file."""
    r = G.read(_path(name))
    m = _oracle_mesh(r)
    assert (m.num_cells, m.num_edges, m.num_nodes) == (2, 5, 4)
    origin = int(np.argmin((r["xy"] ** 2).sum(1)))
    assert _node_phys(r, m)[origin] == [1]
    en, _, _, _ = m.topology()
    ephys = _edge_phys(r, m)
    for e in range(m.num_edges):
        on_arc = all(abs(np.hypot(*r["xy"][v]) - 1) < 1e-6 for v in en[e])
        assert (ephys[e] == [2]) == on_arc
    assert r["phys"][0] == [[3], [3]]
    assert G.name_to_nr(r["names"], "origin") == 1 and G.name_to_nr(r["names"], "arc") == 2
    with pytest.raises(G.GmshError):
        G.nr_to_name(r["names"], 3)


def test_oracle_circle_volume():
    """secondOrderMesh (gmsh_reader_tests.cc:195-228), first-order part: the
    polygon misses pi by more than 0.3."""
    for name in ("circle_first_order.msh", "circle_first_order_v4.msh"):
        r = G.read(_path(name))
        m = _oracle_mesh(r)
        s = O.Space(m, 1)
        area = O.integrate(s, O.INT_VALUE, O.coeff(O.CONSTANT, 1.0), qdeg=10)
        assert abs(area - np.pi) > 0.3


@pytest.mark.parametrize("name", SECOND_ORDER)
def test_oracle_rejects_second_order(name):
    with pytest.raises(G.GmshError) as e:
        G.read(_path(name))
    assert e.value.kind == "unsupported"


# ------------------------------------------------- the library's C++ reader

@pytest.fixture(scope="module")
def L():
    import lehrfempp_gb300 as lib
    lib.load()
    return lib


def _compare(reader, r):
    xy, cells, edges = reader.factory_input()
    assert np.array_equal(xy, r["xy"])
    assert np.array_equal(cells, r["cells"])
    assert np.array_equal(edges, r["edges"])
    for c in range(3):
        n = len(r["phys"][c])
        assert reader.physical_entity_nr(c, n) == r["phys"][c], c


@pytest.mark.parametrize("name", FIRST_ORDER)
def test_capi_reader_matches_oracle_on_fixtures(L, name):
    r = G.read(_path(name))
    reader = L.GmshReader(filename=_path(name))
    _compare(reader, r)
    with open(_path(name), "rb") as fh:
        _compare(L.GmshReader(data=fh.read()), r)
    for d, nr, nm in r["names"]:
        assert reader.physical_entity_nr2name(nr, 2 - d) == nm
        assert reader.physical_entity_name2nr(nm, 2 - d) == nr
    for codim in (0, 1, 2):
        want = sorted({(nr, nm) for d, nr, nm in r["names"] if 2 - d == codim})
        assert sorted(reader.physical_entities(codim)) == want


@pytest.mark.parametrize("name", FIRST_ORDER[:4])
def test_capi_name_lookups(L, name):
    """The lookups and failures of checkTwoElementMesh through the C-ABI."""
    rd = L.GmshReader(filename=_path(name))
    assert rd.physical_entity_nr2name(1, 2) == "physicalEntity1"
    assert rd.physical_entity_nr2name(2) == "physicalEntity2"
    assert rd.physical_entity_name2nr("physicalEntity2") == 2
    assert rd.physical_entity_name2nr("square") == 5
    for bad in (lambda: rd.physical_entity_nr2name(1), lambda: rd.physical_entity_name2nr("physicalEntity1"),
                lambda: rd.physical_entity_nr2name(100), lambda: rd.physical_entity_name2nr("gugus"),
                lambda: rd.physical_entity_nr2name(3, 1)):
        with pytest.raises(L.LfgError) as e:
            bad()
        assert e.value.code == L.NOT_FOUND
    fl = rd.is_physical_entity(0, 3)
    assert list(fl) == [int(3 in p) for p in rd.physical_entity_nr(0)]


@pytest.mark.parametrize("name", SECOND_ORDER)
def test_capi_rejects_second_order(L, name):
    with pytest.raises(L.LfgError) as e:
        L.GmshReader(filename=_path(name))
    assert e.value.code == L.UNSUPPORTED


def test_capi_errors(L, tmp_path):
    with pytest.raises(L.LfgError) as e:
        L.GmshReader(filename=str(tmp_path / "missing.msh"))
    assert e.value.code == L.IO_ERROR
    good = open(_path("two_element_hybrid_2d.msh"), "rb").read()
    for cut in (40, 120, len(good) - 20):
        with pytest.raises(L.LfgError) as e:
            L.GmshReader(data=good[:cut])
        assert e.value.code == L.IO_ERROR, cut
    with pytest.raises(L.LfgError) as e:
        L.GmshReader(data=good.replace(b"2.2 0 8", b"3.0 0 8"))
    assert e.value.code == L.UNSUPPORTED
    with pytest.raises(L.LfgError) as e:   # a tetrahedron
        L.GmshReader(data=good.replace(b"6 3 2 5 1 1 4 5 2", b"6 4 2 5 1 1 4 5 2"))
    assert e.value.code == L.UNSUPPORTED


@pytest.mark.parametrize("version", [2, 4])
@pytest.mark.parametrize("binary", [False, True])
def test_capi_reader_synthetic(L, tmp_path, version, binary):
    """Random hybrid meshes with physical groups and segment elements, written
    in all four encodings, read by both readers."""
    from lehrfempp_gb300 import workloads as W
    for n, seed in ((7, 1), (20, 2)):
        xy, cells = W.hybrid_mesh(n, seed=seed)
        rng = np.random.default_rng(seed)
        cp = rng.integers(1, 5, len(cells))
        # boundary segments of the bottom side, one physical group per half
        bottom = np.where(np.abs(xy[:, 1]) < 1e-12)[0]
        bottom = bottom[np.argsort(xy[bottom, 0])]
        edges = np.stack([bottom[:-1], bottom[1:]], 1)
        ep = np.where(np.arange(len(edges)) < len(edges) // 2, 7, 8)
        names = [(2, 1, "one"), (2, 2, "two"), (1, 7, "left"), (1, 8, "right")]
        p = str(tmp_path / ("m_%d_%d_%d.msh" % (version, binary, n)))
        W.write_msh(p, xy, cells, edges, cell_phys=cp, edge_phys=ep, version=version, binary=binary, names=names)
        r = G.read(p)
        _compare(L.GmshReader(filename=p), r)
        # the file round-trips the mesh: the same node coordinates, cells as a multiset
        assert np.array_equal(r["xy"], xy)
        assert sorted(map(tuple, r["cells"])) == sorted(map(tuple, cells))
