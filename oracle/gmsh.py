"""Oracle (test infrastructure only): a Python restatement of LehrFEM++'s
GmshReader for 2D first-order meshes.

Follows lib/lf/io/gmsh_reader.cc (InitGmshFile for MSH 2.2: lines 116-325,
for MSH 4.1: lines 327-620, ReadGmshFile: 622-660) and the file grammars of
io/gmsh_file_v2.cc:600-739 and io/gmsh_file_v4_{text,binary}.cc.  Only
tests/ and bench.py's CPU-baseline leg use it; the library has its own C++
reader (lehrfempp_gb300/csrc/lfg_gmsh.cc).

read(path_or_bytes) -> dict with
  xy         (N, 2) main nodes in file order (AddPoint order)
  cells      (C, 4) int64 node indices, -1 in slot 3 for triangles
  edges      (E, 2) the segment elements (pre-registered edges), file order
  phys       [cells, edges, nodes]: per entity a list of physical numbers
  names      [(dim, nr, name)] from $PhysicalNames
"""
import struct

import numpy as np

NUM_NODES = {1: 2, 2: 3, 3: 4, 8: 3, 9: 6, 10: 9, 15: 1, 16: 8}
DIM = {15: 0, 1: 1, 8: 1, 2: 2, 3: 2, 9: 2, 10: 2, 16: 2}
MAIN = {15: 1, 1: 2, 8: 2, 2: 3, 9: 3, 3: 4, 10: 4, 16: 4}
SECOND_ORDER = (8, 9, 10, 16)


class GmshError(Exception):
    def __init__(self, kind, msg):
        super().__init__(msg)
        self.kind = kind  # "io" | "unsupported" | "notfound"


class _Tok:
    """ASCII token stream with byte offsets, so binary blocks can follow."""

    def __init__(self, data):
        self.d = data
        self.p = 0

    def skip_ws(self):
        d, p = self.d, self.p
        while p < len(d) and d[p] in b" \t\r\n":
            p += 1
        self.p = p

    def word(self):
        self.skip_ws()
        s = self.p
        d = self.d
        while self.p < len(d) and d[self.p] not in b" \t\r\n":
            self.p += 1
        return d[s:self.p].decode("latin-1")

    def int(self):
        w = self.word()
        try:
            return int(w)
        except ValueError:
            raise GmshError("io", "expected an integer, got %r" % w)

    def float(self):
        w = self.word()
        try:
            return float(w)
        except ValueError:
            raise GmshError("io", "expected a number, got %r" % w)

    def quoted(self):
        self.skip_ws()
        if self.d[self.p:self.p + 1] != b'"':
            raise GmshError("io", "expected a quoted name")
        e = self.d.index(b'"', self.p + 1)
        s = self.d[self.p + 1:e].decode("latin-1")
        self.p = e + 1
        return s

    def expect(self, w):
        got = self.word()
        if got != w:
            raise GmshError("io", "expected %s, got %r" % (w, got))

    def line_end(self):
        e = self.d.index(b"\n", self.p)
        self.p = e + 1

    def take(self, fmt):
        n = struct.calcsize(fmt)
        if self.p + n > len(self.d):
            raise GmshError("io", "binary data ends early")
        v = struct.unpack_from(fmt, self.d, self.p)
        self.p += n
        return v


def _check_type(t):
    if t not in NUM_NODES:
        raise GmshError("unsupported", "Gmsh element type %d not supported" % t)
    return NUM_NODES[t]


def _parse(data):
    tk = _Tok(data)
    tk.expect("$MeshFormat")
    ver = tk.word()
    ftype = tk.int()
    dsize = tk.int()
    if ver not in ("2.2", "4.1"):
        raise GmshError("unsupported", "GmshFiles with Version %s are not yet supported." % ver)
    if dsize != 8:
        raise GmshError("io", "data-size must be 8")
    binary = ftype == 1
    end = "<"
    if binary:
        tk.line_end()
        (one,) = tk.take("<i")
        if one != 1:
            end = ">"
            if struct.unpack(">i", struct.pack("<i", one))[0] != 1:
                raise GmshError("io", "bad binary one")
    tk.expect("$EndMeshFormat")
    f = {"version": 2 if ver == "2.2" else 4, "binary": binary, "names": [], "entities": {}, "nodes": [],
         "elements": [], "blocks": [], "part_entities": {}, "num_partitions": 0}
    while True:
        tk.skip_ws()
        if tk.p >= len(data):
            break
        sec = tk.word()
        if sec == "$PhysicalNames":
            for _ in range(tk.int()):
                dim, nr = tk.int(), tk.int()
                f["names"].append((dim, nr, tk.quoted()))
            tk.expect("$EndPhysicalNames")
        elif sec == "$Entities" and f["version"] == 4:
            _entities_v4(tk, f, binary, end)
            tk.expect("$EndEntities")
        elif sec == "$PartitionedEntities" and f["version"] == 4:
            _partitioned_v4(tk, f, binary, end)
            tk.expect("$EndPartitionedEntities")
        elif sec == "$Nodes":
            (_nodes_v2 if f["version"] == 2 else _nodes_v4)(tk, f, binary, end)
            tk.expect("$EndNodes")
        elif sec == "$Elements":
            (_elements_v2 if f["version"] == 2 else _elements_v4)(tk, f, binary, end)
            tk.expect("$EndElements")
        elif sec.startswith("$"):
            marker = ("$End" + sec[1:]).encode()
            e = data.find(marker, tk.p)
            if e < 0:
                raise GmshError("io", "unterminated section %s" % sec)
            tk.p = e + len(marker)
        else:
            raise GmshError("io", "expected a section, got %r" % sec)
    return f


def _nodes_v2(tk, f, binary, end):
    n = tk.int()
    if not binary:
        for _ in range(n):
            tag = tk.int()
            f["nodes"].append((tag, tk.float(), tk.float(), tk.float()))
    else:
        tk.line_end()
        for _ in range(n):
            f["nodes"].append(tk.take(end + "iddd"))


def _elements_v2(tk, f, binary, end):
    n = tk.int()
    if not binary:
        for _ in range(n):
            tk.int()
            t = tk.int()
            nn = _check_type(t)
            ntags = tk.int()
            tags = [tk.int() for _ in range(ntags)]
            nodes = tuple(tk.int() for _ in range(nn))
            f["elements"].append({"type": t, "phys": tags[0], "nodes": nodes, "block": 0})
    else:
        tk.line_end()
        done = 0
        while done < n:
            t, cnt, ntags = tk.take(end + "iii")
            nn = _check_type(t)
            for _ in range(cnt):
                v = tk.take(end + "i" * (1 + ntags + nn))
                f["elements"].append({"type": t, "phys": v[1], "nodes": tuple(v[1 + ntags:]), "block": 0})
            done += cnt


def _entities_v4(tk, f, binary, end):
    if binary:
        tk.line_end()
        counts = tk.take(end + "QQQQ")
    else:
        counts = [tk.int() for _ in range(4)]
    for dim in range(4):
        for _ in range(counts[dim]):
            if binary:
                (tag,) = tk.take(end + "i")
                tk.take(end + "d" * (3 if dim == 0 else 6))
                (np_,) = tk.take(end + "Q")
                phys = list(tk.take(end + "i" * np_))
                if dim > 0:
                    (nb,) = tk.take(end + "Q")
                    tk.take(end + "i" * nb)
            else:
                tag = tk.int()
                for _ in range(3 if dim == 0 else 6):
                    tk.float()
                phys = [tk.int() for _ in range(tk.int())]
                if dim > 0:
                    for _ in range(tk.int()):
                        tk.int()
            f["entities"][(dim, tag)] = phys


def _partitioned_v4(tk, f, binary, end):
    """$PartitionedEntities: gmsh_file_v4_binary.cc:108-132 / the text grammar."""
    q = (lambda: tk.take(end + "Q")[0]) if binary else tk.int
    i = (lambda: tk.take(end + "i")[0]) if binary else tk.int
    d = (lambda: tk.take(end + "d")[0]) if binary else tk.float
    if binary:
        tk.line_end()
    f["num_partitions"] = q()
    for _ in range(q()):
        i(), i()
    counts = [q() for _ in range(4)]
    for dim in range(4):
        for _ in range(counts[dim]):
            tag = i()
            i(), i()
            for _ in range(q()):
                i()
            for _ in range(3 if dim == 0 else 6):
                d()
            phys = [i() for _ in range(q())]
            if dim > 0:
                for _ in range(q()):
                    i()
            f["part_entities"][(dim, tag)] = phys


def _nodes_v4(tk, f, binary, end):
    if binary:
        tk.line_end()
        nb, nn, _, _ = tk.take(end + "QQQQ")
    else:
        nb, nn = tk.int(), tk.int()
        tk.int(), tk.int()
    for _ in range(nb):
        if binary:
            edim, _, param, n = tk.take(end + "iiiQ")
        else:
            edim, _, param, n = tk.int(), tk.int(), tk.int(), tk.int()
        extra = min(max(edim, 0), 3) if param else 0
        if binary:
            tags = tk.take(end + "Q" * n)
            coords = [tk.take(end + "d" * (3 + extra))[:3] for _ in range(n)]
        else:
            tags = [tk.int() for _ in range(n)]
            coords = []
            for _ in range(n):
                c = [tk.float() for _ in range(3 + extra)]
                coords.append(tuple(c[:3]))
        for t, c in zip(tags, coords):
            f["nodes"].append((t,) + tuple(c))
    if len(f["nodes"]) != nn:
        raise GmshError("io", "node count mismatch")


def _elements_v4(tk, f, binary, end):
    if binary:
        tk.line_end()
        nb, ne, _, _ = tk.take(end + "QQQQ")
    else:
        nb, ne = tk.int(), tk.int()
        tk.int(), tk.int()
    for _ in range(nb):
        if binary:
            edim, etag, t, n = tk.take(end + "iiiQ")
        else:
            edim, etag, t, n = tk.int(), tk.int(), tk.int(), tk.int()
        nn = _check_type(t)
        f["blocks"].append((edim, etag))
        bi = len(f["blocks"]) - 1
        for _ in range(n):
            if binary:
                v = tk.take(end + "Q" * (1 + nn))
            else:
                v = [tk.int() for _ in range(1 + nn)]
            f["elements"].append({"type": t, "phys": 0, "nodes": tuple(v[1:]), "block": bi})
    if len(f["elements"]) != ne:
        raise GmshError("io", "element count mismatch")


def read(src):
    data = src if isinstance(src, (bytes, bytearray)) else open(src, "rb").read()
    f = _parse(bytes(data))
    v4 = f["version"] == 4
    # main nodes (gmsh_reader.cc:135-160 / 350-380)
    main = set()
    ncells = 0
    for el in f["elements"]:
        d = DIM[el["type"]]
        ncells += d == 2
        if (el["type"] != 15) if not v4 else (d == 2):
            main.update(el["nodes"][:MAIN[el["type"]]])
    if ncells == 0:
        raise GmshError("io", "MshFile contains no elements with dimension 2")
    tag2mi = {}
    xy = []
    for tag, x, y, z in f["nodes"]:
        if tag in main:
            if z != 0.0:
                raise GmshError("io", "In a 2D GmshMesh, the z-coordinate of every node must be zero")
            tag2mi[tag] = len(xy)
            xy.append((x, y))
    cells, edges = [], []
    src = {0: [], 1: [], 2: []}   # codim -> per entity: element indices
    node_src = src[2]
    begin = 0
    els = f["elements"]
    for e, el in enumerate(els):
        t = el["type"]
        codim = 2 - DIM[t]
        b = els[begin]
        same = (b["type"] == t) if not v4 else (b["block"] == el["block"])
        if e != begin and same and b["nodes"] == el["nodes"]:
            if codim == 2:
                if node_src:
                    node_src[-1].append(e)
            else:
                src[codim][-1].append(e)
            continue
        begin = e
        if t == 15:
            mi = tag2mi.get(el["nodes"][0])
            if mi is not None:
                while len(node_src) <= mi:
                    node_src.append([])
                node_src[mi].append(e)
            continue
        if t in SECOND_ORDER:
            raise GmshError("unsupported", "second-order element type %d" % t)
        try:
            v = [tag2mi[n] for n in el["nodes"][:MAIN[t]]]
        except KeyError:
            raise GmshError("io", "element references a node that is not a cell corner")
        if t == 1:
            edges.append(v)
        else:
            cells.append(v + [-1] * (4 - len(v)))
        src[codim].append([e])
    phys = []
    for c in (0, 1, 2):
        lists = []
        for lst in src[c]:
            nrs = []
            for e in lst:
                if not v4:
                    nrs.append(els[e]["phys"])
                else:
                    table = f["part_entities"] if f["num_partitions"] > 0 else f["entities"]
                    nrs.extend(table.get(f["blocks"][els[e]["block"]], []))
            lists.append(nrs)
        phys.append(lists)
    return {"xy": np.array(xy, float).reshape(-1, 2), "cells": np.array(cells, np.int64).reshape(-1, 4),
            "edges": np.array(edges, np.int64).reshape(-1, 2), "phys": phys, "names": f["names"]}


def name_to_nr(names, name, codim=-1):
    """PhysicalEntityName2Nr (gmsh_reader.cc:32-66) over $PhysicalNames of a 2D mesh."""
    hits = [(nr, 2 - dim) for dim, nr, nm in names if nm == name]
    if not hits:
        raise GmshError("notfound", "No Physical Entity with this name found.")
    if len(hits) == 1:
        if codim in (-1, hits[0][1]):
            return hits[0][0]
    else:
        if codim == -1:
            raise GmshError("notfound", "multiple physical entities with this name")
        for nr, c in hits:
            if c == codim:
                return nr
    raise GmshError("notfound", "not found")


def nr_to_name(names, nr, codim=-1):
    """PhysicalEntityNr2Name (gmsh_reader.cc:68-99)."""
    hits = [(nm, 2 - dim) for dim, n, nm in names if n == nr]
    if not hits:
        raise GmshError("notfound", "Physical entity with number %d not found." % nr)
    if len(hits) == 1:
        if codim in (-1, hits[0][1]):
            return hits[0][0]
    else:
        if codim == -1:
            raise GmshError("notfound", "multiple physical entities with this number")
        for nm, c in hits:
            if c == codim:
                return nm
    raise GmshError("notfound", "not found")
