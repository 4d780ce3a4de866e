"""Seeded synthetic inputs for the five measured configurations.

Each builder returns a plain description (numpy arrays + coefficient specs)
that both the GPU library and the oracle consume, so the two sides see the
same mesh, numbering input and coefficients.  Sizes are parameters: tests use
small instances of the same generators, the benchmark the full ones.

Coefficient spec: ("zero",) | ("const", v) | ("cell", array) | ("nodal", array)
                  | ("poly", p16) | ("sinsin", p0, p1, p2, p3) | ("sincos", ...)
"""
import numpy as np


def poly(**terms):
    """16 coefficients p[4i+j] of sum c_ij x^i y^j; keys c, x1, y2, x1y1, ..."""
    p = np.zeros(16)
    for k, val in terms.items():
        if k == "c":
            p[0] += val
            continue
        i = int(k[1]) if k.startswith("x") else 0
        j = int(k[k.index("y") + 1]) if "y" in k else 0
        p[4 * i + j] += val
    return p


def tp_triag_spec(n):
    return {"kind": "tptriag", "nx": n, "ny": n}


def config1(n=64):
    """Plain method: 64x64 TPTriag, O1, alpha = 1+x^2+y^2, gamma = 1,
    f = sin(pi x) sin(pi y), degree-4 rules, homogeneous Dirichlet."""
    return {
        "name": "c1_tptriag%d_o1" % n, "mesh": tp_triag_spec(n), "degree": 1,
        "alpha": ("poly", poly(c=1.0, x2=1.0, y2=1.0)), "gamma": ("const", 1.0),
        "f": ("sinsin", 0.0, 1.0, 1.0, 1.0), "qr_tria": 4, "qr_quad": 4, "dirichlet": 0.0,
    }


def hybrid_mesh(n, seed=2, p_quad=0.5, jitter=0.2):
    """n x n squares on [0,1]^2; each square is a quadrilateral or split into
    the two triangles of the TPTriag pattern with probability 1/2; interior
    nodes jittered by U(-jitter h, jitter h) per coordinate.  Cells are listed
    square by square (j outer, i inner); only cells are given to the factory,
    so edges are numbered in (min, max) node order."""
    rng = np.random.default_rng(seed)
    h = 1.0 / n
    i = np.arange(n + 1)
    X, Y = np.meshgrid(i * h, i * h)  # [j, i]
    xy = np.stack([X.ravel(), Y.ravel()], axis=1)
    inner = np.zeros((n + 1, n + 1), bool)
    inner[1:-1, 1:-1] = True
    inner = inner.ravel()
    d = rng.uniform(-jitter * h, jitter * h, size=(inner.sum(), 2))
    xy[inner] += d
    is_quad = rng.random(n * n) < p_quad
    jj, ii = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    ii, jj = ii.ravel(), jj.ravel()
    v00 = ii + jj * (n + 1)
    v10 = v00 + 1
    v01 = v00 + (n + 1)
    v11 = v01 + 1
    quad = np.stack([v00, v10, v11, v01], 1)
    tri_up = np.stack([v00, v11, v01, np.full_like(v00, -1)], 1)
    tri_lo = np.stack([v00, v10, v11, np.full_like(v00, -1)], 1)
    # square s contributes [quad] or [up triangle, low triangle]
    count = np.where(is_quad, 1, 2)
    starts = np.concatenate([[0], np.cumsum(count)[:-1]])
    out = np.empty((int(count.sum()), 4), np.int64)
    out[starts] = np.where(is_quad[:, None], quad, tri_up)
    out[starts[~is_quad] + 1] = tri_lo[~is_quad]
    return xy, out


def config2(n=2048, seed=2):
    """Large hybrid mesh, precision form: O2, alpha per-cell LogNormal(0, 1),
    gamma = 0, f = 1, default rules (degree 4), homogeneous Dirichlet."""
    xy, cells = hybrid_mesh(n, seed=seed)
    rng = np.random.default_rng(seed + 1000)
    alpha = np.exp(rng.standard_normal(len(cells)))
    return {
        "name": "c2_hybrid%d_o2" % n, "mesh": {"kind": "factory", "xy": xy, "cells": cells, "edges": None},
        "degree": 2, "alpha": ("cell", alpha), "gamma": ("zero",), "f": ("const", 1.0),
        "qr_tria": 0, "qr_quad": 0, "dirichlet": 0.0,
    }


def config3(n=1024, seed=3):
    """High order: TPTriag n x n, O3, degree-6 rules, alpha = 1 + 0.5 sin(4 pi x)
    cos(4 pi y), gamma = 1, f = O1 interpolant of i.i.d. N(0,1) nodal values."""
    rng = np.random.default_rng(seed)
    fn = rng.standard_normal((n + 1) * (n + 1))
    return {
        "name": "c3_tptriag%d_o3" % n, "mesh": tp_triag_spec(n), "degree": 3,
        "alpha": ("sincos", 1.0, 0.5, 4.0, 4.0), "gamma": ("const", 1.0), "f": ("nodal", fn),
        "qr_tria": 6, "qr_quad": 6, "dirichlet": 0.0,
    }


def config5(n=1024, seed=5):
    """Differentiation form: TPTriag n x n, O1, alpha = exp(theta) per cell,
    theta ~ N(0, 0.5^2), gamma = 0, f = 1, Dirichlet 0.  Observations are
    u(theta_true(cell centroids)) + observation_noise (built by the caller,
    which owns the solver)."""
    rng = np.random.default_rng(seed)
    theta = 0.5 * rng.standard_normal(2 * n * n)
    return {
        "name": "c5_tptriag%d_o1" % n, "mesh": tp_triag_spec(n), "degree": 1,
        "alpha": ("cell", np.exp(theta)), "gamma": ("zero",), "f": ("const", 1.0),
        "qr_tria": 0, "qr_quad": 0, "dirichlet": 0.0, "theta": theta,
    }


def cell_centroids(xy, cells):
    """Vertex averages of triangles (cells[:, 3] < 0) and quadrilaterals."""
    cells = np.asarray(cells)
    quad = cells[:, 3] >= 0
    c = np.where(cells < 0, cells[:, :1], cells)  # pad triangles with vertex 0
    s = xy[c[:, 0]] + xy[c[:, 1]] + xy[c[:, 2]] + np.where(quad[:, None], xy[c[:, 3]], 0.0)
    return s / np.where(quad, 4.0, 3.0)[:, None]


def theta_true(centroids, seed=55, bumps=8):
    """Smooth log-conductivity: sum of `bumps` Gaussian bumps with centres
    U[0.15, 0.85]^2, widths U[0.05, 0.15] and amplitudes U[-1, 1]."""
    rng = np.random.default_rng(seed)
    ctr = rng.uniform(0.15, 0.85, (bumps, 2))
    wid = rng.uniform(0.05, 0.15, bumps)
    amp = rng.uniform(-1.0, 1.0, bumps)
    t = np.zeros(len(centroids))
    for k in range(bumps):
        d2 = ((centroids - ctr[k]) ** 2).sum(axis=1)
        t += amp[k] * np.exp(-d2 / (2.0 * wid[k] ** 2))
    return t


def observation_noise(ndofs, seed=56, sigma=1e-3):
    return sigma * np.random.default_rng(seed).standard_normal(ndofs)


def batch_sizes(count=512, lo=24, hi=320, seed=4):
    """Config 4: mesh sizes n ~ round(exp(U(ln lo, ln hi))) and degrees 1|2."""
    rng = np.random.default_rng(seed)
    ns = np.rint(np.exp(rng.uniform(np.log(lo), np.log(hi), count))).astype(int)
    degs = np.where(rng.random(count) < 0.5, 1, 2)
    return ns, degs


def config4(count=512, lo=24, hi=320, seed=4):
    """Batching form: `count` TPTriag n x n unit-square meshes (n log-uniform in
    [lo, hi]), O1 or O2 (50/50), alpha per cell LogNormal(0, 0.5^2), gamma = 1,
    f = 1, homogeneous Dirichlet.  alpha is one array over the batch cells
    (mesh after mesh)."""
    ns, degs = batch_sizes(count, lo, hi, seed)
    rng = np.random.default_rng(seed + 1000)
    cells = 2 * ns.astype(np.int64) ** 2
    alpha = np.exp(0.5 * rng.standard_normal(int(cells.sum())))
    return {"name": "c4_batch%d" % count, "ns": ns, "degrees": degs, "alpha": alpha, "gamma": 1.0, "f": 1.0,
            "cells": cells}


# ------------------------------------------------------------- GPU helpers

def build_mesh(ctx, spec):
    import lehrfempp_gb300 as L
    if spec["kind"] == "tptriag":
        return L.Mesh.tp_triag(ctx, spec["nx"], spec["ny"])
    if spec["kind"] == "tpquad":
        return L.Mesh.tp_quad(ctx, spec["nx"], spec["ny"])
    return L.Mesh.from_factory(ctx, spec["xy"], spec["cells"], spec.get("edges"))


def to_coeff(ctx, spec, keep):
    """lfg_coeff for a spec; device arrays are appended to `keep`."""
    import lehrfempp_gb300 as L
    k = spec[0]
    if k == "zero":
        return L.coeff(L.ZERO)
    if k == "const":
        return L.coeff(L.CONSTANT, spec[1])
    if k in ("cell", "nodal"):
        d = ctx.to_device(np.asarray(spec[1], np.float64))
        keep.append(d)
        return L.coeff(L.PER_CELL if k == "cell" else L.NODAL_O1, data=d)
    if k == "poly":
        return L.coeff(L.ANALYTIC, func=L.FN_POLY, params=list(spec[1]))
    if k == "sinsin":
        return L.coeff(L.ANALYTIC, func=L.FN_SINSIN, params=list(spec[1:]))
    if k == "sincos":
        return L.coeff(L.ANALYTIC, func=L.FN_SINCOS, params=list(spec[1:]))
    raise ValueError(spec)


def write_msh(path, xy, cells, edges=None, cell_phys=None, edge_phys=None, version=4, binary=True,
              names=None):
    """Write a 2D first-order mesh as a Gmsh MSH 2.2 or 4.1 file (ASCII or
    binary, little endian) -- the synthetic input of the Gmsh-reader tests and
    benchmark.  cells: (C, 4) node indices, -1 in slot 3 for triangles; edges:
    (E, 2) segment elements written before the cells; *_phys: one physical
    number per element (default 1 for cells, 2 for edges); names: list of
    (dim, nr, name).  Node tags are 1-based node indices.  For 4.1 every
    distinct (dimension, physical number) becomes one model entity and the
    elements are written in blocks per (entity, element type), in order of
    first appearance, keeping their relative order inside a block."""
    import struct
    xy = np.asarray(xy, np.float64).reshape(-1, 2)
    cells = np.asarray(cells, np.int64).reshape(-1, 4)
    edges = np.zeros((0, 2), np.int64) if edges is None else np.asarray(edges, np.int64).reshape(-1, 2)
    cp = np.ones(len(cells), np.int64) if cell_phys is None else np.asarray(cell_phys, np.int64)
    ep = np.full(len(edges), 2, np.int64) if edge_phys is None else np.asarray(edge_phys, np.int64)
    names = names or []
    nn = len(xy)
    quad = cells[:, 3] >= 0
    out = bytearray()

    def w(s):
        out.extend(s.encode())

    w("$MeshFormat\n%s %d 8\n" % ("2.2" if version == 2 else "4.1", 1 if binary else 0))
    if binary:
        out.extend(struct.pack("<i", 1))
        w("\n")
    w("$EndMeshFormat\n")
    if names:
        w("$PhysicalNames\n%d\n" % len(names))
        for d, nr, nm in names:
            w('%d %d "%s"\n' % (d, nr, nm))
        w("$EndPhysicalNames\n")
    if version == 2:
        w("$Nodes\n%d\n" % nn)
        if binary:
            rec = np.zeros(nn, dtype=[("id", "<i4"), ("x", "<f8"), ("y", "<f8"), ("z", "<f8")])
            rec["id"] = np.arange(1, nn + 1)
            rec["x"], rec["y"] = xy[:, 0], xy[:, 1]
            out.extend(rec.tobytes())
            w("\n")
        else:
            w("".join("%d %.17g %.17g 0\n" % (i + 1, x, y) for i, (x, y) in enumerate(xy)))
        w("$EndNodes\n")
        ne = len(edges) + len(cells)
        w("$Elements\n%d\n" % ne)
        groups = [(1, edges, ep)]
        # keep the cell order: runs of equal type become binary groups
        if binary:
            items = [(1, e, p) for e, p in zip(edges, ep)] + \
                    [((3 if q else 2), c, p) for c, p, q in zip(cells, cp, quad)]
            k, num = 0, 1
            while k < len(items):
                t = items[k][0]
                j = k
                while j < len(items) and items[j][0] == t:
                    j += 1
                nv = {1: 2, 2: 3, 3: 4}[t]
                out.extend(struct.pack("<iii", t, j - k, 2))
                arr = np.zeros((j - k, 3 + nv), np.int32)
                arr[:, 0] = np.arange(num, num + j - k)
                arr[:, 1] = [items[m][2] for m in range(k, j)]
                arr[:, 2] = arr[:, 1]
                arr[:, 3:] = np.array([items[m][1][:nv] for m in range(k, j)]) + 1
                out.extend(arr.astype("<i4").tobytes())
                num += j - k
                k = j
            w("\n")
        else:
            lines = []
            num = 1
            for e, p in zip(edges, ep):
                lines.append("%d 1 2 %d %d %d %d\n" % (num, p, p, e[0] + 1, e[1] + 1))
                num += 1
            for c, p, q in zip(cells, cp, quad):
                nv = 4 if q else 3
                lines.append("%d %d 2 %d %d %s\n" % (num, 3 if q else 2, p, p, " ".join(str(v + 1) for v in c[:nv])))
                num += 1
            w("".join(lines))
        del groups
        w("$EndElements\n")
        with open(path, "wb") as fh:
            fh.write(bytes(out))
        return
    # ---- 4.1: entities per (dim, physical number)
    ent = {}
    for d, phys in ((1, ep), (2, cp)):
        for p in phys:
            ent.setdefault((d, int(p)), len([k for k in ent if k[0] == d]) + 1)
    ncurve = len([k for k in ent if k[0] == 1])
    nsurf = len([k for k in ent if k[0] == 2])
    w("$Entities\n")
    if binary:
        out.extend(struct.pack("<QQQQ", 0, ncurve, nsurf, 0))
        for d in (1, 2):
            for (dd, p), tag in ent.items():
                if dd != d:
                    continue
                out.extend(struct.pack("<i6dQi Q", tag, 0, 0, 0, 1, 1, 0, 1, p, 0))
        w("\n")
    else:
        w("0 %d %d 0\n" % (ncurve, nsurf))
        for d in (1, 2):
            for (dd, p), tag in ent.items():
                if dd == d:
                    w("%d 0 0 0 1 1 0 1 %d 0\n" % (tag, p))
    w("$EndEntities\n")
    # nodes: one block on surface entity 1
    w("$Nodes\n")
    if binary:
        out.extend(struct.pack("<QQQQ", 1, nn, 1, nn))
        out.extend(struct.pack("<iiiQ", 2, 1, 0, nn))
        out.extend(np.arange(1, nn + 1, dtype="<u8").tobytes())
        xyz = np.zeros((nn, 3), "<f8")
        xyz[:, :2] = xy
        out.extend(xyz.tobytes())
        w("\n")
    else:
        w("1 %d 1 %d\n2 1 0 %d\n" % (nn, nn, nn))
        w("".join("%d\n" % (i + 1) for i in range(nn)))
        w("".join("%.17g %.17g 0\n" % (x, y) for x, y in xy))
    w("$EndNodes\n")
    # element blocks: per (entity, type) in order of first appearance
    items = [((1, int(p)), 1, e[:2]) for e, p in zip(edges, ep)] + \
            [((2, int(p)), 3 if q else 2, c[:4] if q else c[:3]) for c, p, q in zip(cells, cp, quad)]
    order = []
    blocks = {}
    for key, t, nodes in items:
        b = (key, t)
        if b not in blocks:
            blocks[b] = []
            order.append(b)
        blocks[b].append(nodes)
    ne = len(items)
    w("$Elements\n")
    if binary:
        out.extend(struct.pack("<QQQQ", len(order), ne, 1, ne))
        num = 1
        for (key, t) in order:
            lst = np.array(blocks[(key, t)], np.int64)
            out.extend(struct.pack("<iiiQ", key[0], ent[key], t, len(lst)))
            arr = np.zeros((len(lst), 1 + lst.shape[1]), "<u8")
            arr[:, 0] = np.arange(num, num + len(lst))
            arr[:, 1:] = lst + 1
            out.extend(arr.tobytes())
            num += len(lst)
        w("\n")
    else:
        w("%d %d 1 %d\n" % (len(order), ne, ne))
        num = 1
        for (key, t) in order:
            lst = blocks[(key, t)]
            w("%d %d %d %d\n" % (key[0], ent[key], t, len(lst)))
            w("".join("%d %s\n" % (num + k, " ".join(str(v + 1) for v in nodes)) for k, nodes in enumerate(lst)))
            num += len(lst)
    w("$EndElements\n")
    with open(path, "wb") as fh:
        fh.write(bytes(out))
