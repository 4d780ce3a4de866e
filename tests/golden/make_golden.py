"""Extract the reference's own golden values for this path into a JSON fixture.

Reads (as text) the LehrFEM++ test sources and writes reference_goldens.json
next to this script.  The fixture is committed; the GPU machine never needs the
reference checkout.  Sources:

  lib/lf/assemble/test/assembly_tests.cc   10x10 ref_mat (mat_assembly_test) and
                                           36x36 ref_mat (edge_dof_static)
  lib/lf/assemble/test/coomatrix_tests.cc  fix_dof exact solution
  lib/lf/uscalfe/test/lagr_fe_tests.cc     reaction-diffusion bilinear forms
  lib/lf/fe/test/fe_tools_tests.cc         IntegrateMeshFunction integrals
  lib/lf/uscalfe/test/gfe_tests.cc         L2 norms on test mesh 3
  lib/lf/mesh/test_utils/test_meshes.cc    the nodes and triangles of test mesh 3
  lib/lf/io/test/msh_files/*.msh           copied byte for byte into msh/ (the
                                           reader's input fixtures)
  lib/lf/quad/quad_rules_tria.cc           per degree 1..50: point count, first
                                           point and weight, SHA-256 of all
                                           (x, y, w) as little-endian binary64

usage: python tests/golden/make_golden.py <path of the LehrFEM++ checkout>
"""
import hashlib
import json
import os
import re
import struct
import sys


def _matrix_after(text, marker, n):
    i = text.index(marker)
    j = text.index("<<", i)
    k = text.index(";", j)
    body = text[j + 2:k]
    vals = [float(v) for v in re.findall(r"-?\d+(?:\.\d+)?", body)]
    assert len(vals) == n * n, (marker, len(vals))
    return [vals[r * n:(r + 1) * n] for r in range(n)]


def tria_rule_digests(text):
    """Per tabulated degree of quad_rules_tria.cc: the number of points, the
    first point and weight as written, and a SHA-256 of every (x, y, w) of the
    rule in point order, each parsed as the nearest binary64 (as a C++
    compiler does) and packed little endian."""
    out = {}
    blocks = re.split(r"HardcodedQuadRule<base::RefEl::kTria\(\),\s*(\d+)>\(\)\s*\{", text)
    for k in range(1, len(blocks), 2):
        deg = int(blocks[k])
        body = blocks[k + 1].split("return QuadRule")[0]
        pts = {(int(a), int(b)): v for a, b, v in re.findall(r"points\((\d), (\d+)\) = ([-0-9.eE+]+);", body)}
        wts = {int(a): v for a, v in re.findall(r"weights\((\d+)\) = ([-0-9.eE+]+);", body)}
        n = len(wts)
        assert len(pts) == 2 * n, deg
        packed = b"".join(struct.pack("<3d", float(pts[(0, q)]), float(pts[(1, q)]), float(wts[q])) for q in range(n))
        out[str(deg)] = {"points": n, "first": [pts[(0, 0)], pts[(1, 0)], wts[0]],
                         "sha256_xyw_le": hashlib.sha256(packed).hexdigest()}
    return out


def main():
    if len(sys.argv) != 2:
        sys.exit(__doc__)
    ref = sys.argv[1]
    at = open(os.path.join(ref, "lib/lf/assemble/test/assembly_tests.cc")).read()
    ct = open(os.path.join(ref, "lib/lf/assemble/test/coomatrix_tests.cc")).read()
    lt = open(os.path.join(ref, "lib/lf/uscalfe/test/lagr_fe_tests.cc")).read()

    ft = open(os.path.join(ref, "lib/lf/fe/test/fe_tools_tests.cc")).read()
    gt = open(os.path.join(ref, "lib/lf/uscalfe/test/gfe_tests.cc")).read()
    tm = open(os.path.join(ref, "lib/lf/mesh/test_utils/test_meshes.cc")).read()

    # test mesh 3: the `case 3:` block of GenerateHybrid2DTestMesh
    blk = tm[tm.index("case 3: {"):]
    blk = blk[:blk.index("break;")]
    pts = [[float(a), float(b)] for a, b in
           re.findall(r"AddPoint\(coord_t\(\{(-?[\d.]+) \* scale, (-?[\d.]+) \* scale\}\)\)", blk)]
    tris = [[int(a), int(b), int(c)] for a, b, c in
            re.findall(r"kTria\(\), std::array<size_type, 3>\{\{(\d+), (\d+), (\d+)\}\}", blk)]
    assert len(pts) == 13 and len(tris) == 15, (len(pts), len(tris))

    def expect(text, var):
        # EXPECT_FLOAT_EQ(var, <a> / <b>) or (var, <a>.) with base::kPi allowed
        mm = re.search(r"EXPECT_FLOAT_EQ\(" + re.escape(var) + r", ([^;]+)\);", text)
        expr = mm.group(1).strip()
        val = expr.replace("base::kPi", "3.141592653589793")
        assert re.fullmatch(r"[\d.\s/*3141592653589793]+", val), expr
        return expr, float(eval(val))  # arithmetic on literals only (checked above)

    fe_kat = {}
    for var in ("intScalar", "intVec[0]", "intVec[1]", "intMatrixDyn(0, 0)", "intMatrixDyn(0, 1)",
                "intMatrixDyn(0, 2)", "intMatrixDyn(1, 0)", "intMatrixDyn(1, 1)", "intMatrixDyn(1, 2)"):
        expr, val = expect(ft, var)
        fe_kat[var] = {"expr": expr, "value": val}
    m1 = re.search(r"EXPECT_NEAR\(norm, (5\.\d+), (1E-4)\)", gt)
    m2 = re.search(r"EXPECT_NEAR\(norm, (7\.\d+), (1E-4)\)", gt)

    ref10 = _matrix_after(at, "Eigen::MatrixXd ref_mat(10, 10);", 10)
    ref36 = _matrix_after(at, "Eigen::MatrixXd ref_mat(36, 36);", 36)
    m = re.search(r"exact << (1, 1, -1[^;]+);", ct)
    exact = [float(v) for v in m.group(1).split(",")]

    def near(pattern):
        mm = re.search(pattern, lt)
        return mm.group(1)

    kat = {
        "O1_tensor_deg4": {"value_expr": near(r"EXPECT_NEAR\(product, (7911\. / 8\.)"), "value": 7911.0 / 8.0},
        "O2_deg6": {"value_expr": near(r"EXPECT_NEAR\(product, (81\.)"), "value": 81.0},
        "O3_deg8": {"value_expr": near(r"EXPECT_NEAR\(product, (1996731 / 280\.)"), "value": 1996731.0 / 280.0},
        "tolerance": 1.0e-2,
    }
    out = {
        "source": "LehrFEM++ test sources (read as text by tests/golden/make_golden.py)",
        "mat_assembly_test_ref10": {
            "file": "lib/lf/assemble/test/assembly_tests.cc:256-262",
            "layout": "{Point:1}; compare dense(i,j) == ref[ent(i)][ent(j)], ent = node index of dof",
            "matrix": ref10,
        },
        "edge_dof_static_ref36": {
            "file": "lib/lf/assemble/test/assembly_tests.cc:394-455",
            "layout": "{Segment:2}; compare dense(i,j) == ref[i][j]",
            "matrix": ref36,
        },
        "fix_dof_exact": {
            "file": "lib/lf/assemble/test/coomatrix_tests.cc:118-120",
            "N": 10, "fixed": [[2, -1.0], [4, -2.0], [8, -3.0]], "tolerance": 1.0e-12,
            "solution": exact,
        },
        "reaction_diffusion_kat": dict(kat, file="lib/lf/uscalfe/test/lagr_fe_tests.cc:807-883"),
        "test_mesh_3": {
            "file": "lib/lf/mesh/test_utils/test_meshes.cc:160-224",
            "nodes": pts, "triangles": tris,
        },
        "integrate_mesh_function_kat": {
            "file": "lib/lf/fe/test/fe_tools_tests.cc:44-85",
            "mesh": "test mesh 0, scale 1",
            "integrals": fe_kat,
            "tolerance": "EXPECT_FLOAT_EQ (4 ulp in float)",
        },
        "gfe_norm_kat": {
            "file": "lib/lf/uscalfe/test/gfe_tests.cc:27-45, 141-160",
            "mesh": "test mesh 3",
            "l2norm_x_1my": {"value": float(m1.group(1)), "tolerance": float(m1.group(2))},
            "l2norm_vf_y_mx": {"value": float(m2.group(1)), "tolerance": float(m2.group(2))},
        },
    }
    # the Gmsh reader's test inputs, copied unchanged
    src = os.path.join(ref, "lib/lf/io/test/msh_files")
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "msh")
    os.makedirs(dst, exist_ok=True)
    copied = []
    for name in sorted(os.listdir(src)):
        if name.endswith(".msh"):
            with open(os.path.join(src, name), "rb") as fi, open(os.path.join(dst, name), "wb") as fo:
                fo.write(fi.read())
            copied.append(name)
    qt = open(os.path.join(ref, "lib/lf/quad/quad_rules_tria.cc")).read()
    out["tria_rules"] = {"file": "lib/lf/quad/quad_rules_tria.cc (dispatch make_quad_rule.cc:38-137)",
                         "degrees": tria_rule_digests(qt)}
    out["gmsh_fixtures"] = {"dir": "lib/lf/io/test/msh_files", "files": copied,
                            "tests": "lib/lf/io/test/gmsh_reader_tests.cc"}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_goldens.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main()
