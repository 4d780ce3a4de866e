"""Emit the triangle quadrature-rule table used by the library and by the oracle.

The reference hard-codes its triangle rules as generated constants in
``lib/lf/quad/quad_rules_tria.cc`` (one ``HardcodedQuadRule<kTria, d>`` per
degree d).  Element matrices only agree to 1e-12 with the reference when both
integrate with *the same* points and weights (a different exact rule changes
the result by the quadrature error for non-polynomial coefficients), so the
numbers have to be alike.  This script reads every tabulated degree (1..50;
degree 3 is served by the degree-4 rule) out of the reference source and
writes them in this project's own compact layout:

    {degree, npoints, offset} index + flat {x, y, w} rows

into ``tria_rules.inc`` next to this file (library) and ``oracle/tria_rules.inc``
(oracle).  Both generated files are committed; the script is only re-run when
the table has to be regenerated (it needs the reference checkout).

usage: python lehrfempp_gb300/csrc/gen_tria_rules.py <path of the LehrFEM++ checkout>
"""
import os
import re
import sys

MAX_DEGREE = 50


def parse(src_text):
    rules = {}
    blocks = re.split(r"HardcodedQuadRule<base::RefEl::kTria\(\),\s*(\d+)>\(\)\s*\{", src_text)
    # blocks = [prefix, deg, body, deg, body, ...]
    for k in range(1, len(blocks), 2):
        deg = int(blocks[k])
        body = blocks[k + 1].split("return QuadRule")[0]
        pts = {}
        wts = {}
        for m in re.finditer(r"points\((\d), (\d+)\) = ([-0-9.eE+]+);", body):
            pts[(int(m.group(1)), int(m.group(2)))] = m.group(3)
        for m in re.finditer(r"weights\((\d+)\) = ([-0-9.eE+]+);", body):
            wts[int(m.group(1))] = m.group(2)
        n = len(wts)
        rows = [(pts[(0, q)], pts[(1, q)], wts[q]) for q in range(n)]
        rules[deg] = rows
    return rules


def emit(rules, path, guard_comment):
    lines = [
        "// Generated by lehrfempp_gb300/csrc/gen_tria_rules.py -- do not edit.",
        "// " + guard_comment,
        "// Triangle quadrature rules of degree 1..%d on the reference triangle" % MAX_DEGREE,
        "// {(0,0),(1,0),(0,1)}; weights sum to 1/2.  Degree 3 requests use the",
        "// degree-4 rule (reference: lib/lf/quad/make_quad_rule.cc:44-46).",
        "// Layout: kTriaRuleIndex[d] = {npoints, first row}; kTriaRuleRows = {x, y, w}.",
        "",
    ]
    index = []
    rows = []
    for d in range(0, MAX_DEGREE + 1):
        if d in rules:
            index.append((len(rules[d]), len(rows)))
            rows.extend(rules[d])
        else:
            index.append((0, 0))
    lines.append("static const int kTriaRuleMaxDegree = %d;" % MAX_DEGREE)
    lines.append("static const int kTriaRuleIndex[%d][2] = {" % (MAX_DEGREE + 1))
    lines += ["    {%d, %d}," % ix for ix in index]
    lines.append("};")
    lines.append("static const double kTriaRuleRows[%d][3] = {" % len(rows))
    lines += ["    {%s, %s, %s}," % r for r in rows]
    lines.append("};")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def main():
    if len(sys.argv) != 2:
        sys.exit(__doc__)
    ref = sys.argv[1]
    src = os.path.join(ref, "lib/lf/quad/quad_rules_tria.cc")
    with open(src) as f:
        rules = parse(f.read())
    rules = {d: r for d, r in rules.items() if d <= MAX_DEGREE}
    missing = [d for d in range(1, MAX_DEGREE + 1) if d != 3 and d not in rules]
    if missing:
        sys.exit("degrees not found in %s: %s" % (src, missing))
    for d, rows in rules.items():  # every point and weight parsed
        assert all(len(r) == 3 and all(r) for r in rows), d
    here = os.path.dirname(os.path.abspath(__file__))
    repo = os.path.dirname(os.path.dirname(here))
    emit(rules, os.path.join(here, "tria_rules.inc"), "library copy")
    emit(rules, os.path.join(repo, "oracle", "tria_rules.inc"), "oracle copy")
    print("degrees:", sorted(rules), "points:", {d: len(r) for d, r in sorted(rules.items())})


if __name__ == "__main__":
    main()
