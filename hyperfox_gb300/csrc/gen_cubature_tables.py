"""Generate ``cubature_tables.inc`` from the Witherden-Vincent rule files.

The simplex cubature rules used by HyperFox (``src/element/Cubature.cpp``) are
the published symmetric rules of F. D. Witherden and P. E. Vincent ("On the
identification of symmetric quadrature rules for finite element methods",
2015).  HyperFox ships them as text files (``ressources/CubatureRules/
expanded/{tri,tet}/<strength>-<npts>.txt``) whose point order equals the order
hard-coded in ``Cubature.cpp`` (e.g. ``Cubature.cpp:310-320`` for the 3-point
triangle rule, ``Cubature.cpp:1966-1990`` for the 4-point tet rule).

The integration points must be the same points, in the same order, as the
reference's: the source term is sampled at the physical integration points,
so a different rule of the same strength would change the right-hand side.

The rule chosen for a polynomial order follows ``Cubature.cpp`` (``nIPMap``):
it is the rule with the fewest points whose strength is at least the order.

Usage (needs the HyperFox source tree, only run when refreshing the table)::

    python gen_cubature_tables.py <hyperfox-root> > cubature_tables.inc
"""
import os
import sys

# (dim, order) -> file stem, as selected by Cubature.cpp's nIPMap for simplices
# (TestCubature.cpp:43-44 lists the resulting point counts).
RULES = {
    (2, 1): "1-1", (2, 2): "2-3", (2, 3): "4-6", (2, 4): "4-6", (2, 5): "5-7",
    (2, 6): "6-12", (2, 7): "7-15", (2, 8): "8-16", (2, 9): "9-19", (2, 10): "10-25",
    (3, 1): "1-1", (3, 2): "2-4", (3, 3): "3-8", (3, 4): "5-14", (3, 5): "5-14",
    (3, 6): "6-24", (3, 7): "7-35", (3, 8): "8-46", (3, 9): "9-59", (3, 10): "10-81",
}


def main(root):
    base = os.path.join(root, "ressources", "CubatureRules", "expanded")
    out = []
    out.append("// Generated by gen_cubature_tables.py from the Witherden-Vincent rule files")
    out.append("// shipped with HyperFox. Each row: coordinates then weight. Do not edit.")
    out.append("// Point order equals HyperFox src/element/Cubature.cpp.")
    stems = {}
    for (dim, order), stem in sorted(RULES.items()):
        stems.setdefault((dim, stem), []).append(order)
    for (dim, stem), orders in sorted(stems.items()):
        sub = "tri" if dim == 2 else "tet"
        path = os.path.join(base, sub, stem + ".txt")
        rows = []
        with open(path) as fh:
            for line in fh:
                parts = line.split()
                if not parts:
                    continue
                vals = [float(v) for v in parts]
                assert len(vals) == dim + 1, (path, line)
                rows.append(vals)
        npts = int(stem.split("-")[1])
        assert len(rows) == npts, (path, len(rows))
        name = "kCub%dD_%s" % (dim, stem.replace("-", "_"))
        out.append("static const double %s[%d] = {" % (name, npts * (dim + 1)))
        for r in rows:
            out.append("  " + ", ".join(repr(v) for v in r) + ",")
        out.append("};")
    out.append("struct CubatureRuleEntry { int dim; int order; int npts; const double* data; };")
    out.append("static const CubatureRuleEntry kCubatureRules[] = {")
    for (dim, order), stem in sorted(RULES.items()):
        npts = int(stem.split("-")[1])
        out.append("  {%d, %d, %d, kCub%dD_%s}," % (dim, order, npts, dim, stem.replace("-", "_")))
    out.append("};")
    out.append("static const int kNumCubatureRules = %d;" % len(RULES))
    print("\n".join(out))


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("HYPERFOX_REFERENCE")
    if not root:
        sys.exit("usage: gen_cubature_tables.py <HyperFox source tree> (or set HYPERFOX_REFERENCE)")
    main(root)
