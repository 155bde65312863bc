"""Writes gmsh 2.2 ASCII files for the mesh-input tests (the format the reference ships)."""


def write_gmsh22(path, coords, cells, with_boundary=True):
    dim = coords.shape[1]
    lines = ["$MeshFormat", "2.2 0 8", "$EndMeshFormat", "$Nodes", str(coords.shape[0])]
    for i, x in enumerate(coords):
        xyz = list(x) + [0.0] * (3 - dim)
        lines.append("%d %.17g %.17g %.17g" % (i + 1, *xyz))
    lines.append("$EndNodes")
    elems = []
    if with_boundary:
        elems.append((15, [1]))  # a point entity, as gmsh writes for corner vertices
    etype = 2 if dim == 2 else 4
    for c in cells:
        elems.append((etype, [int(v) + 1 for v in c]))
    lines += ["$Elements", str(len(elems))]
    for k, (t, nodes) in enumerate(elems):
        lines.append("%d %d 2 7 6 %s" % (k + 1, t, " ".join(str(v) for v in nodes)))
    lines.append("$EndElements")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
