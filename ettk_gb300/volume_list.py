"""The reference's 33-column volume-list text format
(nbfWedgedSubImage3D::writeHeader/serialize/unserialize/read/write, inc/em/nbfWedgedSubImage3D.h:343-600).

Row: number, lwedge, uwedge, posX..Z, geomX..Z, normalX..Z, matrix[0..15], magnification[0..2],
cutOffset, filename — tab separated, numbers printed like a default C++ ostream (6 significant
digits, %g style).
"""
import numpy as np

HEADER = (["number", "lwedge", "uwedge", "posX", "posY", "posZ", "geomX", "geomY", "geomZ",
           "normalX", "normalY", "normalZ"] + ["matrix[%d]" % i for i in range(16)] +
          ["magnification[0]", "magnification[1]", "magnification[2]", "cutOffset", "filename"])


def _fmt(x):
    """Default std::ostream formatting of a float/double (precision 6, general notation)."""
    s = "%g" % float(x)
    return s


def write(path, rows):
    """rows: list of dicts with keys lwedge, uwedge, position, geometry, normal, matrix,
    magnification, cut_offset, filename."""
    out = ["\t".join(HEADER)]
    for i, r in enumerate(rows):
        vals = [r["lwedge"], r["uwedge"], *r["position"], *r.get("geometry", (0, 0, 0)), *r.get("normal", (0, 0, 0)),
                *np.asarray(r.get("matrix", np.eye(4)), np.float64).reshape(16),
                *r.get("magnification", (1, 1, 1)), r.get("cut_offset", 0.0)]
        out.append(str(i + 1) + "\t" + "\t".join(_fmt(v) for v in vals) + "\t" + str(r.get("filename", "NA")))
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


def read(path):
    with open(path) as f:
        tok = f.read().split()
    tok = tok[33:]
    rows = []
    i = 0
    while i + 33 <= len(tok):
        t = tok[i:i + 33]
        try:
            v = [float(x) for x in t[1:32]]
        except ValueError:
            break
        rows.append({
            "lwedge": v[0], "uwedge": v[1], "position": tuple(v[2:5]), "geometry": tuple(v[5:8]),
            "normal": tuple(v[8:11]), "matrix": np.array(v[11:27]).reshape(4, 4),
            "magnification": tuple(v[27:30]), "cut_offset": v[30], "filename": t[32],
        })
        i += 33
    return rows


def write_alignments(path, D):
    """Result rows as getDistances writes them: D[i, :, 0] per pair (distance, [scale], [overlap], matrix)."""
    D = np.asarray(D)
    with open(path, "w") as f:
        for i in range(D.shape[0]):
            f.write("\t".join(_fmt(x) for x in D[i, :, 0]) + "\n")
