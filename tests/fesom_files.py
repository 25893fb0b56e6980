"""FESOM mesh directories for the tests: the pi fixture (tests/golden/pi_mesh.npz,
made by tests/golden/make_pi_fixture.py) written back in the ASCII format the
reference reads (lib/oce_mesh.F90 read_mesh, load_edges, find_levels)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_pi():
    with np.load(os.path.join(GOLDEN, "pi_mesh.npz")) as z:
        return {k: z[k] for k in z.files}


def write_mesh_dir(path, lonlat, elem, zbar, edges, edge_tri, edgenum, elvls, nlvls, coast=None):
    """Write a FESOM mesh directory; floats as shortest round-trip decimals."""
    os.makedirs(path, exist_ok=True)
    N, M = len(lonlat), len(elem)
    coast = np.zeros(N, np.int32) if coast is None else coast
    with open(os.path.join(path, "nod2d.out"), "w") as f:
        f.write(f"{N:8d}\n")
        for i in range(N):
            f.write(f"{i + 1:8d} {float(lonlat[i, 0])!r} {float(lonlat[i, 1])!r} {int(coast[i]):8d}\n")
    with open(os.path.join(path, "elem2d.out"), "w") as f:
        f.write(f"{M:8d}\n")
        for a, b, c in elem:
            f.write(f"{a:8d} {b:8d} {c:8d}\n")
    with open(os.path.join(path, "aux3d.out"), "w") as f:
        f.write(f"{len(zbar)}\n")
        for z in zbar:
            f.write(f"{float(z)!r}\n")
    with open(os.path.join(path, "edgenum.out"), "w") as f:
        f.write(f"{int(edgenum[0]):12d}\n{int(edgenum[1]):12d}\n")
    for name, arr in (("edges.out", edges), ("edge_tri.out", edge_tri)):
        with open(os.path.join(path, name), "w") as f:
            for a, b in arr:
                f.write(f"{a:12d} {b:12d}\n")
    for name, arr in (("elvls.out", elvls), ("nlvls.out", nlvls)):
        with open(os.path.join(path, name), "w") as f:
            for v in arr:
                f.write(f"{int(v):12d}\n")
    return path


def write_pi(path):
    d = load_pi()
    return write_mesh_dir(path, d["lonlat"], d["elem"], d["zbar"], d["edges"], d["edge_tri"], d["edgenum"],
                          d["elvls"], d["nlvls"], d["coast"])
