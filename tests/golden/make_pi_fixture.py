#!/usr/bin/env python3
"""Make tests/golden/pi_mesh.npz from the reference's pi mesh directory.

The pi mesh (3140 nodes, 5839 elements, 8986 edges, 48 levels, closed coasts,
ragged bottom) is the one unstructured mesh the reference ships
(tests/data/pi/, loaded by python/test_mesh_from_files.py). The fixture keeps
what a one-partition read uses: node longitudes/latitudes (degrees) and coast
flags, elements, levels, edges, edge_tri, edge counts and the element and
node bottom levels, parsed from the ASCII files as the reference's
list-directed reads do. tests/fesom_files.py writes it back as a FESOM mesh
directory.

    python tests/golden/make_pi_fixture.py [PI_DIR]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.oracle import read_fesom_dir  # noqa: E402


def main():
    src = sys.argv[1] if len(sys.argv) > 1 else "/root/reference/tests/data/pi"
    d = read_fesom_dir(src)
    out = os.path.join(HERE, "pi_mesh.npz")
    np.savez_compressed(out, lonlat=d["lonlat"], coast=d["coast"].astype(np.int8), elem=d["elem"],
                        zbar=d["zbar"], edges=d["edges"], edge_tri=d["edge_tri"],
                        edgenum=np.array([d["edge2D"], d["edge2D_in"]], np.int32),
                        elvls=d["elvls"].astype(np.int8), nlvls=d["nlvls"].astype(np.int8))
    print(out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    main()
