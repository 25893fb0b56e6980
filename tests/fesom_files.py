"""FESOM mesh directories for the tests: the pi fixture (tests/golden/pi_mesh.npz,
made by tests/golden/make_pi_fixture.py) written back in the ASCII format the
reference reads (lib/oce_mesh.F90 read_mesh, load_edges, find_levels), and
refinements of it (fesom2_tracer_dwarf_gb300.meshfiles)."""
import os

import numpy as np

from fesom2_tracer_dwarf_gb300.meshfiles import refine, write_fesom_dir

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_pi():
    with np.load(os.path.join(GOLDEN, "pi_mesh.npz")) as z:
        return {k: z[k] for k in z.files}


def write_mesh_dir(path, lonlat, elem, zbar, edges, edge_tri, edgenum, elvls, nlvls, coast=None):
    return write_fesom_dir(path, lonlat, elem, zbar, edges, edge_tri, edgenum, elvls, nlvls, coast)


def write_pi(path):
    d = load_pi()
    return write_mesh_dir(path, d["lonlat"], d["elem"], d["zbar"], d["edges"], d["edge_tri"], d["edgenum"],
                          d["elvls"], d["nlvls"], d["coast"])


def write_pi_refined(path, times):
    r = refine(load_pi(), times)
    return write_fesom_dir(path, r["lonlat"], r["elem"], r["zbar"], r["edges"], r["edge_tri"], r["edgenum"],
                           r["elvls"], r["nlvls"])
