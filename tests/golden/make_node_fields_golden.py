"""Golden nodal E/H fields from petgem's own VTK postprocessing loop.

Run in the build container, where the petgem sources are available:

    python tests/golden/make_node_fields_golden.py --ref <petgem checkout>   (or PETGEM_REF=<petgem checkout>)

petgem computes the nodal fields it writes to VTK inside
``Postprocessing.run`` (petgem/postprocessing.py:172-261), a loop that also
needs PETSc vectors, meshio and h5py.  This script runs the body of that loop
unchanged in order: per element ``computeJacobian``,
``computeElementOrientation``, the centroid pull of the vertices by 0.9999,
``tetrahedronXYZToXiEtaZeta``, ``computeBasisFunctions``, the per-vertex
sums over the element's DOFs (l inner, as the reference's loops), the
accumulation into the nodes in element order, the division by the number of
elements sharing each node (``np.count_nonzero(elemsN == i)``) and H /= i
omega mu.  The solution vector stands in for ``x[i].getValues``.

Output: tests/golden/node_fields.npz
  n3_*   3^3 Kuhn box, p = 2, the direct solution of pipeline_n3.npz
  tm_*   the first 300 elements of petgem's tests/data/test_mesh.msh
         (renumbered nodes), p = 1 and p = 3, a seeded complex vector
"""
import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)


def reference_node_fields(hvfem, points, tets, topo, dofs, x, p, frequency):
    """petgem/postprocessing.py:172-261 for one polarisation."""
    elemsE, edgesN, elemsF, facesN, facesE = topo[:5]
    nNodes, nElems = points.shape[0], tets.shape[0]
    omega = 2.0 * np.pi * frequency
    mu = 4.0 * np.pi * 1e-7
    Const = np.sqrt(-1.0 + 0.j) * omega * mu
    scaledCoord = np.zeros((4, 3), dtype=float)
    local = np.zeros((4, 6), dtype=complex)
    fields = np.zeros((nNodes, 6), dtype=complex)
    nd = dofs.shape[1]
    for j in range(nElems):
        nodesEle = tets[j, :]
        coordEle = points[nodesEle, :]
        edgesEle = elemsE[j, :]
        edgesFace = facesE[elemsF[j, :], :]
        jac, ijac = hvfem.computeJacobian(coordEle)
        eo, fo = hvfem.computeElementOrientation(edgesEle, nodesEle, edgesN[edgesEle, :], edgesFace)
        centroid = np.sum(coordEle, axis=0) / 4.0
        for c in range(3):
            scaledCoord[:, c] = centroid[c] + (coordEle[:, c] - centroid[c]) * 0.9999
        xi = hvfem.tetrahedronXYZToXiEtaZeta(coordEle, scaledCoord)
        basis, curl = hvfem.computeBasisFunctions(eo, fo, jac, ijac, p, xi)
        xe = x[dofs[j, :]]
        re, im = np.real(xe), np.imag(xe)
        for k in range(4):
            for l in range(nd):
                for c in range(3):
                    local[k, c] += re[l] * basis[c, l, k] + 1j * im[l] * basis[c, l, k]
                    local[k, 3 + c] += re[l] * curl[c, l, k] + 1j * im[l] * curl[c, l, k]
        fields[nodesEle, :] += local
        local[:] = 0.0
    shared = np.array([np.count_nonzero(tets == i) for i in range(nNodes)], dtype=float)
    for c in range(6):
        fields[:, c] /= shared
    for c in range(3, 6):
        fields[:, c] /= Const
    return fields


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("PETGEM_REF"), required="PETGEM_REF" not in os.environ,
                    help="path of a petgem source checkout (default: $PETGEM_REF)")
    args = ap.parse_args()
    import make_golden as mg
    hvfem, mesh = mg.shim(args.ref)
    from petgem_gb300 import gmsh
    out = {}
    g = np.load(os.path.join(HERE, "pipeline_n3.npz"))
    pts, tets, x = g["points"], g["tets"], g["x"]
    _, topo = mg.ref_topology(mesh, hvfem, tets, ps=(2,))
    dofs, _, _, _, _ = hvfem.computeConnectivityDOFS(topo[0], topo[2], 2)
    out.update({"n3_points": pts, "n3_tets": tets, "n3_x": x, "n3_p": 2, "n3_frequency": 1.0,
                "n3_fields": reference_node_fields(hvfem, pts, tets, topo, dofs, x, 2, 1.0)})
    m = gmsh.read(os.path.join(args.ref, "tests", "data", "test_mesh.msh"))
    sel = m.tets[:300]
    used = np.unique(sel)
    remap = -np.ones(len(m.points), dtype=np.int64)
    remap[used] = np.arange(len(used))
    pts2, tets2 = m.points[used], remap[sel]
    _, topo2 = mg.ref_topology(mesh, hvfem, tets2, ps=(1, 3))
    rng = np.random.default_rng(42)
    out.update({"tm_points": pts2, "tm_tets": tets2, "tm_frequency": 2.0})
    for p in (1, 3):
        dofs, _, _, _, nd = hvfem.computeConnectivityDOFS(topo2[0], topo2[2], p)
        xr = rng.standard_normal(nd) + 1j * rng.standard_normal(nd)
        out[f"tm_p{p}_x"] = xr
        out[f"tm_p{p}_fields"] = reference_node_fields(hvfem, pts2, tets2, topo2, dofs, xr, p, 2.0)
    np.savez_compressed(os.path.join(HERE, "node_fields.npz"), **out)
    print("wrote", os.path.join(HERE, "node_fields.npz"))


if __name__ == "__main__":
    main()
