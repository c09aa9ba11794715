"""Generate golden vectors by running petgem's own code (the reference).

Run in the build container, where the petgem sources are available:

    python tests/golden/make_golden.py --ref <petgem checkout>   (or PETGEM_REF=<petgem checkout>)

petgem needs petsc4py, mpi4py, PyYAML, colorama, singleton_decorator, h5py
and meshio at import time; none of them is used by the functions called
here, so they are replaced by empty stub modules.  numpy >= 1.24 dropped the
``np.int``/``np.float``/``np.complex`` aliases the reference uses; they are
restored.  PETSc's ``Mat.setValues(ADD_VALUES)`` assembly is restated with a
scipy COO sum in element order (petgem/solver.py:191-235), and its point
location with scipy's ``Delaunay.find_simplex`` exactly as the reference
does (petgem/preprocessing.py:414-425).

Outputs (tests/golden/):
  test_mesh.npz         points / tets / physical tags of tests/data/test_mesh.msh
  topology.json         counts, first rows and sha256 of the reference's
                        topology + DOF maps + PEC DOFs on test_mesh and on
                        a 3^3 Kuhn box
  basis.npz             shape3DETet values and curls, p = 1..6
  elemental.npz         computeElementalMatrices on sampled elements, p = 1..3
  system_n2.npz         assembled A (before PEC), PEC DOFs, source b, for a
                        2^3 Kuhn box, p = 1, 2, 3
  pipeline_n3.npz       direct solution and fieldInterpolator receiver fields
                        on a 3^3 Kuhn box, p = 2
"""
import argparse
import hashlib
import json
import os
import sys
import types

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def shim(ref):
    np.int = int
    np.float = float
    np.complex = complex
    for name in ["colorama", "singleton_decorator", "yaml", "mpi4py", "petsc4py", "h5py", "meshio"]:
        sys.modules.setdefault(name, types.ModuleType(name))
    sys.modules["colorama"].Fore = types.SimpleNamespace(**{k: "" for k in (
        "BLACK BLUE CYAN GREEN LIGHTBLACK_EX LIGHTBLUE_EX LIGHTCYAN_EX LIGHTGREEN_EX LIGHTMAGENTA_EX "
        "LIGHTRED_EX LIGHTWHITE_EX LIGHTYELLOW_EX MAGENTA RED WHITE YELLOW").split()})
    sys.modules["colorama"].Style = types.SimpleNamespace(RESET_ALL="", BRIGHT="")
    sys.modules["colorama"].init = lambda *a, **k: None
    sys.modules["singleton_decorator"].singleton = lambda c: c
    mpi = types.ModuleType("mpi4py.MPI")
    sys.modules["mpi4py.MPI"] = mpi
    sys.modules["mpi4py"].MPI = mpi
    pm = types.ModuleType("petsc4py.PETSc")
    pm.IntType = np.int64
    sys.modules["petsc4py.PETSc"] = pm
    sys.modules["petsc4py"].PETSc = pm
    sys.path.insert(0, ref)
    from petgem import hvfem, mesh  # noqa: E402
    return hvfem, mesh


def sha(a):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.int64))
    return hashlib.sha256(a.tobytes() + str(a.shape).encode()).hexdigest()


def ref_topology(mesh, hvfem, tets, ps=(1, 2, 3)):
    T = len(tets)
    elemsE, edgesN = mesh.computeEdges(tets, T)
    elemsF, facesN = mesh.computeFaces(tets, T)
    facesE = mesh.computeFacesEdges(elemsF, elemsE, facesN.shape[0], T)
    bfacesN, bFaces, nbF = mesh.computeBoundaryFaces(elemsF, facesN)
    bEdges = mesh.computeBoundaryEdges(edgesN, bfacesN)
    out = {"nElems": int(T), "nEdges": int(edgesN.shape[0]), "nFaces": int(facesN.shape[0]),
           "elemsE0": elemsE[0].tolist(), "elemsF0": elemsF[0].tolist(),
           "sha": {"elemsE": sha(elemsE), "elemsF": sha(elemsF), "edgesNodes": sha(edgesN),
                   "facesN": sha(facesN), "facesE": sha(facesE), "bFaces": sha(bFaces), "bEdges": sha(bEdges)},
           "nBoundaryFaces": int(nbF), "nBoundaryEdges": int(len(bEdges))}
    eo = np.zeros((T, 6), np.int64)
    fo = np.zeros((T, 4), np.int64)
    for e in range(T):
        a, b = hvfem.computeElementOrientation(elemsE[e], tets[e], edgesN[elemsE[e]], facesE[elemsF[e]])
        eo[e], fo[e] = a, b
    out["sha"]["eo"] = sha(eo)
    out["sha"]["fo"] = sha(fo)
    out["n_orientation_tuples"] = int(len({tuple(r) for r in np.concatenate([eo, fo], 1)}))
    for p in ps:
        dofs, de, df, dv, nd = hvfem.computeConnectivityDOFS(elemsE, elemsF, p)
        _, bnd = mesh.computeBoundaries(dofs, de, df, bEdges, bFaces, p)
        out[f"p{p}"] = {"total_num_dofs": int(nd), "dofs_sha": sha(dofs), "boundary_sha": sha(bnd),
                        "n_boundary": int(len(bnd)), "dofs0": dofs[0].tolist()}
    return out, (elemsE, edgesN, elemsF, facesN, facesE, eo, fo, bFaces, bEdges)


def locate_ref(points, tets, pos):
    from scipy.spatial import Delaunay
    tri = Delaunay(points)
    tri.simplices = tets.astype(np.int32)
    return tri.find_simplex(np.atleast_2d(pos), bruteforce=True, tol=1.0e-12)


def assemble_ref(hvfem, points, tets, topo, sigma, p, freq):
    elemsE, edgesN, elemsF, facesN, facesE, eo, fo, bFaces, bEdges = topo
    dofs, de, df, dv, ndof = hvfem.computeConnectivityDOFS(elemsE, elemsF, p)
    omega = 2.0 * np.pi * freq
    mu = 4.0 * np.pi * 1e-7
    Const = np.sqrt(-1.0 + 0.j) * omega * mu
    nd = dofs.shape[1]
    rows, cols, vals = [], [], []
    for e in range(len(tets)):
        J, iJ = hvfem.computeJacobian(points[tets[e]])
        M, K = hvfem.computeElementalMatrices(eo[e], fo[e], J, iJ, p, sigma[e])
        Ae = K - Const * M
        rows.append(np.repeat(dofs[e], nd))
        cols.append(np.tile(dofs[e], nd))
        vals.append(Ae.ravel())
    A = sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(ndof, ndof)).tocsr()
    A.sum_duplicates()
    A.sort_indices()
    return A, dofs, de, df


def source_ref(hvfem, points, tets, topo, dofs, p, src, ndof):
    """petgem/solver.py:247-316 with the source element of preprocessing.py:414-425."""
    elemsE, edgesN, elemsF, facesN, facesE, eo, fo, bFaces, bEdges = topo
    pos = np.asarray(src["position"], dtype=float)
    se = int(locate_ref(points, tets, pos)[0])
    rot = hvfem.computeSourceVectorRotation(src["azimuth"], src["dip"])
    IL = src["current"] * src["length"]
    field = rot[0] * np.array([IL, 0, 0.]) + rot[1] * np.array([0, IL, 0.]) + rot[2] * np.array([0, 0, IL])
    coord = points[tets[se]]
    J, iJ = hvfem.computeJacobian(coord)
    a, b = hvfem.computeElementOrientation(elemsE[se], tets[se], edgesN[elemsE[se]], facesE[elemsF[se]])
    xi = hvfem.tetrahedronXYZToXiEtaZeta(coord, pos)
    B, _ = hvfem.computeBasisFunctions(a, b, J, iJ, p, xi)
    Const = np.sqrt(-1.0 + 0.j) * 2.0 * np.pi * src["frequency"] * 4.0 * np.pi * 1e-7
    rhs = np.matmul(field, B[:, :, 0]) * Const
    bvec = np.zeros(ndof, complex)
    np.add.at(bvec, dofs[se], rhs)
    return bvec, se


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("PETGEM_REF"), required="PETGEM_REF" not in os.environ,
                    help="path of a petgem source checkout (default: $PETGEM_REF)")
    args = ap.parse_args()
    hvfem, mesh = shim(args.ref)
    from petgem_gb300 import gmsh, synthetic
    rng = np.random.default_rng(20261203)

    # ---- test mesh input fixture + reference topology
    m = gmsh.read(os.path.join(args.ref, "tests", "data", "test_mesh.msh"))
    np.savez_compressed(os.path.join(HERE, "test_mesh.npz"), points=m.points, tets=m.tets, physical=m.physical)
    topo_json = {}
    topo_json["test_mesh"], tm_topo = ref_topology(mesh, hvfem, m.tets)
    kn, kt = synthetic.kuhn_box(3)
    topo_json["kuhn3"], _ = ref_topology(mesh, hvfem, kt)

    # ---- basis values, p = 1..6
    bas = {}
    for p in range(1, 7):
        eo = rng.integers(0, 2, (4, 6))
        fo = rng.integers(0, 6, (4, 4))
        X = rng.dirichlet(np.ones(4), 4)[:, 1:]
        N = np.zeros((4, 4, 3, p * (p + 2) * (p + 3) // 2))
        C = np.zeros_like(N)
        for a in range(4):
            for i in range(4):
                nr, S, Cr = hvfem.shape3DETet(X[i], np.ones(11, int) * p, eo[a], fo[a])
                N[a, i] = S[:, :nr]
                C[a, i] = Cr[:, :nr]
        bas.update({f"p{p}_eo": eo, f"p{p}_fo": fo, f"p{p}_X": X, f"p{p}_N": N, f"p{p}_C": C})
    np.savez_compressed(os.path.join(HERE, "basis.npz"), **bas)

    # ---- elemental matrices: test-mesh elements (own orientation) + random tets/orientations
    el = {}
    elemsE, edgesN, elemsF, facesN, facesE, eo_tm, fo_tm, _, _ = tm_topo
    for p, k in ((1, 40), (2, 32), (3, 10)):
        half = k // 2
        idx = rng.choice(len(m.tets), half, replace=False)
        coords = [m.points[m.tets[e]] for e in idx]
        eos = [eo_tm[e] for e in idx]
        fos = [fo_tm[e] for e in idx]
        for _ in range(k - half):
            c = rng.normal(size=(4, 3)) * rng.uniform(1, 300)
            if np.linalg.det(c[1:] - c[0]) < 0 and rng.random() < 0.7:
                c[[1, 2]] = c[[2, 1]]      # mostly positive, some negative orientation
            coords.append(c)
            eos.append(rng.integers(0, 2, 6))
            fos.append(rng.integers(0, 6, 4))
        sig = 10.0 ** rng.uniform(-2, 0.6, (k, 2))
        Ms, Ks = [], []
        for c, a, b, s in zip(coords, eos, fos, sig):
            J, iJ = hvfem.computeJacobian(c)
            M, K = hvfem.computeElementalMatrices(a, b, J, iJ, p, s)
            Ms.append(M)
            Ks.append(K)
        el.update({f"p{p}_coords": np.array(coords), f"p{p}_eo": np.array(eos), f"p{p}_fo": np.array(fos),
                   f"p{p}_sigma": sig, f"p{p}_M": np.array(Ms), f"p{p}_K": np.array(Ks)})
    np.savez_compressed(os.path.join(HERE, "elemental.npz"), **el)

    # ---- small assembled systems (2^3 Kuhn box)
    sysd = {}
    pts, tets = synthetic.kuhn_box(2)
    _, topo = ref_topology(mesh, hvfem, tets)
    cen = pts[tets].mean(1)
    s = np.where(cen[:, 2] > 0, 3.3, 1.0)
    sigma = np.stack([s, s * 0.5], 1)      # anisotropic on purpose
    src = {"frequency": 1.5, "position": [120.0, -40.0, 50.0], "azimuth": 30.0, "dip": 10.0,
           "current": 2.0, "length": 0.5}
    for p in (1, 2, 3):
        A, dofs, de, df = assemble_ref(hvfem, pts, tets, topo, sigma, p, src["frequency"])
        _, bnd = mesh.computeBoundaries(dofs, de, df, topo[8], topo[7], p)
        b, se = source_ref(hvfem, pts, tets, topo, dofs, p, src, A.shape[0])
        sysd.update({f"p{p}_data": A.data, f"p{p}_indices": A.indices, f"p{p}_indptr": A.indptr,
                     f"p{p}_bnd": bnd, f"p{p}_b": b, f"p{p}_src_elem": se})
    sysd.update({"points": pts, "tets": tets, "sigma": sigma, "src": json.dumps(src)})
    np.savez_compressed(os.path.join(HERE, "system_n2.npz"), **sysd)

    # ---- pipeline: direct solve + reference receiver interpolation (3^3 box, p=2)
    import petgem.postprocessing as post
    pts, tets = synthetic.kuhn_box(3)
    _, topo = ref_topology(mesh, hvfem, tets)
    cen = pts[tets].mean(1)
    s = np.where(cen[:, 2] > 0, 3.3, 1.0)
    sigma = np.stack([s, s], 1)
    src = {"frequency": 1.0, "position": [0.0, 0.0, 50.0], "azimuth": 0.0, "dip": 0.0, "current": 1.0,
           "length": 1.0}
    p = 2
    A, dofs, de, df = assemble_ref(hvfem, pts, tets, topo, sigma, p, src["frequency"])
    _, bnd = mesh.computeBoundaries(dofs, de, df, topo[8], topo[7], p)
    b, se = source_ref(hvfem, pts, tets, topo, dofs, p, src, A.shape[0])
    keep = np.ones(A.shape[0])
    keep[bnd] = 0
    Dk = sp.diags(keep)
    Ap = (Dk @ A @ Dk + sp.diags(1 - keep)).tocsc()
    bp = b.copy()
    bp[bnd] = 0
    x = spla.spsolve(Ap, bp)
    rx = np.stack([np.linspace(-800, 800, 7), np.linspace(-300, 300, 7), np.zeros(7)], 1)
    rx = np.vstack([rx, [[5000.0, 0.0, 0.0]]])        # one receiver outside the mesh

    class Vec:
        def getValues(self, idx):
            return x[np.asarray(idx)]

    setup = types.SimpleNamespace(model={"mode": "csem", "csem": {"source": src}}, run={"nord": p})
    post.Print = types.SimpleNamespace(master=lambda *a, **k: None)
    # fieldInterpolator adds basis[0, j] (a shape-(1,) array for its single
    # point) into a complex scalar slot, which numpy >= 2 refuses; hand it the
    # single-point basis with the point axis dropped (same values).
    post.computeBasisFunctions = lambda *a: tuple(v[:, :, 0] for v in hvfem.computeBasisFunctions(*a))
    F = post.fieldInterpolator(Vec(), pts, tets, topo[0], topo[1], topo[2], topo[4], dofs, rx, setup)
    np.savez_compressed(os.path.join(HERE, "pipeline_n3.npz"), points=pts, tets=tets, sigma=sigma,
                        src=json.dumps(src), bnd=bnd, b=bp, x=x, receivers=rx, fields=F, src_elem=se)
    with open(os.path.join(HERE, "topology.json"), "w") as f:
        json.dump(topo_json, f, indent=1, sort_keys=True)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
