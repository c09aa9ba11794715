"""Golden vectors for the magnetotelluric (MT) right-hand side, by running
petgem's own functions in the order of its MT assembly branch.

Run in the build container, where the petgem sources are available:

    python tests/golden/make_mt_golden.py --ref <petgem checkout>   (or PETGEM_REF=<petgem checkout>)

petgem's MT right-hand side is built inside Solver.assembly
(petgem/solver.py:318-512), which needs PETSc objects; here the same
reference functions are called in the same order on numpy arrays:
computeBoundaryFaces / computeBoundaryElements / computeFacePlane
(petgem/mesh.py:128-429), compute2DGaussPoints (hvfem.py:1613),
transform2Dto3DInReferenceElement / getRealFromReference (hvfem.py:2686,
2727), eval_MT1D (mt1d.py:21-76), getNormalVector / get2DJacobDet /
getNeumannBCface / computeBasisFunctionsReferenceElement (hvfem.py:2556-2780)
and computeElementOrientation; the PETSc ADD_VALUES sums become a COO sum
in boundary-face order.  computeImpedance (postprocessing.py:619-688) is
evaluated on seeded random receiver fields.

numpy >= 2 cannot store a 1-element array into an array element, which
mt1d.py:527 does; the script hands that value over as a 0-d array.

Writes tests/golden/mt_n4.npz: a 4^3 Kuhn box over [-5000, 5000]^2 x
[-5000, 2000] m (interior nodes jittered, seed 0), air 1e-8 S/m above z = 0,
0.1 S/m down to -1000 m, 0.01 S/m below; 1 Hz; p = 1 and 2.
"""
import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from make_golden import shim  # noqa: E402
from petgem_gb300 import synthetic  # noqa: E402

MU = 4.0 * np.pi * 1e-7


def mt_model(n=4):
    lo, hi = (-5000.0, -5000.0, -5000.0), (5000.0, 5000.0, 2000.0)
    nodes, tets = synthetic.kuhn_box(n, lo, hi)
    nodes = synthetic.jitter_interior(nodes, n, 0.15, 0, lo, hi)
    cz = nodes[tets].mean(axis=1)[:, 2]
    s = np.where(cz > 0.0, 1e-8, np.where(cz > -1000.0, 0.1, 0.01))
    return nodes, tets, np.stack([s, s], axis=1)


def reference_mt_rhs(hvfem, mesh, mt1d, nodes, tets, sigma, p, freq, pols=(1, 2), rule=None):
    T = len(tets)
    elemsE, edgesN = mesh.computeEdges(tets, T)
    elemsF, facesN = mesh.computeFaces(tets, T)
    nF = facesN.shape[0]
    facesE = mesh.computeFacesEdges(elemsF, elemsE, nF, T)
    bfacesN, bFaces, nbF = mesh.computeBoundaryFaces(elemsF, facesN)
    bElems, nbE = mesh.computeBoundaryElements(elemsF, bFaces, nF)
    planes = mesh.computeFacePlane(nodes, bFaces, bfacesN)
    dofs, _, _, _, N = hvfem.computeConnectivityDOFS(elemsE, elemsF, p)
    gp, w = rule if rule is not None else hvfem.compute2DGaussPoints(2 * p)
    ng = gp.shape[0]
    omega = 2.0 * np.pi * freq
    zpts = np.zeros((nbF, ng))
    cz4, s4 = [], []
    for i in range(nbF):
        e = bElems[i]
        coord = nodes[tets[e]]
        lf = np.where(elemsF[e] == bFaces[i])[0][0]
        for j in range(ng):
            q3 = hvfem.transform2Dto3DInReferenceElement(gp[j, :], lf)
            zpts[i, j] = hvfem.getRealFromReference(q3, coord)[2]
        if planes[i] == 3:
            nf = hvfem.getFaceByLocalNodes(lf)
            cz4.append((np.sum(coord[nf], axis=0) / 3.0)[2])
            s4.append(sigma[e, 0])
    za, zb = np.max(nodes[tets][:, :, 2]), np.min(nodes[tets][:, :, 2])
    u = mt1d.eval_MT1D(za, zb, 1.0, 0.0, np.asarray(s4), np.asarray(cz4), omega, MU, int(1e6), 1, zpts)
    const = 1j * omega * MU
    bs = []
    for pol in pols:
        b = np.zeros(N, dtype=np.complex128)
        for i in range(nbF):
            e = bElems[i]
            coord = nodes[tets[e]]
            _, invJ = hvfem.computeJacobian(coord)
            eo, fo = hvfem.computeElementOrientation(elemsE[e], tets[e], edgesN[elemsE[e]], facesE[elemsF[e]])
            lf = np.where(elemsF[e] == bFaces[i])[0][0]
            nv = hvfem.getNormalVector(lf, invJ)
            nu = nv / np.linalg.norm(nv)
            det2 = hvfem.get2DJacobDet(coord, lf)
            ex, ey, ez = hvfem.getNeumannBCface(planes[i], pol, u)
            contrib = np.zeros(dofs.shape[1], dtype=np.complex128)
            for k in range(ng):
                q3 = hvfem.transform2Dto3DInReferenceElement(gp[k, :], lf)
                B = hvfem.computeBasisFunctionsReferenceElement(eo, fo, p, q3)
                Br = np.matmul(invJ, B[:, :, 0])
                ev = np.array([ex[i, k], ey[i, k], ez[i, k]], dtype=np.complex128)
                it = np.zeros(dofs.shape[1], dtype=np.complex128)
                for l in range(dofs.shape[1]):
                    it[l] = np.dot(np.cross(np.cross(nu, Br[:, l]), nu), ev)
                contrib += w[k] * it * det2
            contrib = contrib * const
            np.add.at(b, dofs[e], contrib)
        bs.append(b)
    return dict(bFaces=bFaces, bElems=bElems, planes=planes, zpts=zpts, u=u, za=za, zb=zb,
                cz4=np.asarray(cz4), s4=np.asarray(s4), b=np.stack(bs), N=N, dofs=dofs)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("PETGEM_REF"), required="PETGEM_REF" not in os.environ,
                    help="path of a petgem source checkout (default: $PETGEM_REF)")
    args = ap.parse_args()
    hvfem, mesh = shim(args.ref)
    from petgem import mt1d
    # numpy >= 2 rejects storing a 1-element array into one array element
    # (mt1d.py:527, inside the triangle reference element that eval_MT1D
    # builds); return jacobiP_vect's value for a 1-element input as a 0-d
    # array, the same number
    jac = mt1d.jacobiP_vect

    def jacobi_scalar_safe(x, a, b, n):
        r = jac(x, a, b, n)
        return np.asarray(r).reshape(()) if np.ndim(x) == 1 and np.size(x) == 1 else r
    mt1d.jacobiP_vect = jacobi_scalar_safe
    nodes, tets, sigma = mt_model()
    out = {"nodes": nodes, "tets": tets, "sigma": sigma, "freq": 1.0}
    for order in (2, 4, 6):
        gp, w = hvfem.compute2DGaussPoints(order)
        out[f"rule{order}_points"], out[f"rule{order}_weights"] = gp, w
    for p in (1, 2):
        r = reference_mt_rhs(hvfem, mesh, mt1d, nodes, tets, sigma, p, 1.0)
        for k, v in r.items():
            out[f"p{p}_{k}"] = v
        print("p", p, "boundary faces", len(r["bFaces"]), "N", r["N"], "|b|", np.linalg.norm(r["b"], axis=1))
    # computeImpedance on seeded random fields (2 polarisations x 7 receivers x 6 components)
    rng = np.random.default_rng(21)
    fields = [rng.standard_normal((7, 6)) + 1j * rng.standard_normal((7, 6)) for _ in range(2)]
    try:
        from petgem import postprocessing
        rho, phase, tip, imp = postprocessing.computeImpedance(fields, 2.0 * np.pi, MU)
        out["imp_fields"] = np.stack(fields)
        out["imp_rho"], out["imp_phase"] = np.stack(rho), np.stack(phase)
        out["imp_tipper"], out["imp_Z"] = np.stack(tip), np.stack(imp)
    except Exception as exc:     # noqa: BLE001
        print("computeImpedance not importable:", exc)
    path = os.path.join(HERE, "mt_n4.npz")
    np.savez_compressed(path, **out)
    print("wrote", path)


if __name__ == "__main__":
    main()
