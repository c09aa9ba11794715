"""Copy petgem's PETSc-binary test system (tests/data/matrix-A.dat,
vector-b.dat, vector-x.dat: the system petgem's tests/test_petsc.py solves
with KSP, x being the zero initial guess) and its h5py-written receiver file
(tests/data/receiver_pos.h5) into tests/golden/ under petgem_* names,
unchanged.

    python tests/golden/copy_petsc_fixtures.py --ref <petgem checkout>   (or PETGEM_REF=<petgem checkout>)
"""
import argparse
import os
import shutil

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("PETGEM_REF"), required="PETGEM_REF" not in os.environ,
                    help="path of a petgem source checkout (default: $PETGEM_REF)")
    args = ap.parse_args()
    for name in ("matrix-A.dat", "vector-b.dat", "vector-x.dat", "receiver_pos.h5"):
        src = os.path.join(args.ref, "tests", "data", name)
        dst = os.path.join(HERE, "petgem_" + name)
        shutil.copyfile(src, dst)
        print("copied", src, "->", dst, os.path.getsize(dst), "bytes")


if __name__ == "__main__":
    main()
