"""Command-line driver, like petgem's ``python3 kernel.py -options_file petsc.opts params.yaml``
(petgem/kernel.py:15,35): the params file is the last argument ending in .yaml/.yml."""
import sys

from .pipeline import run_kernel


def main(argv=None):
    argv = list(sys.argv[1:] if argv is None else argv)
    params = [a for a in argv if a.endswith((".yaml", ".yml"))]
    if not params:
        print("usage: python -m petgem_gb300 [-options_file petsc.opts] [-ksp_type cocg] params.yaml")
        return 2
    run_kernel(params[-1], argv)
    return 0


if __name__ == "__main__":
    sys.exit(main())
