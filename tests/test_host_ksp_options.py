"""The PETSc options a petgem options file gives the solve (petgem/solver.py:
584-594) map to this build's solver and preconditioner, and the ones it does
not serve are rejected with ValueError (petgem would exit)."""
import pytest

from petgem_gb300.pipeline import ksp_settings


@pytest.mark.parametrize("opts, nord, want", [
    ({}, 2, ("gmres", "jacobi")),
    ({"ksp_type": "cocg"}, 1, ("cocg", "jacobi")),
    ({"pc_type": "bjacobi"}, 3, ("gmres", "block")),
    ({"pc_type": "sor"}, 6, ("gmres", "block")),
    ({"pc_type": "none"}, 2, ("gmres", "block")),
    ({"pc_type": "hypre"}, 1, ("gmres", "grad")),
    ({"pc_type": "hypre", "pc_hypre_type": "ams", "ksp_type": "cocg"}, 3, ("cocg", "grad")),
])
def test_ksp_settings_accepts(opts, nord, want):
    assert ksp_settings(opts, nord) == want


@pytest.mark.parametrize("opts, nord, msg", [
    ({"ksp_type": "bicg"}, 2, "-ksp_type"),
    ({"pc_type": "ilu"}, 2, "-pc_type"),
    ({"pc_type": "hypre", "pc_hypre_type": "boomeramg"}, 2, "pc_hypre_type"),
    ({"pc_type": "hypre"}, 4, "nord <= 3"),
])
def test_ksp_settings_rejects(opts, nord, msg):
    with pytest.raises(ValueError, match=msg):
        ksp_settings(opts, nord)
