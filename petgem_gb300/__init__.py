"""petgem_gb300: GB300-native (sm_103a) forward-modelling hot path of petgem.

H(curl) elemental matrices -> deterministic CSR assembly -> complex Krylov
solve -> receiver interpolation, as hand-written CUDA behind a C ABI
(``include/petgem_gb300.h``), with petgem's entry points mirrored on top.
"""
__version__ = "0.1.0"
