"""GB300 (sm_103a) implementation of the smartpca hot path of EIGENSOFT (DReichLab/EIG).

The product is the C ABI in include/gpupca.h + include/gpupca_run.h (libgpupca.so) and the
drop-in CLI gpusmartpca; eig_gb300.native is the ctypes caller of the same entry points.
"""
__all__ = ["native"]
