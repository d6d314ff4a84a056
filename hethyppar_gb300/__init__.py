"""GB300-native (sm_103a) BiCGStab and CSR SpMV: the HetHypPar solver path as a C-ABI CUDA library
(libhhp_gpu.so, include/hhp_gpu.h) with a thin Python face."""
from .api import (Context, Matrix, SolveResult, bicgstab, bicgstab_backward, bicgstab_iter_bytes,  # noqa: F401
                  csr_file_write, mtx_read, plan_dump, plan_stats, reorder_color, reorder_rcm, spmv_bytes, vector_read,
                  vector_write)
from ._lib import HHPError  # noqa: F401
