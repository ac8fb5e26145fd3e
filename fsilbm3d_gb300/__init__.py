"""GB300 (sm_103a) implementation of FSILBM3D's per-time-step hot path.

The compute lives in libfsi_gpu.so (CUDA kernels behind the C-ABI of
include/fsi_gpu.h). This package is the host layer above that ABI: it loads
the library, mirrors the reference's block and body interfaces
(FluidDomain.f90 LBMBlock, Solidbody.f90 VirtualBody) and the per-step
orchestration of LBMBlockComm.f90:279-338.

Modules: abi (the ctypes binding: Block, Pair, Mlp, Batch), bodies (rigid
plate markers, Solidbody.f90:604-646), inflow (the fluid sections of the
reference's inFlow.dat), d3q19 (lattice tables), build (the in-tree nvcc
build).

There is no CPU fallback: if the CUDA library cannot be loaded, or no GPU is
present, every compute call raises.
"""
from .abi import (FsiError, Block, Pair, Mlp, Batch, lib, load_library, library_path, PREC_F64, PREC_F64_FAST,
                  PREC_F32, PREC_F16, PREC_BF16, PREC_F64_DW, PRECISIONS, device_info, FSI_OK, FSI_E_ARG, FSI_E_CUDA,
                  FSI_E_NAN, FSI_E_TIMEOUT, FSI_E_BC, FSI_E_RANGE, FSI_E_STATE, continue_write, continue_read)
from .d3q19 import E, OPPO, WT, Q

__all__ = ["FsiError", "Block", "Pair", "Mlp", "Batch", "lib", "load_library", "library_path", "PREC_F64", "PREC_F64_FAST",
           "PREC_F32", "PREC_F16", "PREC_BF16", "PREC_F64_DW", "PRECISIONS", "device_info", "E", "OPPO", "WT", "Q",
           "FSI_OK", "FSI_E_ARG", "FSI_E_CUDA", "FSI_E_NAN", "FSI_E_TIMEOUT", "FSI_E_BC", "FSI_E_RANGE", "FSI_E_STATE",
           "continue_write", "continue_read"]
