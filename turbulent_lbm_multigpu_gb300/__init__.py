"""GB300-native D3Q19 lattice Boltzmann hot path (CUDA sm_103a behind a C ABI).

The compute path is liblbm_gb300.so (include/lbm_gb300.h); `capi` binds it,
`solver` mirrors the reference's CLbmSolver / CController / CManager / CComm /
CDomain interfaces over it, `config` reads the reference's conf.xml schema.
"""
__all__ = ["capi", "solver", "config", "build"]
