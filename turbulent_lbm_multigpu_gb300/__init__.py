"""GB300-native D3Q19 lattice Boltzmann hot path (CUDA sm_103a behind a C ABI).

The compute path is liblbm_gb300.so (include/lbm_gb300.h, built by `build`);
`capi` binds every entry point for Python.  The reference's C++ interfaces
(CLbmSolver / CController / CManager / CComm / CDomain, the conf.xml reader,
the VTK writer) are the headers in include/lbm_gb300/, and the command-line
driver lbm_gb300 uses them.  `experiments` measures the precision, batching
and serving patterns, `scaling` runs decomposition sweeps.
"""
__all__ = ["build", "capi", "experiments", "scaling"]
