"""GB300-native (sm_103a) solve phase of fhhos4: FCG(1)/PCG preconditioned by a geometric
multigrid V-cycle on the statically condensed HHO face system.

The compute path is libfhg (CUDA kernels + C ABI, ``include/fhg.h``), built in-tree by
:mod:`fhhos4_gb300.build`; :mod:`fhhos4_gb300.solver` mirrors the reference's solver classes and
:mod:`fhhos4_gb300.hho` produces the multigrid hierarchy on the host.
"""
