"""GB300 (sm_103a) spectral-element time step with the SPECFEM3D GPU C ABI.

Modules: ``build`` (nvcc build of the in-tree library), ``abi`` (ctypes
binding), ``meshgen`` (block mesh databases), ``configs`` (workloads),
``solver`` (host driver of the time loop), ``attenuation`` (N_SLS=3 constants).
"""
__version__ = "0.1.0"
