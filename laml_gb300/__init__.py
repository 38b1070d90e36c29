"""laml_gb300: a GB300 (sm_103a) engine for LAML's PMM likelihood / EM path.

Compute runs in hand-written CUDA kernels behind the C ABI of
``laml_gb300/_lib/liblaml_gb300.so`` (declared in ``include/laml_gb300.h``);
this package holds the host-side mirror of the reference interface.
"""
__version__ = "0.1.0"
