"""jyulb drop-in for one GB300: the jyulb isothermal D3Q19 solver API with the
time-step loop running as hand-written sm_103a CUDA kernels.

Modules mirror the reference package (jyulb/__init__.py):
``isothermal`` (Solver), ``D3Q19`` (lattice tables and moment maps), ``bcs``
(Zou-He boundary maps), ``defs`` (enumerations) and ``flow_field`` (analytic
profiles).
"""
__all__ = ['isothermal', 'D3Q19', 'bcs', 'defs', 'flow_field']
