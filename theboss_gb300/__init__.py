"""GB300-native (sm_103a) implementation of theboss's permanent hot path.

Drop-in classes (same names and API as theboss):
  permanent_calculators    Ryser / Chin-Huh / Glynn-Gray / Classic calculators + factory
  submatrices_calculators  BSCCRyser / BSCCCH all-minors calculators
  simulation_strategies    generalized Clifford & Clifford samplers (B version, uniform
                           losses, network losses) on the batched GPU sampler
"""
__version__ = "0.1.0"
