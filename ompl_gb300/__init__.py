"""GB300 (sm_103a) implementation of OMPL's data-parallel inner loop: state sampling, state validity,
discrete motion checking and nearest-neighbour queries, behind OMPL's plugin interfaces.

The compute path is libgbompl.so (C ABI in include/gbompl.h); this package is its Python host
mirror. Importing the package does not load the library; the first call does, and fails loudly
when the library is missing (there is no CPU fallback).
"""
__all__ = ["base", "capi", "workloads"]
