"""mglc_gb300 -- the MGLC lattice-Boltzmann time step on one GB300 GPU.

The product is ``libmglc_gb300.so`` (C-ABI declared in include/mglc.h, CUDA
kernels for sm_103a under csrc/).  This package builds it and offers a thin
Python host API that mirrors the reference's routines.
"""
from .capi import FORMS, MglcError, lib  # noqa: F401
from .cavity import (BuoyancyCavity, LidDrivenCavity, LidDrivenCavity2D, NuReMonitor,  # noqa: F401
                     ParticleFlow, ParticleFlow2D, ShearFlow2D)
from .serve import SolveServer  # noqa: F401

__all__ = ["LidDrivenCavity", "LidDrivenCavity2D", "BuoyancyCavity", "ParticleFlow",
           "ParticleFlow2D", "ShearFlow2D", "NuReMonitor", "SolveServer", "MglcError", "FORMS",
           "lib"]
