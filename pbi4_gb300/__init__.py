"""GB300 (sm_103a) implementation of the PBI4 estimator hot path.

Modules:
  powerI4, bispectrumI4  drop-ins for the reference's f2py modules (host numpy in/out)
  estimator              device-resident plan (positions in HBM -> P(k), B(k))
  pbi4                   IO / DENSITIES / MEASUREMENTS with the reference's method names
  serve                  continuous-batching request loop over resident plans
  synthetic              seeded synthetic particle boxes
The CUDA work is done by libpbi4gpu.so (include/pbi4gpu.h); there is no CPU path.
"""
__version__ = "0.1.0"
