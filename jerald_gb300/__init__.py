"""GB300-native (sm_103a) Lagrangian-Deep-Learning hot path of JERALD.

Modules:
  _lib           ctypes binding of libjld.so (the C ABI of include/jld.h)
  jaxpops_bind   drop-in primitive surface (ppaint, preadout, pfft, ...)
  pmesh          PMesh facade, model  JERALDModel on the primitives
  synth          seeded synthetic workloads
  build          nvcc build of libjld.so
"""
__version__ = "0.1.0"
