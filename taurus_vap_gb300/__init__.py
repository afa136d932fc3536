"""GB300 (sm_103a) implementation of TAURUS_vap's PNVAP gradient hot path.

Modules
  model    model-space setup (basis, interaction, operators, seeds), host C++
  native   C ABI binding of the device library (include/tvap.h)
  vap      host mirror of the gradient loop over the device entry points
  autograd torch.autograd.Function of the projected energy E(Z)
"""

__all__ = ["model", "native", "vap"]
