"""torch.autograd.Function of the projected energy E(Z).

E(Z) is the particle-number projected energy of the state obtained from
(U0, V0) by the Thouless evolution with the real matrix Z
(cholesky_factorization + evolve_wavefunction, module_constraints.f90:497-590).
The backward pass calls the device adjoint (tvap_energy_adjoint), which
recomputes the per-angle densities instead of keeping them from the forward
pass: only Z is saved for backward.
"""

from __future__ import annotations

import math

import numpy as np
import torch


class ProjectedEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, Z, tvap_ctx, U0, V0, Mphip, Mphin, valence_Z, valence_N, facpi=2 * math.pi):
        n = tvap_ctx.n
        Zn = Z.detach().to("cpu", torch.float64).numpy().reshape(n, n)
        E, _ = tvap_ctx.energy_adjoint(U0, V0, np.asfortranarray(Zn), Mphip, Mphin, facpi, valence_Z, valence_N)
        ctx.save_for_backward(Z.detach())
        ctx.args = (tvap_ctx, U0, V0, Mphip, Mphin, valence_Z, valence_N, facpi)
        return Z.new_tensor(E)

    @staticmethod
    def backward(ctx, grad_out):
        (Z,) = ctx.saved_tensors
        tvap_ctx, U0, V0, Mphip, Mphin, valence_Z, valence_N, facpi = ctx.args
        n = tvap_ctx.n
        Zn = Z.to("cpu", torch.float64).numpy().reshape(n, n)
        _, G = tvap_ctx.energy_adjoint(U0, V0, np.asfortranarray(Zn), Mphip, Mphin, facpi, valence_Z, valence_N)
        g = torch.from_numpy(np.ascontiguousarray(G)).to(Z.device, Z.dtype)
        return (grad_out * g, None, None, None, None, None, None, None, None)


def projected_energy(Z, tvap_ctx, U0, V0, Mphip, Mphin, valence_Z, valence_N, facpi=2 * math.pi):
    """E(Z) with a hand-written adjoint; Z is a real (n, n) tensor (its rows
    and columns index quasiparticles as in the reference's gradient_Zi)."""
    return ProjectedEnergy.apply(Z, tvap_ctx, U0, V0, Mphip, Mphin, valence_Z, valence_N, facpi)
