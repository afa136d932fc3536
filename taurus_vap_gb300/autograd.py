"""torch.autograd.Function of the projected energy E(Z).

E(Z) is the particle-number projected energy of the state obtained from
(U0, V0) by the Thouless evolution with the real matrix Z
(cholesky_factorization + evolve_wavefunction, module_constraints.f90:497-590).
The device adjoint (tvap_energy_adjoint) forms E and dE/dZ in one call,
recomputing the per-angle densities for the gradient instead of storing
them; the forward pass keeps only dE/dZ (n x n), and the backward pass scales
it by the incoming gradient without another device call.
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
        E, G = tvap_ctx.energy_adjoint(U0, V0, np.asfortranarray(Zn), Mphip, Mphin, facpi, valence_Z, valence_N)
        # dE/dZ[i, j] = dE/dZ(i, j), in Z's layout
        ctx.save_for_backward(torch.from_numpy(np.ascontiguousarray(G)).to(Z.device, Z.dtype).reshape(Z.shape))
        return Z.new_tensor(E)

    @staticmethod
    def backward(ctx, grad_out):
        (g,) = ctx.saved_tensors
        return (grad_out * g, None, None, None, None, None, None, None, None)


def projected_energy(Z, tvap_ctx, U0, V0, Mphip, Mphin, valence_Z, valence_N, facpi=2 * math.pi):
    """E(Z) with a hand-written adjoint; Z is a real (n, n) tensor (its rows
    and columns index quasiparticles as in the reference's gradient_Zi)."""
    return ProjectedEnergy.apply(Z, tvap_ctx, U0, V0, Mphip, Mphin, valence_Z, valence_N, facpi)
