"""Host mirror of TAURUS_vap's gradient loop (taurus_vap.f90:77-123) over the
device entry points.

Device (libtvap_gpu.so):  project_wavefunction + calculate_projected_H20,
calculate_gradient, cholesky_factorization + evolve_wavefunction.
Host (NumPy):  the constraint algebra -- set_operator_qpbasis, the Lagrange
multipliers and the adjust_constraints Newton loop
(module_constraints.f90:270-484, module_operators.f90:49-97) -- which works on
a handful of n x n real matrices per iteration.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .native import Context, TvapError, gradient_parameters


def set_operator_qpbasis(part: str, U, V, A):
    """module_operators.f90:49-97 (U, V, A real, column-major n x n)."""
    if part == "f11":
        fac, A2, A3 = 1.0, U.T @ A @ U, V.T @ A.T @ V
    elif part == "g11":
        fac, A2, A3 = 1.0, U.T @ A @ V, V.T @ A @ U
    elif part == "f20":
        fac, A2, A3 = -1.0, U.T @ A @ V, V.T @ A.T @ U
    else:  # g20
        fac, A2, A3 = -1.0, U.T @ A @ U, V.T @ A @ V
    A1 = A2 - A3
    return 0.5 * (A1 + fac * A1.T)


def expectval_obo(rho, B):
    """<B> = Tr(B rho), the proton and neutron halves summed
    (calculate_expectval_obo, module_operators.f90); formed as the sum of
    B_ik rho_ki, without the n^3 product."""
    return float(np.sum(B * rho.T))


def expectval_pair(kappa, B):
    """Tr(B kappa^T) (calculate_expectval_pair) as the sum of B_ik kappa_ik."""
    return float(np.sum(B * kappa))


@dataclass
class Constraints:
    """Constraint operators in the HO basis (constraint_HO, vectorised as in
    the reference: entry k of operator j is element (i, j) with k = i + j n)."""

    ops: list = field(default_factory=list)  # n*n vectors
    values: list = field(default_factory=list)
    npair: int = 0
    eps: float = 1e-6

    @property
    def dim(self) -> int:
        return len(self.values)


class VAP:
    """State and loop of one PNVAP minimisation."""

    def __init__(self, ctx: Context, U0, V0, Mphip, Mphin, valence_Z, valence_N, eta, mu, gradient_eps=1e-4,
                 constraints: Constraints | None = None, facpi=2 * np.pi, factor_delta=1.0, mode=0,
                 gradient_type=0):
        self.ctx = ctx
        self.n = ctx.n
        self.U0 = np.asfortranarray(U0, dtype=np.float64)
        self.V0 = np.asfortranarray(V0, dtype=np.float64)
        self.Mp, self.Mn, self.facpi = Mphip, Mphin, facpi
        self.Z, self.N = valence_Z, valence_N
        self.eta, self.mu, self.geps = eta, mu, gradient_eps
        self.cons = constraints or Constraints()
        self.factor_delta = factor_delta
        self.mode = mode
        self.gradient_type = gradient_type
        self.step_sizes = (eta, mu)
        n = self.n
        self.Zi = np.zeros(n * n)
        self.Zim1 = np.zeros(n * n)
        self.lam0 = np.zeros(self.cons.dim)
        self.lam1 = np.zeros(self.cons.dim)
        self.C20 = np.zeros((self.cons.dim, n * n))
        self._ops = [np.reshape(o, (n, n), order="F") for o in self.cons.ops]
        self.control_NZ = [0] * 5
        self.history = []
        self.adjust_steps = 0  # evolutions made by the last adjust_constraints (100: the targets were not met)
        self._c20_of = None  # the (U, V) arrays C20 belongs to (replaced, not modified in place)

    def _part(self, i):
        return "f20" if i < self.cons.dim - self.cons.npair else "g20"

    def update_constraints_qpbasis(self, U, V):
        for i, A in enumerate(self._ops):
            self.C20[i] = set_operator_qpbasis(self._part(i), U, V, A).reshape(-1, order="F")
        self._c20_of = (U, V)

    def _c20_current(self):
        return self._c20_of is not None and self._c20_of[0] is self.U0 and self._c20_of[1] is self.V0

    def lagrange_multipliers(self, H20v):
        c = self.cons.dim
        if c == 0:
            return
        # Tr(C_i C_j^T) and Tr(H C_i^T) are dot products of the vectorised
        # matrices (module_constraints.f90:413-484)
        A = self.C20 @ self.C20.T
        B = self.C20 @ np.asarray(H20v, dtype=np.float64).reshape(-1)
        try:
            self.lam1 = np.linalg.solve(A, B)
        except np.linalg.LinAlgError:
            self.lam1 = self.lam0.copy()
        self.lam0 = self.lam1.copy()

    def adjust_constraints(self):
        """module_constraints.f90:270-373.  On a device context the whole
        Newton loop runs there (tvap_adjust_constraints); otherwise the loop
        runs here around the context's evolution."""
        c = self.cons.dim
        if hasattr(self.ctx, "adjust_constraints"):
            U1, V1, Zi, C20, self.adjust_steps = self.ctx.adjust_constraints(
                self.U0, self.V0, self.Zi, np.stack(self.cons.ops) if c else None, list(self.cons.values),
                cpair=self.cons.npair, eps=self.cons.eps)
            self.Zi = Zi
            self.U0, self.V0 = np.asfortranarray(U1), np.asfortranarray(V1)
            if c:
                # the device loop ends with C20 of the state it returns
                self.C20 = C20
                self._c20_of = (self.U0, self.V0)
            return
        U1, V1 = self.U0, self.V0
        self.adjust_steps = 0
        for _ in range(100):
            U1, V1 = self.ctx.evolve(self.U0, self.V0, self.Zi)
            self.adjust_steps += 1
            rho = V1 @ V1.T
            kap = V1 @ U1.T
            expec = np.array([expectval_obo(rho, A) if i < c - self.cons.npair else expectval_pair(kap, A)
                              for i, A in enumerate(self._ops)])
            B = np.asarray(self.cons.values, dtype=np.float64) - expec if c else np.zeros(0)
            ia = int(np.sum(np.abs(B) > self.cons.eps))
            self.update_constraints_qpbasis(U1, V1)
            if ia == 0:
                break
            A = self.C20 @ self.C20.T  # Tr(C_i^T C_j)
            B = np.linalg.solve(A, B)
            self.Zi = self.Zi + B @ self.C20
        self.U0, self.V0 = np.asfortranarray(U1), np.asfortranarray(V1)
        if self.adjust_steps:
            self._c20_of = (self.U0, self.V0)  # the loop's last update was of (U1, V1)

    def iterate(self):
        """One gradient iteration.  Returns (status, info) with status 0
        continue, 1 converged; info = gradient norm, E, <Z>, Var Z, <N>, Var N."""
        # C20 of the current state: the constraint loop that produced it
        # leaves it behind (module_constraints.f90:381-397 on the same state)
        if not self._c20_current():
            self.update_constraints_qpbasis(self.U0, self.V0)
        pnp, H20v = self.ctx.project(self.U0, self.V0, self.Mp, self.Mn, self.facpi, self.Z, self.N,
                                     self.factor_delta, mode=self.mode)
        self.lagrange_multipliers(H20v)
        eta, mu = self.eta, self.mu
        if self.gradient_type > 0:
            # diagonalize_hsp_and_H11(0), then the step sizes of
            # calculate_gradient (taurus_vap.f90:93; module_gradient.f90:86-119)
            c = self.cons.dim
            eh, e11, info = self.ctx.diagonalize_hsp_and_H11(
                self.U0, self.V0, self.lam1 if c else None, np.stack(self.cons.ops) if c else None,
                cpair=self.cons.npair, factor_delta=self.factor_delta)
            eta, mu = gradient_parameters(self.gradient_type, eh, e11, info, self.eta, self.mu)
        self.step_sizes = (eta, mu)
        self.Zi, gnorm = self.ctx.calculate_gradient(H20v, self.lam1 if self.cons.dim else None,
                                                     self.C20 if self.cons.dim else None, self.Zim1, eta, mu)
        over = pnp.c("over")
        ener = (pnp.c("ener") / over).real
        prot = (pnp.c("prot") / over).real
        neut = (pnp.c("neut") / over).real
        prot2 = abs((pnp.c("prot2") / over).real - prot**2)
        neut2 = abs((pnp.c("neut2") / over).real - neut**2)
        info = (gnorm, ener, prot, prot2, neut, neut2)
        self.history.append(info)
        self.control_NZ = [1 if (abs(prot - self.Z) > 0.5 or abs(neut - self.N) > 0.5) else 0] + self.control_NZ[:4]
        if sum(self.control_NZ) >= 3:
            raise TvapError(18, "print_iteration")
        if gnorm <= self.geps:
            return 1, info
        self.adjust_constraints()
        self.Zim1 = self.Zi.copy()
        return 0, info

    def run(self, iter_max=3000, initial_adjust=True):
        if initial_adjust:
            self.adjust_constraints()
        info = None
        for it in range(1, iter_max + 1):
            st, info = self.iterate()
            if st == 1:
                return it, info
        return iter_max, info


def particle_number_ops(n: int):
    """partnumb_Z, partnumb_N (module_particlenumber.f90:30-57), vectorised."""
    Qz = np.zeros(n * n)
    Qn = np.zeros(n * n)
    for i in range(n // 2):
        Qz[i * n + i] = 1.0
        j = i + n // 2
        Qn[j * n + j] = 1.0
    return Qz, Qn
