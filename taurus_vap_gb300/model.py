"""Model-space setup: HO basis, two-body interaction, operators, seeds.

Thin ctypes layer over ``libtvap_setup.so`` (``include/tvap_setup.h``), which
restates the reference's initialisation (set_basis, set_hamiltonian,
set_multipoles).  The arrays it returns are exactly the module globals the
hot path reads in the reference (``hamil_abcd``, ``hamil_H2``,
``hamil_trperm``, ``hamil_H1``, ``HOsp_*``), with the reference's values
(1-based indices) and column-major complex matrices.
"""

from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field

import numpy as np

from . import _build

_lib = None


def _setup_lib():
    global _lib
    if _lib is None:
        path = _build.SETUP_LIB
        if not os.path.exists(path):
            _build.build_setup()
        L = ctypes.CDLL(path)
        vp = ctypes.c_void_p
        L.tvs_load_antoine.restype = vp
        L.tvs_load_antoine.argtypes = [ctypes.c_char_p, ctypes.c_double, ctypes.c_double]
        L.tvs_synthetic.restype = vp
        L.tvs_synthetic.argtypes = [
            ctypes.c_int, vp, vp, vp, ctypes.c_double, ctypes.c_double, ctypes.c_double,
            ctypes.c_double, ctypes.c_double, ctypes.c_ulonglong, ctypes.c_double, ctypes.c_double,
        ]
        L.tvs_error.restype = ctypes.c_char_p
        L.tvs_error.argtypes = [vp]
        L.tvs_free.argtypes = [vp]
        for name in ("tvs_dim", "tvs_nshells"):
            getattr(L, name).argtypes = [vp]
            getattr(L, name).restype = ctypes.c_int
        L.tvs_nelements.argtypes = [vp]
        L.tvs_nelements.restype = ctypes.c_longlong
        for name in ("tvs_hw", "tvs_oscillator_length"):
            getattr(L, name).argtypes = [vp]
            getattr(L, name).restype = ctypes.c_double
        L.tvs_get_basis.argtypes = [vp] * 8
        L.tvs_get_shells.argtypes = [vp, vp]
        L.tvs_get_hamiltonian.argtypes = [vp] * 6
        L.tvs_multipoles.argtypes = [vp, vp]
        L.tvs_coeff_betalm.argtypes = [vp, vp]
        L.tvs_observable_ops.argtypes = [vp, vp, vp]
        L.tvs_write_red.argtypes = [vp, ctypes.c_char_p]
        L.tvs_write_red.restype = ctypes.c_int
        L.tvs_read_red.argtypes = [vp, ctypes.c_char_p]
        L.tvs_read_red.restype = ctypes.c_int
        L.tvs_clebsch.restype = ctypes.c_double
        L.tvs_clebsch.argtypes = [ctypes.c_int] * 6
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


@dataclass
class Basis:
    """Spherical HO single-particle basis (module_basis.f90:73-245)."""

    shells: np.ndarray  # HOsh_na labels (ANTOINE: 1000 n + 100 l + 2 j)
    sp_n: np.ndarray
    sp_l: np.ndarray
    sp_2j: np.ndarray
    sp_2mj: np.ndarray
    sp_2mt: np.ndarray
    sp_sh: np.ndarray  # 1-based shell index
    sp_tr: np.ndarray  # 1-based time-reversal partner
    hw: float
    b: float

    @property
    def n(self) -> int:
        return int(self.sp_n.size)


@dataclass
class Hamiltonian:
    """m-scheme Hamiltonian arrays (module_hamiltonian.f90:53-58)."""

    H0: complex
    H1: np.ndarray  # complex128 (n, n), Fortran order
    abcd: np.ndarray  # int16 [4 S], 1-based
    h2: np.ndarray  # float32 [S]
    trperm: np.ndarray  # int8 [S]

    @property
    def S(self) -> int:
        return int(self.h2.size)


@dataclass
class Model:
    basis: Basis
    ham: Hamiltonian
    valence_Z: float
    valence_N: float
    core_Z: float = 0.0
    core_N: float = 0.0
    _handle: int | None = field(default=None, repr=False)

    @property
    def n(self) -> int:
        return self.basis.n

    def multipoles(self) -> np.ndarray:
        """Q_lm operators, shape (4 lambda, 2 isospin, 5 |mu|, n*n) in the
        reference's vectorised layout (set_multipoles)."""
        n = self.n
        q = np.zeros((4, 2, 5, n * n), dtype=np.float64)
        _setup_lib().tvs_multipoles(self._handle, _ptr(q))
        return q

    def observable_operators(self) -> dict:
        """The operators whose projected expectation values print_results
        reports (project_wavefunction with iopt = 1, module_projection.f90:
        298-354), as complex n x n matrices used the way the reference uses
        its vectorised tables: ``obo`` (one-body: Jx, i Jy, Jz, spin-orbit,
        Q_lm for l = 1..4 and m = 0..l with both isospins, r^2), ``sq`` (the
        pairs (O, O^2) of <J_i^2>: (Jx, Jx^2), (-i Jy, -Jy^2), (Jz, Jz^2)),
        ``parity`` ((-1)^l per state) and ``shell_size`` (2j + 1 per shell,
        for the occupation numbers)."""
        n = self.n
        ops = np.zeros((9, n * n), dtype=np.float64)
        par = np.zeros(n, dtype=np.int32)
        _setup_lib().tvs_observable_ops(self._handle, _ptr(ops), _ptr(par))
        mat = lambda v: np.reshape(v, (n, n), order="F").astype(np.complex128)
        q = self.multipoles()
        names, obo = ["Jx", "Jy", "Jz", "so"], [mat(ops[0]), 1j * mat(ops[1]), mat(ops[2]), mat(ops[6])]
        for lam in range(1, 5):
            for mu in range(lam + 1):
                names.append(f"Q{lam}{mu}")
                obo.append(mat(q[lam - 1, 0, mu] + q[lam - 1, 1, mu]))
        names.append("r2")
        obo.append(mat(ops[7] + ops[8]))
        sq = [(mat(ops[0]), mat(ops[3])), (-1j * mat(ops[1]), -mat(ops[4])), (mat(ops[2]), mat(ops[5]))]
        return {"obo_names": names, "obo": np.array(obo), "sq_names": ["Jx2", "Jy2", "Jz2"], "sq": np.array(sq),
                "parity": par, "shell_size": np.array([s % 100 + 1 for s in self.basis.shells], dtype=np.int32)}

    def coeff_betalm(self) -> np.ndarray:
        c = np.zeros((4, 4), dtype=np.float64)
        _setup_lib().tvs_coeff_betalm(self._handle, _ptr(c))
        return c

    def write_red(self, path: str) -> None:
        rc = _setup_lib().tvs_write_red(self._handle, path.encode())
        if rc:
            raise IOError(f"cannot write {path}")

    def __del__(self):
        if self._handle is not None and _lib is not None:
            _lib.tvs_free(self._handle)
            self._handle = None


def _extract(handle, valence_Z, valence_N, core_Z=0.0, core_N=0.0) -> Model:
    L = _setup_lib()
    err = L.tvs_error(handle)
    if err:
        L.tvs_free(handle)
        raise ValueError(err.decode())
    n = L.tvs_dim(handle)
    nsh = L.tvs_nshells(handle)
    arrs = [np.zeros(n, dtype=np.int32) for _ in range(7)]
    L.tvs_get_basis(handle, *[_ptr(a) for a in arrs])
    shells = np.zeros(nsh, dtype=np.int32)
    L.tvs_get_shells(handle, _ptr(shells))
    basis = Basis(shells, *arrs, hw=L.tvs_hw(handle), b=L.tvs_oscillator_length(handle))
    S = L.tvs_nelements(handle)
    H0 = np.zeros(2)
    H1 = np.zeros((n, n), dtype=np.complex128, order="F")
    abcd = np.zeros(4 * S, dtype=np.int16)
    h2 = np.zeros(S, dtype=np.float32)
    tr = np.zeros(S, dtype=np.int8)
    L.tvs_get_hamiltonian(handle, _ptr(H0), _ptr(H1), _ptr(abcd), _ptr(h2), _ptr(tr))
    ham = Hamiltonian(complex(H0[0], H0[1]), H1, abcd, h2, tr)
    return Model(basis, ham, valence_Z, valence_N, core_Z, core_N, _handle=handle)


def load_antoine(path: str, valence_Z: float, valence_N: float) -> Model:
    """Basis + interaction from an ANTOINE (hamil_type 1/2) ``.sho`` file."""
    h = _setup_lib().tvs_load_antoine(path.encode(), float(valence_Z), float(valence_N))
    return _extract(h, valence_Z, valence_N)


# Shells up to major quantum number e = 2n + l, ordered by e then by the
# ANTOINE label of the shell (n, l, j).
def shells_up_to(emax: int) -> list[int]:
    out = []
    for e in range(emax + 1):
        for l in range(e, -1, -2):
            nr = (e - l) // 2
            for twoj in ((2 * l + 1, 2 * l - 1) if l > 0 else (1,)):
                out.append(1000 * nr + 100 * l + twoj)
    return out


SD_SHELLS = [205, 1001, 203]
SD_SPE = [-3.9, -3.2, 2.1]


def synthetic(shells, spe, hw: float, valence_Z: float, valence_N: float, seed: int,
              core_Z: float = 0.0, core_N: float = 0.0, scale: float = 1.0, damp: float = 0.0) -> Model:
    """Seeded rotation- and isospin-invariant JT interaction on ``shells``."""
    sh = np.asarray(shells, dtype=np.int32)
    sp = np.asarray(spe, dtype=np.float64)
    h = _setup_lib().tvs_synthetic(len(sh), _ptr(sh), _ptr(sp), _ptr(sp), float(hw), float(core_Z),
                                   float(core_N), float(valence_Z), float(valence_N), int(seed),
                                   float(scale), float(damp))
    return _extract(h, valence_Z, valence_N, core_Z, core_N)


def sd_model(seed: int = 1, valence_Z: float = 4, valence_N: float = 4) -> Model:
    """sd valence space (0d5/2, 1s1/2, 0d3/2; n = 24), spe -3.9/-3.2/+2.1 MeV."""
    return synthetic(SD_SHELLS, SD_SPE, hw=0.0, valence_Z=valence_Z, valence_N=valence_N, seed=seed,
                     core_Z=8, core_N=8)


def noncore_model(emax: int, seed: int = 1, hw: float = 20.0, valence_Z: float = 8,
                  valence_N: float = 8) -> Model:
    """No-core SHO basis up to emax with V ~ N(0,1) exp(-(e_a+e_b+e_c+e_d)/8);
    single-particle energies hw (e + 3/2) / 2 (the HO kinetic expectation)."""
    shells = shells_up_to(emax)
    spe = [hw * ((2 * (s // 1000) + (s % 1000) // 100) + 1.5) / 2.0 for s in shells]
    return synthetic(shells, spe, hw=hw, valence_Z=valence_Z, valence_N=valence_N, seed=seed,
                     scale=1.0, damp=8.0)


# ---------------------------------------------------------------------------
# Wave functions
# ---------------------------------------------------------------------------

def read_wavefunction_text(path: str, n: int):
    """initial_wf.txt text format (module_wavefunctions.f90:568-655)."""
    vals = [float(x.replace("D", "E").replace("d", "E")) for x in open(path).read().split()]
    nsh = int(vals[0])
    k = 1 + nsh + 1
    U = np.array(vals[k:k + n * n]).reshape(n, n).T.copy(order="F")
    V = np.array(vals[k + n * n:k + 2 * n * n]).reshape(n, n).T.copy(order="F")
    return U, V


def random_bogoliubov(basis: Basis, valence_Z: float, valence_N: float, seed: int,
                      block: int = 0, mix_isospin: bool = True, zero_pair: int | None = None,
                      v2: np.ndarray | None = None):
    """Random real Bogoliubov seed in the spirit of seed_type 0
    (module_wavefunctions.f90:134-204,250-354,442-547): BCS occupations drawn
    until the particle numbers are reached, then two random orthogonal
    transformations D (left) and C (right).  ``block`` > 0 exchanges the
    columns of U and V for that quasiparticle (block_quasiparticle,
    :959-984).  With ``mix_isospin`` false, D and C act on the proton and the
    neutron states separately, so that the state has good proton and neutron
    number parities (the states the half-circle projection, proj_facpi = pi,
    is meant for).  ``zero_pair`` = k zeroes the columns of U and V of the
    k-th canonical pair and leaves out the right transformation C, so that
    the two columns stay zero: the result is not a Bogoliubov transformation
    (U_phi has two zero rows at every gauge angle), while rho and kappa are
    those of a valid state with that pair empty -- an input for the
    singular-U_phi failure path.  ``v2`` (n/2 values: the proton pairs in the
    basis order, then the neutron pairs) replaces the drawn occupations, e.g.
    for nearly closed shells.  The random stream is NumPy's, not the Fortran
    processor's."""
    rng = np.random.default_rng(seed)
    n = basis.n
    v2c = np.zeros(n // 2)

    def fill(lo, hi, target):
        num = -1.0
        while num < 0.98 * target:
            num = 0.0
            for i in range(lo, hi):
                v2c[i] = min(0.99, v2c[i] + rng.random())
                num += 2.0 * v2c[i]
        if num > target and target > 0:
            v2c[lo:hi] /= num / target

    if v2 is None:
        fill(0, n // 4, valence_Z)
        fill(n // 4, n // 2, valence_N)
    else:
        v2c[:] = np.asarray(v2, dtype=np.float64)
    U = np.zeros((n, n))
    V = np.zeros((n, n))
    ipos = 0
    k = 0
    pairs = []
    shells2j = [s % 100 for s in basis.shells]
    for j in shells2j:
        for m in range(1, (j + 1) // 2 + 1):
            p1 = ipos + m - 1
            p2 = ipos + j + 2 - m - 1
            p3, p4 = p1 + n // 2, p2 + n // 2
            U[p1, p1] = np.sqrt(1 - v2c[k])
            U[p2, p2] = U[p1, p1]
            U[p3, p3] = np.sqrt(1 - v2c[k + n // 4])
            U[p4, p4] = U[p3, p3]
            V[p1, p2] = np.sqrt(v2c[k])
            V[p2, p1] = -V[p1, p2]
            V[p3, p4] = np.sqrt(v2c[k + n // 4])
            V[p4, p3] = -V[p3, p4]
            pairs += [(p1, p2), (p3, p4)]
            k += 1
        ipos += j + 1
    if zero_pair is not None:
        cols = list(pairs[zero_pair])
        U[:, cols] = 0.0
        V[:, cols] = 0.0

    def unitary(m=n):
        B = rng.random((m, m))
        B = np.triu(B) + np.triu(B, 1).T
        return np.linalg.eigh(B)[1]

    def transform():
        if mix_isospin:
            return unitary()
        T = np.zeros((n, n))
        T[: n // 2, : n // 2] = unitary(n // 2)
        T[n // 2:, n // 2:] = unitary(n // 2)
        return T

    D = transform()
    U, V = D @ U, D @ V
    C = transform()
    if zero_pair is None:
        U, V = U @ C, V @ C
    if block > 0:
        U[:, block - 1], V[:, block - 1] = V[:, block - 1].copy(), U[:, block - 1].copy()
    return np.asfortranarray(U), np.asfortranarray(V)


def spherical_seed(basis: Basis, valence_Z: float, valence_N: float, seed: int = 0, slater: bool = False,
                   mix_quasiparticles: bool = True):
    """Spherical real Bogoliubov state: one occupation v^2 per j-shell and
    isospin for all its m-states, so that every shell is a (2j+1)-fold
    degenerate level of the canonical basis (the case the reference
    Schur-reduces with DGEES, module_wavefunctions.f90:873-906).  BCS
    occupations are drawn from ``seed`` and scaled to the particle numbers;
    with ``slater`` the lowest shells (in the basis order) are filled (v^2 = 1)
    and the rest left empty, which needs closed-shell particle numbers.  A
    random orthogonal mixing of the quasiparticles (right transformation)
    leaves rho and kappa unchanged."""
    rng = np.random.default_rng(seed)
    n = basis.n
    shells2j = [s % 100 for s in basis.shells]
    v2 = np.zeros((2, len(shells2j)))
    for t, target in enumerate((valence_Z, valence_N)):
        if slater:
            left = target
            for k, j in enumerate(shells2j):
                if left >= j + 1 - 1e-9:
                    v2[t, k] = 1.0
                    left -= j + 1
            if abs(left) > 1e-9:
                raise ValueError("a Slater determinant needs closed-shell particle numbers")
        else:
            w = rng.random(len(shells2j)) * np.exp(-0.3 * np.arange(len(shells2j)))
            deg = np.array([j + 1 for j in shells2j], dtype=float)
            # scale the occupations to the particle number, keeping 0 < v^2 < 1
            lo, hi = 0.0, 1e6
            for _ in range(200):
                mid = 0.5 * (lo + hi)
                num = float(np.sum(deg * (mid * w) / (1.0 + mid * w)))
                lo, hi = (mid, hi) if num < target else (lo, mid)
            v2[t] = (lo * w) / (1.0 + lo * w)
    U = np.zeros((n, n))
    V = np.zeros((n, n))
    ipos = 0
    for k, j in enumerate(shells2j):
        for m in range(1, (j + 1) // 2 + 1):
            p1 = ipos + m - 1
            p2 = ipos + j + 2 - m - 1
            for t in (0, 1):
                a, b = p1 + t * (n // 2), p2 + t * (n // 2)
                U[a, a] = U[b, b] = np.sqrt(1.0 - v2[t, k])
                V[a, b] = np.sqrt(v2[t, k])
                V[b, a] = -V[a, b]
        ipos += j + 1
    if mix_quasiparticles:
        B = rng.random((n, n))
        C = np.linalg.eigh(np.triu(B) + np.triu(B, 1).T)[1]
        U, V = U @ C, V @ C
    return np.asfortranarray(U), np.asfortranarray(V)
