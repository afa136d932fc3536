"""ctypes binding of ``libtvap_gpu.so`` (include/tvap.h) with the argument
meaning of the reference's Fortran routines.

The library is the only compute path: there is no CPU fallback.  Importing
this module on a machine without the built library, or calling it without a
CUDA device, raises.
"""

from __future__ import annotations

import ctypes
import math
import os

import numpy as np

from . import _build

TVAP_OK = 0
ERRORS = {
    1: "bad argument", 2: "CUDA error", 3: "hamiltonian not set",
    10: "U_phi singular (calculate_thouless)",
    11: "canonical overlap matrix singular (calculate_overlap: info from zgetrf)",
    13: "the gradient has non-zero imaginary part (calculate_projected_H20)",
    14: "Cholesky factorization has failed (cholesky_factorization)",
    15: "error in the inverse of L (evolve_wavefunction)",
    16: "canonical basis: eigen solver did not converge or a degenerate subspace could not be reduced",
    18: "particle numbers wrong three times in the last five iterations",
    19: "a bounded wait inside a device kernel ran out (the kernel stopped and released its resources)",
}


class TvapError(RuntimeError):
    def __init__(self, code: int, where: str, detail: str = ""):
        self.code = code
        msg = f"{where}: status {code} ({ERRORS.get(code, 'unknown')})"
        if detail:
            msg += f": {detail}"
        super().__init__(msg)


class TvapPnp(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double * 2) for k in ("over", "ener", "prot", "neut", "prot2", "neut2")] + [
        ("nocc", ctypes.c_int), ("nemp", ctypes.c_int)]

    def c(self, k: str) -> complex:
        v = getattr(self, k)
        return complex(v[0], v[1])


class TvapPnpObs(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double * 2) for k in ("over", "ener", "prot", "neut", "prot2", "neut2", "pari")] + [
        ("ecomp", (ctypes.c_double * 2) * 12), ("nocc", ctypes.c_int), ("nemp", ctypes.c_int)]

    def c(self, k: str) -> complex:
        v = getattr(self, k)
        return complex(v[0], v[1])


class TvapProjOpts(ctypes.Structure):
    _fields_ = [("Mphip", ctypes.c_int), ("Mphin", ctypes.c_int), ("facpi", ctypes.c_double),
                ("valence_Z", ctypes.c_double), ("valence_N", ctypes.c_double),
                ("factor_delta", ctypes.c_double), ("seed_occeps", ctypes.c_double),
                ("seed_allemp", ctypes.c_int), ("mode", ctypes.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.GPU_LIB
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: run __graft_entry__.build() (no CPU fallback exists)")
        L = ctypes.CDLL(path)
        vp, ci, cd = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        L.tvap_init.argtypes = [ctypes.POINTER(vp), ctypes.c_int64, vp, vp, vp, ci]
        L.tvap_init.restype = ci
        L.tvap_destroy.argtypes = [vp]
        L.tvap_last_error.restype = ctypes.c_char_p
        L.tvap_kernel_launches.argtypes = [vp]
        L.tvap_kernel_launches.restype = ci
        L.tvap_set_stream.argtypes = [vp, vp]
        L.tvap_set_stream.restype = ci
        L.tvap_set_timing.argtypes = [vp, ci]
        L.tvap_set_timing.restype = ci
        L.tvap_get_timing.argtypes = [vp, vp, vp, ci]
        L.tvap_get_timing.restype = ci
        L.tvap_get_timeline.argtypes = [vp, vp, vp, ci]
        L.tvap_get_timeline.restype = ci
        L.tvap_get_counters.argtypes = [vp, vp, ci]
        L.tvap_get_counters.restype = ci
        L.tvap_set_gemm_mode.argtypes = [vp, ci]
        L.tvap_set_gemm_mode.restype = ci
        L.tvap_set_hamiltonian.argtypes = [vp, ctypes.c_int64, vp, vp, vp, vp, vp]
        L.tvap_set_hamiltonian.restype = ci
        L.tvap_calculate_fields.argtypes = [vp] * 8
        L.tvap_calculate_fields.restype = ci
        L.tvap_calculate_fields_batched.argtypes = [vp, ci] + [vp] * 7
        L.tvap_calculate_fields_batched.restype = ci
        L.tvap_project.argtypes = [vp, vp, vp, ctypes.POINTER(TvapProjOpts), ctypes.POINTER(TvapPnp), vp]
        L.tvap_project.restype = ci
        L.tvap_project_batched.argtypes = [vp, ci, vp, vp, ctypes.POINTER(TvapProjOpts), ctypes.POINTER(TvapPnp), vp]
        L.tvap_project_batched.restype = ci
        L.tvap_calculate_gradient.argtypes = [vp, vp, ci, vp, vp, vp, cd, cd, vp, vp]
        L.tvap_calculate_gradient.restype = ci
        L.tvap_evolve.argtypes = [vp] * 6
        L.tvap_evolve.restype = ci
        L.tvap_evolve_noalloc.argtypes = [vp] * 6
        L.tvap_evolve_noalloc.restype = ci
        L.tvap_energy_adjoint.argtypes = [vp, vp, vp, vp, ctypes.POINTER(TvapProjOpts), vp, vp]
        L.tvap_energy_adjoint.restype = ci
        L.tvap_iterate.argtypes = [vp, vp, vp, ctypes.POINTER(TvapProjOpts), cd, cd, vp, vp, vp, vp,
                                   ctypes.POINTER(TvapPnp), vp, vp]
        L.tvap_iterate.restype = ci
        L.tvap_diagonalize_hsp_and_H11.argtypes = [vp, vp, vp, ci, ci, vp, vp, cd, vp, vp, vp]
        L.tvap_diagonalize_hsp_and_H11.restype = ci
        L.tvap_gradient_parameters.argtypes = [ci, ci, vp, vp, vp, cd, cd, vp, vp]
        L.tvap_gradient_parameters.restype = ci
        L.tvap_adjust_constraints.argtypes = [vp, vp, vp, vp, ci, ci, vp, vp, cd, vp, vp, vp, vp]
        L.tvap_adjust_constraints.restype = ci
        L.tvap_iterate_many.argtypes = [ci, vp, vp, vp, ctypes.POINTER(TvapProjOpts), vp, vp, vp, vp, vp, vp,
                                        ctypes.POINTER(TvapPnp), vp, vp]
        L.tvap_iterate_many.restype = ci
        L.tvap_project_observables.argtypes = [vp, vp, vp, ctypes.POINTER(TvapProjOpts), ci, vp, ci, vp, vp, ci, vp,
                                               ctypes.POINTER(TvapPnpObs), vp, vp, vp, vp]
        L.tvap_project_observables.restype = ci
        L.tvap_autotune.argtypes = [vp, vp, vp, ctypes.POINTER(TvapProjOpts), ci, vp, ci]
        L.tvap_autotune.restype = ci
        L.tvap_set_tuning.argtypes = [vp, ci, ci, ci]
        L.tvap_set_tuning.restype = ci
        L.tvap_get_tuning.argtypes = [vp, vp]
        L.tvap_get_tuning.restype = ci
        L.tvap_set_option.argtypes = [vp, ci, ci]
        L.tvap_set_option.restype = ci
        L.tvap_get_option.argtypes = [vp, ci]
        L.tvap_get_option.restype = ci
        L.tvap_test_wait_timeout.argtypes = [vp]
        L.tvap_test_wait_timeout.restype = ci
        L.tvap_zskpfa_batched.argtypes = [vp, ci, ctypes.c_int64, vp, vp]
        L.tvap_zskpfa_batched.restype = ci
        cc = ctypes.c_char
        for name in ("tvap_zgemm", "tvap_dgemm"):
            getattr(L, name).argtypes = [vp, cc, cc, ci, ci, ci, vp, vp, ci, vp, ci, vp, vp, ci]
            getattr(L, name).restype = ci
        _lib = L
    return _lib


def _p(a):
    if a is None:
        return None
    if hasattr(a, "data_ptr"):  # torch tensor (host or device)
        return ctypes.c_void_p(a.data_ptr())
    return a.ctypes.data_as(ctypes.c_void_p)


def _check(rc: int, where: str):
    if rc != TVAP_OK:
        raise TvapError(rc, where, lib().tvap_last_error().decode(errors="replace"))


def _f(a, dtype):
    if hasattr(a, "data_ptr"):
        return a
    return np.asfortranarray(np.asarray(a, dtype=dtype))


class Context:
    """One device context: basis tables and the uploaded Hamiltonian."""

    def __init__(self, basis, ham=None, device: int = -1):
        L = lib()
        self.n = basis.n
        self._tables = [np.ascontiguousarray(x, dtype=np.int32) for x in (basis.sp_2mj, basis.sp_tr, basis.sp_l)]
        h = ctypes.c_void_p()
        _check(L.tvap_init(ctypes.byref(h), self.n, *[_p(t) for t in self._tables], device), "tvap_init")
        self.h = h
        if ham is not None:
            self.set_hamiltonian(ham)

    def close(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.tvap_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    @property
    def kernel_launches(self) -> int:
        return lib().tvap_kernel_launches(self.h)

    SECTIONS = ("canonical", "blocks", "solve", "uv", "densities", "fields_gamma", "fields_delta", "traces",
                "h20", "overlap", "pfaffian", "sums", "gradient", "evolve", "h20_tc")

    def set_timing(self, on: bool):
        _check(lib().tvap_set_timing(self.h, 1 if on else 0), "tvap_set_timing")

    def get_timing(self):
        ms = np.zeros(16)
        calls = np.zeros(16, dtype=np.int64)
        _check(lib().tvap_get_timing(self.h, _p(ms), _p(calls), 16), "tvap_get_timing")
        return {k: (float(ms[i]), int(calls[i])) for i, k in enumerate(self.SECTIONS)}

    def get_timeline(self):
        """Mean (start, end) in ms of every timed section from the start of
        its projection (gradient and evolution: from the projection before)."""
        t0 = np.zeros(16)
        t1 = np.zeros(16)
        _check(lib().tvap_get_timeline(self.h, _p(t0), _p(t1), 16), "tvap_get_timeline")
        return {k: (float(t0[i]), float(t1[i])) for i, k in enumerate(self.SECTIONS)}

    def canonical_paths(self):
        """Canonical-basis counters since the last set_timing: (FP32 Jacobi +
        refinement attempts, accepted, exact FP64 Jacobi runs, FP32 sweeps,
        rejections for coupled clusters, for lost orthonormality, for
        clusters that could not be diagonalised (each failed check counts),
        large clusters diagonalised by the FP64 Jacobi of their block,
        refinements continued by two second-order steps)."""
        out = np.zeros(9, dtype=np.int64)
        _check(lib().tvap_get_counters(self.h, _p(out), 9), "tvap_get_counters")
        return tuple(int(v) for v in out)

    GEMM_FP64, GEMM_MMA_SYNC, GEMM_TCGEN05 = 0, 1, 2
    GEMM_EMULATED = GEMM_TCGEN05

    def set_gemm_mode(self, mode: int):
        """0: dense products on the FP64 pipe; 1: FP64 emulated on the bf16
        tensor cores with mma.sync; 2 (default): the same with tcgen05 MMAs and
        tensor-memory accumulators for the batched products."""
        _check(lib().tvap_set_gemm_mode(self.h, int(mode)), "tvap_set_gemm_mode")

    def set_stream(self, stream_handle: int):
        """Run the context's calls in order on this CUDA stream (a raw
        cudaStream_t handle, e.g. torch.cuda.Stream.cuda_stream)."""
        _check(lib().tvap_set_stream(self.h, ctypes.c_void_p(stream_handle)), "tvap_set_stream")

    def set_hamiltonian(self, ham):
        abcd = np.ascontiguousarray(ham.abcd, dtype=np.int16)
        h2 = np.ascontiguousarray(ham.h2, dtype=np.float32)
        tr = np.ascontiguousarray(ham.trperm, dtype=np.int8)
        H1 = np.asfortranarray(ham.H1, dtype=np.complex128)
        H0 = np.array([ham.H0.real, ham.H0.imag])
        _check(lib().tvap_set_hamiltonian(self.h, ham.S, _p(abcd), _p(h2), _p(tr), _p(H1), _p(H0)),
               "tvap_set_hamiltonian")

    # -- calculate_fields (module_fields.f90:99-189) --------------------------
    def calculate_fields(self, rhoLR, kappaLR, kappaRL):
        n = self.n
        rho, kl, kr = (_f(x, np.complex128) for x in (rhoLR, kappaLR, kappaRL))
        outs = [np.zeros((n, n), dtype=np.complex128, order="F") for _ in range(4)]
        _check(lib().tvap_calculate_fields(self.h, _p(rho), _p(kl), _p(kr), *[_p(o) for o in outs]),
               "tvap_calculate_fields")
        return tuple(outs)  # gammaLR, hspLR, deltaLR, deltaRL

    def calculate_fields_batched(self, rho, kLR, kRL):
        """rho, kLR, kRL: arrays (ncol, n, n) of Fortran-ordered matrices."""
        ncol = rho.shape[0]
        n = self.n
        conv = [np.ascontiguousarray(np.transpose(np.asarray(x, dtype=np.complex128), (0, 2, 1)))
                for x in (rho, kLR, kRL)]
        outs = [np.zeros((ncol, n, n), dtype=np.complex128) for _ in range(4)]
        _check(lib().tvap_calculate_fields_batched(self.h, ncol, *[_p(x) for x in conv], *[_p(o) for o in outs]),
               "tvap_calculate_fields_batched")
        return tuple(np.transpose(o, (0, 2, 1)) for o in outs)

    # -- project_wavefunction(0, ...) + calculate_projected_H20 ----------------
    def project(self, U0, V0, Mphip, Mphin, facpi, valence_Z, valence_N, factor_delta=1.0, seed_occeps=0.0,
                seed_allemp=0, mode=0):
        n = self.n
        U, V = _f(U0, np.float64), _f(V0, np.float64)
        o = TvapProjOpts(Mphip, Mphin, facpi, valence_Z, valence_N, factor_delta, seed_occeps, seed_allemp, mode)
        out = TvapPnp()
        H20v = np.zeros(n * n)
        _check(lib().tvap_project(self.h, _p(U), _p(V), ctypes.byref(o), ctypes.byref(out), _p(H20v)),
               "tvap_project")
        return out, H20v

    def project_observables(self, U0, V0, Mphip, Mphin, facpi, valence_Z, valence_N, ops, factor_delta=1.0,
                            seed_occeps=0.0, seed_allemp=0, with_parity=True):
        """tvap_project_observables (project_wavefunction with iopt = 1):
        returns a dict with 'scal' (over, ener, prot, neut, prot2, neut2,
        pari, ecomp[12]: the complex gauge sums), 'obo' (nobo x (p, n)), 'sq'
        (nsq), 'occnum' (nshell x (p, n)), 'rho' (pnp_rho, n x n), 'nocc',
        'nemp'.  ops: taurus_vap_gb300.model.Model.observable_operators()."""
        n = self.n
        U, V = _f(U0, np.float64), _f(V0, np.float64)
        o = TvapProjOpts(Mphip, Mphin, facpi, valence_Z, valence_N, factor_delta, seed_occeps, seed_allemp, 0)
        obo = np.ascontiguousarray(np.stack([np.asfortranarray(b).ravel(order="F") for b in ops["obo"]]))
        sq = np.ascontiguousarray(np.stack([np.asfortranarray(b).ravel(order="F") for pr in ops["sq"] for b in pr]))
        par = np.ascontiguousarray(ops["parity"], dtype=np.int32)
        shells = np.ascontiguousarray(ops["shell_size"], dtype=np.int32)
        nobo, nsq, nsh = len(ops["obo"]), len(ops["sq"]), len(shells)
        out = TvapPnpObs()
        bs = np.zeros((nobo, 2), dtype=np.complex128)
        ss = np.zeros(nsq, dtype=np.complex128)
        oc = np.zeros((nsh, 2), dtype=np.complex128)
        rho = np.zeros((n, n), dtype=np.complex128, order="F")
        _check(lib().tvap_project_observables(self.h, _p(U), _p(V), ctypes.byref(o), nobo, _p(obo), nsq, _p(sq),
                                              _p(par) if with_parity else None, nsh, _p(shells), ctypes.byref(out),
                                              _p(bs), _p(ss), _p(oc), _p(rho)), "tvap_project_observables")
        scal = np.array([out.c(k) for k in ("over", "ener", "prot", "neut", "prot2", "neut2", "pari")] +
                        [complex(out.ecomp[q][0], out.ecomp[q][1]) for q in range(12)])
        return {"scal": scal, "obo": bs, "sq": ss, "occnum": oc, "rho": rho, "nocc": out.nocc, "nemp": out.nemp}

    def project_batched(self, U0s, V0s, opts):
        """tvap_project_batched: states U0s[s], V0s[s] (n x n each) with
        options opts[s] = dict(Mphip=, Mphin=, facpi=, valence_Z=,
        valence_N=, factor_delta=1.0, seed_occeps=0.0, seed_allemp=0,
        mode=0); returns the list of (pnp, H20v)."""
        n, ns = self.n, len(opts)
        U = np.stack([_f(u, np.float64) for u in U0s]).transpose(0, 2, 1).copy()  # column-major per state
        V = np.stack([_f(v, np.float64) for v in V0s]).transpose(0, 2, 1).copy()
        O = (TvapProjOpts * ns)()
        for s, d in enumerate(opts):
            O[s] = TvapProjOpts(d["Mphip"], d["Mphin"], d["facpi"], d["valence_Z"], d["valence_N"],
                                d.get("factor_delta", 1.0), d.get("seed_occeps", 0.0), d.get("seed_allemp", 0),
                                d.get("mode", 0))
        outs = (TvapPnp * ns)()
        H20v = np.zeros(ns * n * n)
        _check(lib().tvap_project_batched(self.h, ns, _p(U), _p(V), O, outs, _p(H20v)), "tvap_project_batched")
        return [(outs[s], H20v[s * n * n:(s + 1) * n * n]) for s in range(ns)]

    # -- calculate_gradient (module_gradient.f90:79-143), gradient_type 0 -----
    def calculate_gradient(self, H20v, lambdas, C20, Zim1, eta, mu):
        n = self.n
        cdim = 0 if lambdas is None else len(lambdas)
        H = np.ascontiguousarray(H20v, dtype=np.float64)
        Zm = np.ascontiguousarray(Zim1, dtype=np.float64).reshape(-1)
        lam = None if cdim == 0 else np.ascontiguousarray(lambdas, dtype=np.float64)
        C = None if cdim == 0 else np.ascontiguousarray(C20, dtype=np.float64)
        Zi = np.zeros(n * n)
        norm = ctypes.c_double()
        _check(lib().tvap_calculate_gradient(self.h, _p(H), cdim, _p(lam), _p(C), _p(Zm), eta, mu, _p(Zi),
                                             ctypes.byref(norm)), "tvap_calculate_gradient")
        return Zi, norm.value

    # -- cholesky_factorization + evolve_wavefunction --------------------------
    def evolve(self, U0, V0, Z):
        n = self.n
        U, V, Zm = _f(U0, np.float64), _f(V0, np.float64), _f(np.reshape(Z, (n, n), order="F"), np.float64)
        U1 = np.zeros((n, n), order="F")
        V1 = np.zeros((n, n), order="F")
        _check(lib().tvap_evolve(self.h, _p(U), _p(V), _p(Zm), _p(U1), _p(V1)), "tvap_evolve")
        return U1, V1

    # -- launch shapes by measurement ------------------------------------------
    OPT_SOLVE_LOOKAHEAD, OPT_PFAFFIAN_BLOCKED, OPT_COMPLEX_PAIRS = 1, 2, 3
    TUNE_CANDIDATES = [(bn, g, cap, la, pf) for pf in (0, 1) for la in (1, 0) for g in (2, 1)
                       for cap in ((0, 1, 2) if g == 2 else (0,)) for bn in (0, 1, 2)]

    def autotune(self, U0, V0, Mphip, Mphin, facpi, valence_Z, valence_N, reps=3):
        """tvap_autotune: times the projection for every candidate launch
        shape and keeps the fastest; returns {(bn, groups, cap, lookahead,
        pfaffian_blocked): ms}."""
        U, V = _f(U0, np.float64), _f(V0, np.float64)
        o = TvapProjOpts(Mphip, Mphin, facpi, valence_Z, valence_N, 1.0, 0.0, 0, 0)
        table = np.zeros(len(self.TUNE_CANDIDATES))
        _check(lib().tvap_autotune(self.h, _p(U), _p(V), ctypes.byref(o), reps, _p(table), table.size),
               "tvap_autotune")
        return dict(zip(self.TUNE_CANDIDATES, table.tolist()))

    def tuning(self):
        """(bn, groups, cap, lookahead, pfaffian_blocked) of the context."""
        k = np.zeros(3, dtype=np.int32)
        _check(lib().tvap_get_tuning(self.h, _p(k)), "tvap_get_tuning")
        return tuple(int(x) for x in k) + (int(lib().tvap_get_option(self.h, self.OPT_SOLVE_LOOKAHEAD)),
                                           int(lib().tvap_get_option(self.h, self.OPT_PFAFFIAN_BLOCKED)))

    def set_option(self, option, value):
        """tvap_set_option (OPT_SOLVE_LOOKAHEAD, OPT_PFAFFIAN_BLOCKED,
        OPT_COMPLEX_PAIRS; 0 or 1)."""
        _check(lib().tvap_set_option(self.h, option, value), "tvap_set_option")

    def option(self, option):
        return int(lib().tvap_get_option(self.h, option))

    def set_tuning(self, bn_policy, solve_groups, solve_cap, lookahead=0, pfaffian_blocked=0):
        _check(lib().tvap_set_tuning(self.h, bn_policy, solve_groups, solve_cap), "tvap_set_tuning")
        _check(lib().tvap_set_option(self.h, self.OPT_SOLVE_LOOKAHEAD, lookahead), "tvap_set_option")
        _check(lib().tvap_set_option(self.h, self.OPT_PFAFFIAN_BLOCKED, pfaffian_blocked), "tvap_set_option")

    # -- adjust_constraints (module_constraints.f90:270-373) -------------------
    def adjust_constraints(self, U0, V0, Zi, constraints_HO, values, cpair=0, eps=1e-6):
        """The constraint Newton loop on the device: returns (U1, V1, Zi, C20,
        steps) with Zi the adjusted step."""
        n = self.n
        U, V = _f(U0, np.float64), _f(V0, np.float64)
        Z = np.array(np.reshape(Zi, -1), dtype=np.float64)
        cdim = len(values)
        C = None if cdim == 0 else np.ascontiguousarray(constraints_HO, dtype=np.float64).reshape(-1)
        vals = None if cdim == 0 else np.ascontiguousarray(values, dtype=np.float64)
        U1 = np.zeros((n, n), order="F")
        V1 = np.zeros((n, n), order="F")
        C20 = np.zeros((max(cdim, 1), n * n))
        it = ctypes.c_int()
        _check(lib().tvap_adjust_constraints(self.h, _p(U), _p(V), _p(Z), cdim, cpair, _p(C), _p(vals), eps, _p(U1),
                                             _p(V1), _p(C20), ctypes.byref(it)), "tvap_adjust_constraints")
        return U1, V1, Z, C20[:cdim], it.value

    # -- diagonalize_hsp_and_H11(0) (module_gradient.f90:158-453) -------------
    def diagonalize_hsp_and_H11(self, U0, V0, lambdas=None, constraints_HO=None, cpair=0, factor_delta=1.0):
        """Eigenvalues of h^RR and H11 (with the constraint terms of the
        multipliers): (eigen_hsp, eigen_H11, (info_hsp, info_H11))."""
        n = self.n
        U, V = _f(U0, np.float64), _f(V0, np.float64)
        cdim = 0 if lambdas is None else len(lambdas)
        lam = None if cdim == 0 else np.ascontiguousarray(lambdas, dtype=np.float64)
        C = None if cdim == 0 else np.ascontiguousarray(constraints_HO, dtype=np.float64).reshape(-1)
        eh = np.zeros(n)
        e11 = np.zeros(n)
        info = np.zeros(2, dtype=np.int32)
        _check(lib().tvap_diagonalize_hsp_and_H11(self.h, _p(U), _p(V), cdim, cpair, _p(lam), _p(C), factor_delta,
                                                  _p(eh), _p(e11), _p(info)), "tvap_diagonalize_hsp_and_H11")
        return eh, e11, (int(info[0]), int(info[1]))

    # -- one gradient iteration (taurus_vap.f90:86-113), gradient_type 0 -------
    def iterate(self, U0, V0, Zim1, Mphip, Mphin, facpi, valence_Z, valence_N, eta, mu, factor_delta=1.0,
                seed_occeps=0.0, seed_allemp=0, want_H20v=False):
        """Projection, gradient and Thouless evolution with one host round
        trip: returns (pnp, Zi, gradient_norm, U1, V1[, H20v]).  A caller
        whose convergence test stops the loop keeps (U0, V0)."""
        n = self.n
        U, V = _f(U0, np.float64), _f(V0, np.float64)
        Zm = np.ascontiguousarray(Zim1, dtype=np.float64).reshape(-1)
        o = TvapProjOpts(Mphip, Mphin, facpi, valence_Z, valence_N, factor_delta, seed_occeps, seed_allemp, 0)
        out = TvapPnp()
        Zi = np.zeros(n * n)
        U1 = np.zeros((n, n), order="F")
        V1 = np.zeros((n, n), order="F")
        H = np.zeros(n * n) if want_H20v else None
        norm = ctypes.c_double()
        _check(lib().tvap_iterate(self.h, _p(U), _p(V), ctypes.byref(o), eta, mu, _p(Zm), _p(Zi), _p(U1), _p(V1),
                                  ctypes.byref(out), _p(H), ctypes.byref(norm)), "tvap_iterate")
        res = (out, Zi, norm.value, U1, V1)
        return res + (H,) if want_H20v else res

    # -- adjoint of E(Z) -------------------------------------------------------
    def energy_adjoint(self, U0, V0, Z, Mphip, Mphin, facpi, valence_Z, valence_N, factor_delta=1.0, mode=0):
        n = self.n
        U, V, Zm = _f(U0, np.float64), _f(V0, np.float64), _f(np.reshape(Z, (n, n), order="F"), np.float64)
        o = TvapProjOpts(Mphip, Mphin, facpi, valence_Z, valence_N, factor_delta, 0.0, 0, mode)
        E = ctypes.c_double()
        G = np.zeros((n, n), order="F")
        _check(lib().tvap_energy_adjoint(self.h, _p(U), _p(V), _p(Zm), ctypes.byref(o), ctypes.byref(E), _p(G)),
               "tvap_energy_adjoint")
        return E.value, G

    # -- ZSKPFA('U', 'P') of PFAPACK (subroutines_pfaffian.f:12-258) ------------
    def zskpfa_batched(self, A):
        """Pfaffians of a batch (b, m, m) of complex skew-symmetric matrices
        (A[q] is matrix q, indexed [row, column]; only the upper triangle is
        read)."""
        A = np.asarray(A, dtype=np.complex128)
        if A.ndim == 2:
            A = A[None]
        b, m = A.shape[0], A.shape[1]
        cm = np.ascontiguousarray(np.transpose(A, (0, 2, 1)))  # column-major per matrix
        pf = np.zeros(2 * b)
        _check(lib().tvap_zskpfa_batched(self.h, b, m, _p(cm), _p(pf)), "tvap_zskpfa_batched")
        return pf[0::2] + 1j * pf[1::2]

    # -- ZGEMM / DGEMM in the context's arithmetic -----------------------------
    def gemm(self, A, B, transa="N", transb="N", alpha=1.0, beta=0.0, C=None):
        """C = alpha op(A) op(B) + beta C (complex when any operand is)."""
        cplx = any(np.iscomplexobj(x) for x in (A, B, C) if x is not None) or isinstance(alpha, complex) or \
            isinstance(beta, complex)
        dt = np.complex128 if cplx else np.float64
        A = np.asfortranarray(A, dtype=dt)
        B = np.asfortranarray(B, dtype=dt)
        m = A.shape[1] if transa.upper() != "N" else A.shape[0]
        k = A.shape[0] if transa.upper() != "N" else A.shape[1]
        n = B.shape[0] if transb.upper() != "N" else B.shape[1]
        C = np.zeros((m, n), dtype=dt, order="F") if C is None else np.array(C, dtype=dt, order="F")
        if cplx:
            al = np.array([complex(alpha).real, complex(alpha).imag])
            be = np.array([complex(beta).real, complex(beta).imag])
            fn = lib().tvap_zgemm
        else:
            al, be = np.array([float(alpha)]), np.array([float(beta)])
            fn = lib().tvap_dgemm
        _check(fn(self.h, transa.encode(), transb.encode(), m, n, k, _p(al), _p(A), max(1, A.shape[0]), _p(B),
                  max(1, B.shape[0]), _p(be), _p(C), max(1, m)), "tvap_gemm")
        return C


TWO_PI = 2.0 * math.pi


def gradient_parameters(gradient_type, eigen_hsp, eigen_H11, info, eta_in, mu_in):
    """(eta, mu) of calculate_gradient (module_gradient.f90:86-119) for
    gradient_type 0, 1 or 2 (tvap_gradient_parameters)."""
    eh = np.ascontiguousarray(eigen_hsp, dtype=np.float64)
    e11 = np.ascontiguousarray(eigen_H11, dtype=np.float64)
    inf = np.ascontiguousarray(info, dtype=np.int32)
    eta = ctypes.c_double()
    mu = ctypes.c_double()
    _check(lib().tvap_gradient_parameters(int(gradient_type), eh.size, _p(eh), _p(e11), _p(inf), eta_in, mu_in,
                                          ctypes.byref(eta), ctypes.byref(mu)), "tvap_gradient_parameters")
    return eta.value, mu.value


def iterate_many(contexts, U0s, V0s, Zim1s, opts, etas, mus):
    """tvap_iterate_many: one gradient iteration for each state s on
    contexts[s] (states of one context in order, distinct contexts
    concurrently).  opts[s] is a dict of tvap_proj_opts fields (Mphip, Mphin,
    facpi, valence_Z, valence_N[, factor_delta, seed_occeps, seed_allemp]).
    Returns [(pnp, Zi, gradient_norm, U1, V1)] per state."""
    ns = len(contexts)
    P = ctypes.c_void_p * ns
    Us = [_f(u, np.float64) for u in U0s]
    Vs = [_f(v, np.float64) for v in V0s]
    Zm = [np.ascontiguousarray(z, dtype=np.float64).reshape(-1) for z in Zim1s]
    Zi = [np.zeros(c.n * c.n) for c in contexts]
    U1 = [np.zeros((c.n, c.n), order="F") for c in contexts]
    V1 = [np.zeros((c.n, c.n), order="F") for c in contexts]
    O = (TvapProjOpts * ns)()
    for s, d in enumerate(opts):
        O[s] = TvapProjOpts(d["Mphip"], d["Mphin"], d["facpi"], d["valence_Z"], d["valence_N"],
                            d.get("factor_delta", 1.0), d.get("seed_occeps", 0.0), d.get("seed_allemp", 0), 0)
    outs = (TvapPnp * ns)()
    eta = np.ascontiguousarray(etas, dtype=np.float64)
    mu = np.ascontiguousarray(mus, dtype=np.float64)
    gn = np.zeros(ns)
    st = np.zeros(ns, dtype=np.int32)
    ptrs = lambda arrs: P(*[a.ctypes.data for a in arrs])
    _check(lib().tvap_iterate_many(ns, P(*[c.h.value for c in contexts]), ptrs(Us), ptrs(Vs), O, _p(eta), _p(mu),
                                   ptrs(Zm), ptrs(Zi), ptrs(U1), ptrs(V1), outs, _p(gn), _p(st)),
           "tvap_iterate_many")
    return [(outs[s], Zi[s], float(gn[s]), U1[s], V1[s]) for s in range(ns)]
