"""ORACLE -- test infrastructure only (loaded by tests/, smoke() and bench.py's
CPU legs; never by the product path).

ctypes wrapper of ``liboracle.so`` (tvap_oracle.cpp), the CPU restatement of the
reference's PNVAP path.  BLAS/LAPACK addresses are taken from SciPy's
``cython_blas`` / ``cython_lapack`` capsules and handed to the library once.
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

_lib = None


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "tvap_oracle.cpp")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(src) > os.path.getmtime(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def _capsule_address(capsule) -> int:
    get_name = ctypes.pythonapi.PyCapsule_GetName
    get_name.restype = ctypes.c_char_p
    get_name.argtypes = [ctypes.py_object]
    get_ptr = ctypes.pythonapi.PyCapsule_GetPointer
    get_ptr.restype = ctypes.c_void_p
    get_ptr.argtypes = [ctypes.py_object, ctypes.c_char_p]
    return get_ptr(capsule, get_name(capsule))


class OrcPnp(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double * 2) for k in ("over", "ener", "prot", "neut", "prot2", "neut2")] + [
        ("nocc", ctypes.c_int), ("nemp", ctypes.c_int)]

    def c(self, k):
        v = getattr(self, k)
        return complex(v[0], v[1])


class OrcAngle(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double * 2) for k in ("over", "ener", "prot", "neut", "prot2", "neut2")]


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        from scipy.linalg import cython_blas, cython_lapack

        b, l = cython_blas.__pyx_capi__, cython_lapack.__pyx_capi__
        ptrs = [_capsule_address(x) for x in (b["zgemm"], b["dgemm"], l["zgetrf"], l["zgetri"], l["dsyev"],
                                              l["dgees"], l["dpbtrf"], l["dtrtri"], l["dsysv"])]
        L.orc_set_lapack.argtypes = [ctypes.c_void_p] * 9
        L.orc_set_lapack(*ptrs)
        vp, ci, cd = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        L.orc_model_new.restype = vp
        L.orc_model_new.argtypes = [ci, vp, vp, vp, ctypes.c_longlong, vp, vp, vp, vp, vp]
        L.orc_model_free.argtypes = [vp]
        L.orc_calculate_fields.argtypes = [vp] * 8 + [ci]
        L.orc_calculate_fields_diag.argtypes = [vp] * 7 + [ci]
        L.orc_pfaffian.argtypes = [ci, vp, vp]
        L.orc_pfaffian.restype = ci
        L.orc_canonical.argtypes = [vp, vp, ci, cd, ci, vp, vp, vp, vp, vp]
        L.orc_canonical.restype = ci
        L.orc_project.argtypes = [vp, vp, vp, ci, ci, cd, cd, cd, cd, cd, ci, vp, vp, vp, vp, vp, vp, ci]
        L.orc_project.restype = ci
        L.orc_project_observables.argtypes = [vp, vp, vp, ci, ci, cd, cd, cd, cd, cd, ci, ci, vp, ci, vp, vp, ci, vp,
                                              vp, vp, vp, vp, vp, ci]
        L.orc_project_observables.restype = ci
        L.orc_angle_densities.argtypes = [vp, vp, vp, cd, cd, vp, vp, vp, vp]
        L.orc_angle_densities.restype = ci
        L.orc_overlap.argtypes = [vp, vp, ci, cd, cd, cd, ci, vp]
        L.orc_overlap.restype = ci
        L.orc_vap_new.restype = vp
        L.orc_vap_new.argtypes = [vp, vp, vp, ci, ci, cd, cd, cd, ci, cd, cd, cd, ci, ci, vp, vp, cd, cd, ci]
        L.orc_vap_free.argtypes = [vp]
        L.orc_vap_initial_adjust.argtypes = [vp]
        L.orc_vap_initial_adjust.restype = ci
        L.orc_vap_iterate.argtypes = [vp, vp]
        L.orc_vap_iterate.restype = ci
        L.orc_vap_get_state.argtypes = [vp] * 5
        L.orc_vap_get_multipliers.argtypes = [vp, vp]
        L.orc_thouless_evolve.argtypes = [vp, vp, vp, ci, vp, vp]
        L.orc_thouless_evolve.restype = ci
        L.orc_vap_get_step.argtypes = [vp] * 5
        L.orc_diagonalize_hsp_and_H11.argtypes = [vp, vp, vp, ci, ci, ci, vp, vp, cd, vp, vp, vp, ci]
        L.orc_diagonalize_hsp_and_H11.restype = ci
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _cf(a, dtype=np.complex128):
    return np.asfortranarray(np.asarray(a, dtype=dtype))


class OracleModel:
    """The reference's hot-path module globals for one model."""

    def __init__(self, model):
        L = lib()
        b, h = model.basis, model.ham
        self.n = b.n
        self._keep = [np.ascontiguousarray(x) for x in (b.sp_2mj, b.sp_tr, b.sp_l, h.abcd, h.h2, h.trperm)]
        H1 = _cf(h.H1)
        H0 = np.array([h.H0.real, h.H0.imag])
        self._keep += [H1, H0]
        self.h = L.orc_model_new(self.n, *[_p(x) for x in self._keep[:3]], h.S, *[_p(x) for x in self._keep[3:6]],
                                 _p(H1), _p(H0))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_model_free(self.h)
            self.h = None

    def calculate_fields(self, rho, kLR, kRL, nthreads=0):
        n = self.n
        rho, kLR, kRL = _cf(rho), _cf(kLR), _cf(kRL)
        out = [np.zeros((n, n), dtype=np.complex128, order="F") for _ in range(4)]
        lib().orc_calculate_fields(self.h, _p(rho), _p(kLR), _p(kRL), *[_p(o) for o in out], nthreads)
        return tuple(out)  # gamma, h, deltaLR, deltaRL

    def calculate_fields_diag(self, rho, kLR, nthreads=0):
        n = self.n
        rho, kLR = _cf(rho), _cf(kLR)
        out = [np.zeros((n, n), dtype=np.complex128, order="F") for _ in range(4)]
        lib().orc_calculate_fields_diag(self.h, _p(rho), _p(kLR), *[_p(o) for o in out], nthreads)
        return tuple(out)

    def angle_densities(self, U, V, php, phn):
        n = self.n
        U, V = _cf(U, np.float64), _cf(V, np.float64)
        out = [np.zeros((n, n), dtype=np.complex128, order="F") for _ in range(4)]
        st = lib().orc_angle_densities(self.h, _p(U), _p(V), php, phn, *[_p(o) for o in out])
        return st, out  # rho, kLR, kRL, Aphi

    def project(self, U, V, Mp, Mn, facpi, Z, N, factor_delta=1.0, occeps=0.0, allemp=0, nthreads=0,
                want_matrices=False, want_angles=False):
        n = self.n
        U, V = _cf(U, np.float64), _cf(V, np.float64)
        out = OrcPnp()
        H20v = np.zeros(n * n)
        mats = [np.zeros((n, n), dtype=np.complex128, order="F") for _ in range(3)] if want_matrices else [None] * 3
        angles = (OrcAngle * (Mp * Mn))() if want_angles else None
        st = lib().orc_project(self.h, _p(U), _p(V), Mp, Mn, facpi, Z, N, factor_delta, occeps, allemp,
                               ctypes.byref(out), _p(H20v), *[_p(m) for m in mats],
                               ctypes.cast(angles, ctypes.c_void_p) if angles is not None else None, nthreads)
        res = {"status": st, "pnp": out, "H20v": H20v}
        if want_matrices:
            res["pnpA"], res["pnpH20"], res["pnpAH20"] = mats
        if want_angles:
            res["angles"] = angles
        return res

    def project_observables(self, U, V, Mp, Mn, facpi, Z, N, ops, factor_delta=1.0, occeps=0.0, allemp=0,
                            nthreads=0, with_parity=True):
        """project_wavefunction with iopt = 1 and its gauge sums: the scalars
        (over, ener, prot, neut, prot2, neut2, pari, ecomp[12]), the one-body
        traces (nobo x (p, n)), the <O^2> of the pairs, the occupation
        numbers (nshell x (p, n)) and pnp_rho.  ops: the dictionary of
        taurus_vap_gb300.model.Model.observable_operators()."""
        n = self.n
        U, V = _cf(U, np.float64), _cf(V, np.float64)
        obo = np.ascontiguousarray(np.stack([np.asfortranarray(b).ravel(order="F") for b in ops["obo"]]))
        sq = np.ascontiguousarray(np.stack([np.asfortranarray(b).ravel(order="F") for pr in ops["sq"] for b in pr]))
        par = np.ascontiguousarray(ops["parity"], dtype=np.int32)
        shells = np.ascontiguousarray(ops["shell_size"], dtype=np.int32)
        nobo, nsq, nsh = len(ops["obo"]), len(ops["sq"]), len(shells)
        scal = np.zeros(19, dtype=np.complex128)
        bs = np.zeros((nobo, 2), dtype=np.complex128)
        ss = np.zeros(nsq, dtype=np.complex128)
        oc = np.zeros((nsh, 2), dtype=np.complex128)
        rho = np.zeros((n, n), dtype=np.complex128, order="F")
        st = lib().orc_project_observables(self.h, _p(U), _p(V), Mp, Mn, facpi, Z, N, factor_delta, occeps, allemp,
                                           nobo, _p(obo), nsq, _p(sq), _p(par) if with_parity else None, nsh,
                                           _p(shells), _p(scal), _p(bs), _p(ss), _p(oc), _p(rho), nthreads)
        return {"status": st, "scal": scal, "obo": bs, "sq": ss, "occnum": oc, "rho": rho}


def pfaffian(A):
    A = _cf(A).copy(order="F")
    pf = np.zeros(2)
    info = lib().orc_pfaffian(A.shape[0], _p(A), _p(pf))
    return complex(pf[0], pf[1]), info


def canonical(U, V, occeps=0.0, allemp=0):
    n = U.shape[0]
    U, V = _cf(U, np.float64), _cf(V, np.float64)
    nocc, nemp = ctypes.c_int(), ctypes.c_int()
    ovac = ctypes.c_double()
    vu = np.zeros(n)
    D = np.zeros((n, n), order="F")
    info = lib().orc_canonical(_p(U), _p(V), n, occeps, allemp, ctypes.byref(nocc), ctypes.byref(nemp),
                               ctypes.byref(ovac), _p(vu), _p(D))
    return {"nocc": nocc.value, "nemp": nemp.value, "ovac": ovac.value, "voveru": vu[: n - nocc.value], "D": D,
            "info": info}


def overlap(U, V, php, phn, occeps=0.0, allemp=0):
    n = U.shape[0]
    U, V = _cf(U, np.float64), _cf(V, np.float64)
    ov = np.zeros(2)
    st = lib().orc_overlap(_p(U), _p(V), n, php, phn, occeps, allemp, _p(ov))
    return complex(ov[0], ov[1]), st


def thouless_evolve(U, V, Z):
    n = U.shape[0]
    U, V, Z = _cf(U, np.float64), _cf(V, np.float64), _cf(Z, np.float64)
    U1 = np.zeros((n, n), order="F")
    V1 = np.zeros((n, n), order="F")
    st = lib().orc_thouless_evolve(_p(U), _p(V), _p(Z), n, _p(U1), _p(V1))
    return st, U1, V1


class OracleVAP:
    """The reference's gradient loop (taurus_vap.f90:77-123), gradient_type 0."""

    def __init__(self, omodel: OracleModel, U, V, Mp, Mn, facpi, Z, N, eta, mu, geps, constraints_HO,
                 constraint_vals, ceps=1e-6, cpair=0, factor_delta=1.0, nthreads=0, gradient_type=0):
        n = omodel.n
        self.om = omodel
        self.n = n
        U, V = _cf(U, np.float64), _cf(V, np.float64)
        cHO = np.ascontiguousarray(np.asarray(constraints_HO, dtype=np.float64).reshape(-1))
        cval = np.ascontiguousarray(np.asarray(constraint_vals, dtype=np.float64).reshape(-1))
        self.cdim = cval.size
        self._keep = [U, V, cHO, cval]
        self.h = lib().orc_vap_new(omodel.h, _p(U), _p(V), Mp, Mn, facpi, Z, N, gradient_type, eta, mu, geps,
                                   self.cdim, cpair,
                                   _p(cHO) if cHO.size else None, _p(cval) if cval.size else None, ceps,
                                   factor_delta, nthreads)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_vap_free(self.h)
            self.h = None

    def initial_adjust(self):
        return lib().orc_vap_initial_adjust(self.h)

    def iterate(self):
        info = np.zeros(6)
        st = lib().orc_vap_iterate(self.h, _p(info))
        return st, info

    def step(self):
        """Eigenvalues of h^RR and H11, their DSYEV infos and the (eta, mu) of
        the last iteration."""
        n = self.n
        eh = np.zeros(n)
        e11 = np.zeros(n)
        infos = np.zeros(2, dtype=np.int32)
        em = np.zeros(2)
        lib().orc_vap_get_step(self.h, _p(eh), _p(e11), _p(infos), _p(em))
        return eh, e11, (int(infos[0]), int(infos[1])), (float(em[0]), float(em[1]))

    def state(self):
        n = self.n
        U = np.zeros((n, n), order="F")
        V = np.zeros((n, n), order="F")
        Zi = np.zeros(n * n)
        H = np.zeros(n * n)
        lib().orc_vap_get_state(self.h, _p(U), _p(V), _p(Zi), _p(H))
        return U, V, Zi, H


def diagonalize_hsp_and_H11(om: OracleModel, U, V, lam=(), constraints_HO=None, cpair=0, factor_delta=1.0, Mphip=2,
                            nthreads=0):
    """diagonalize_hsp_and_H11(0) (module_gradient.f90:158-453): eigenvalues
    of h^RR and of H11 for the state (U, V), with the constraint terms of the
    multipliers lam; Mphip = 1 takes the fields of the phi = 0 transition
    densities, as the reference does without projection.  Returns
    (eigen_hsp, eigen_H11, (info_hsp, info_H11))."""
    n = om.n
    U, V = _cf(U, np.float64), _cf(V, np.float64)
    lam = np.ascontiguousarray(lam, dtype=np.float64)
    cdim = lam.size
    cHO = np.ascontiguousarray(np.zeros(1) if cdim == 0 else np.asarray(constraints_HO, dtype=np.float64).reshape(-1))
    eh = np.zeros(n)
    e11 = np.zeros(n)
    infos = np.zeros(2, dtype=np.int32)
    lib().orc_diagonalize_hsp_and_H11(om.h, _p(U), _p(V), Mphip, cdim, cpair, _p(lam) if cdim else None, _p(cHO),
                                      factor_delta, _p(eh), _p(e11), _p(infos), nthreads)
    return eh, e11, (int(infos[0]), int(infos[1]))
