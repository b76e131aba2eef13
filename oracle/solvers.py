"""Krylov drivers of the oracle -- TEST INFRASTRUCTURE ONLY.

numpy/scipy restatements of the QS3 solver loops on top of the C++ oracle's
H*v (``oracle.Sector.hv``) or any other callable.  Level-1 BLAS maps to numpy
(``zdotc`` -> ``np.vdot``, ``dznrm2`` -> ``np.linalg.norm``); LAPACK maps to
scipy (``zheevr`` -> ``scipy.linalg.eigh(driver='evr')``, ``dstevx('V','A')`` and
``dstevx('V','I',1,1)`` -> ``scipy.linalg.lapack.dstev``, which computes the
same eigenpairs of the same tridiagonal matrix).

The start vector replaces the reference's unseeded ``random_number`` by the
counter-based generator :func:`start_vector`, which the GPU library
implements identically, so both sides start from the same vector.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla
from scipy.linalg import lapack

_M64 = (1 << 64) - 1
GOLDEN = 0x9E3779B97F4A7C15


def _mix64(z):
    """SplitMix64 finaliser (Vigna), vectorised on uint64."""
    z = np.asarray(z, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniform(seed, n0, n):
    """u_k = mix64(seed + (k+1)*GOLDEN) >> 11 * 2^-53 for k = n0 .. n0+n-1."""
    k = np.arange(n0, n0 + n, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = np.uint64(seed & _M64) + (k + np.uint64(1)) * np.uint64(GOLDEN)
    return (_mix64(z) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


def start_vector(D, seed):
    """psi(l) = (u_{2l} - 0.5, u_{2l+1} - 0.5): eigen_solver.f90:92-96 with a seeded generator."""
    u = uniform(seed, 0, 2 * D)
    return (u[0::2] - 0.5) + 1j * (u[1::2] - 0.5)


class NotConverged(RuntimeError):
    pass


def trlan(hv, D, NOE, NOK, NOM, maxitr, tol, start):
    """lancz_eigen_val_complex (eigen_solver.f90:69-261) + the NOM/NOK checks of
    my_trlanczos_routines_complex (eigen_solver.f90:19-22).

    Returns (ene[NOM], psi[:, :NOK], tritr, converged).
    """
    if NOE > NOK:
        raise ValueError("ne must be eaqual or smaller than NOK!")
    if NOM < 2 * NOK:
        NOM = 2 * NOK
    if D < NOE or D < NOK or D < NOM:
        raise ValueError("stop 999: dim smaller than NOM")
    psi = np.zeros((D, NOM + 1), dtype=np.complex128)
    alpha = np.zeros(NOM + 1)
    beta = np.zeros(NOM + 1)
    psi[:, 0] = start

    def reorth(i):  # full_reorthogonalization_complex, j = 1 .. i-1
        for j in range(1, i):
            ov = np.vdot(psi[:, j - 1], psi[:, i])
            psi[:, i] -= ov * psi[:, j - 1]

    beta[0] = np.linalg.norm(psi[:, 0])
    for i in range(1, NOM + 1):
        psi[:, i - 1] *= 1.0 / beta[i - 1]
        Q = hv(psi[:, i - 1])
        alpha[i] = np.vdot(psi[:, i - 1], Q).real
        if i > 1:
            psi[:, i] = Q - alpha[i] * psi[:, i - 1] - beta[i - 1] * psi[:, i - 2]
            reorth(i)
        else:
            psi[:, i] = Q - alpha[i] * psi[:, i - 1]
        beta[i] = np.linalg.norm(psi[:, i])
    psi[:, NOM] *= 1.0 / beta[NOM]
    ene, coef, info = lapack.dstev(alpha[1:NOM + 1].copy(), beta[1:NOM].copy(), compute_v=1)
    if info != 0:
        raise RuntimeError(f"error in dstevx, info = {info}")
    ccoef = coef.astype(np.complex128)
    calpha = alpha[1:].astype(np.complex128)          # calpha(1:NOM) -> [0:NOM]
    cbeta = beta.astype(np.complex128)                # cbeta(0:NOM)
    flag = 0
    converged = False
    tritr = 0
    for tritr in range(1, maxitr + 1):
        Qk = psi[:, :NOM] @ ccoef[:, :NOK]
        psi[:, :NOK] = Qk
        conv = np.abs(calpha[:NOK] / ene[:NOK] - 1.0)
        max_conv = conv.max()
        flag = flag + 1 if max_conv < tol else 0
        if flag == 2:
            converged = True
            break
        if tritr == maxitr:
            break
        psi[:, NOK] = psi[:, NOM]
        calpha[:NOK] = ene[:NOK]
        for j in range(1, NOK + 1):
            cbeta[j] = cbeta[NOM] * ccoef[NOM - 1, j - 1]
        i = NOK + 1
        Q = hv(psi[:, i - 1])
        calpha[i - 1] = np.vdot(psi[:, i - 1], Q)
        for j in range(1, NOK + 1):
            Q = Q - cbeta[j] * psi[:, j - 1]
        psi[:, i] = Q - calpha[i - 1] * psi[:, i - 1]
        reorth(i)
        cbeta[i] = np.linalg.norm(psi[:, i])
        for i in range(NOK + 2, NOM + 1):
            psi[:, i - 1] *= 1.0 / cbeta[i - 1]
            Q = hv(psi[:, i - 1])
            calpha[i - 1] = np.vdot(psi[:, i - 1], Q)
            psi[:, i] = Q - calpha[i - 1] * psi[:, i - 1] - cbeta[i - 1] * psi[:, i - 2]
            reorth(i)
            cbeta[i] = np.linalg.norm(psi[:, i])
        psi[:, NOM] *= 1.0 / cbeta[NOM]
        T = np.zeros((NOM, NOM), dtype=np.complex128)
        for j in range(NOM):
            T[j, j] = calpha[j]
        T[:NOK, NOK] = cbeta[1:NOK + 1]
        for j in range(NOK + 1, NOM):
            T[j - 1, j] = cbeta[j]
        ene, ccoef = sla.eigh(T, lower=False, driver="evr")
    return ene, psi[:, :NOK].copy(), tritr, converged


def lanczos(hv, D, maxitr, minitr, itrint, tol, start):
    """lancz_eigen_val (lanczos.f90:50-152): returns (ene, psi, ite_lancz)."""
    alpha = np.zeros(maxitr + 2)
    beta = np.zeros(maxitr + 2)
    v1 = np.array(start, dtype=np.complex128)
    beta[0] = np.linalg.norm(v1)
    v1 *= 1.0 / beta[0]
    psi_io = v1.copy()
    tmp = 0.0
    mitr = min(maxitr, D)
    z = None
    ene = None
    ite = None
    for i in range(1, mitr + 1):
        v2 = hv(v1)
        alpha[i] = np.vdot(v1, v2).real
        if i > 1:
            v2 = v2 - alpha[i] * v1 - beta[i - 1] * v3
        else:
            v2 = v2 + (-alpha[i]) * v1
        beta[i] = np.linalg.norm(v2)
        v3 = v1.copy()
        v1 = v2 / beta[i]
        if i == mitr or (i >= minitr and i % itrint == 0):
            if i == 1:
                out = np.zeros(D, dtype=np.complex128)
                out[0] = 1.0
                return alpha[1], out, 1
            w, zz, info = lapack.dstev(alpha[1:i + 1].copy(), beta[1:i].copy(), compute_v=1)
            if info != 0:
                raise RuntimeError(f"error in dstevx, info = {info}")
            ene = w[0]
            conv = abs(tmp / ene - 1.0)
            if i == maxitr or conv < tol:
                z = zz[:, 0]
                ite = i
                break
            tmp = ene
    if z is None:
        # lanczos.f90:93-125 falls through with z deallocated here.
        raise NotConverged("lanczos: mitr reached without convergence")
    v1 = psi_io.copy()
    psi_io = psi_io * z[0]
    for i in range(1, ite):
        v2 = hv(v1)
        if i > 1:
            v2 = v2 - alpha[i] * v1 - beta[i - 1] * v3
        else:
            v2 = v2 - alpha[i] * v1
        v3 = v1.copy()
        v1 = v2 / beta[i]
        psi_io = psi_io + z[i] * v1
    psi_io = psi_io / np.linalg.norm(psi_io)
    return ene, psi_io, ite


def dsf_recursion(hv_new, fn0, itr_dsf, rfield, NOS, NOD_new):
    """calcu_DSF_wavevector (get_expectation_values.f90:486-592) from the
    unnormalised start vector fn0 = S^a(q)|GS> (calcu_Sq_a output).

    Returns (alpha[itr], beta2[itr], norm1, nlevels): alpha(n), beta_dsf(n) as
    written to the -tmp.d file (beta_dsf(1) = 0), nlevels = lines written.
    """
    D = len(fn0)
    la = max(itr_dsf, 1)
    alpha = np.full(la + 1, 1.0e300)
    beta = np.zeros(la + 2)
    norm1 = np.vdot(fn0, fn0).real
    fn = fn0 * (1.0 / np.sqrt(norm1))
    if np.linalg.norm(fn) - 1.0 > 1.0e-8:
        raise RuntimeError("<f1|f1> is not 1")
    sz_new = NOS / 2.0 - NOD_new
    fnp1 = hv_new(fn)
    fnp1 = fnp1 + (-rfield * sz_new) * fn
    alpha[1] = np.vdot(fn, fnp1).real
    beta[1] = 0.0
    nlev = 1
    if D > 1:
        fnp1 = fnp1 + (-alpha[1]) * fn
        beta[2] = np.vdot(fnp1, fnp1).real
        fnp1 = fnp1 * (1.0 / np.sqrt(beta[2]))
        for itr in range(2, itr_dsf + 1):
            fnm1 = fn
            fn = fnp1
            fnp1 = hv_new(fn)
            fnp1 = fnp1 + (-rfield * sz_new) * fn
            alpha[itr] = np.vdot(fn, fnp1).real
            nlev = itr
            if itr == D:
                break
            fnp1 = fnp1 - alpha[itr] * fn - np.sqrt(beta[itr]) * fnm1
            beta[itr + 1] = np.vdot(fnp1, fnp1).real
            fnp1 = fnp1 * (1.0 / np.sqrt(beta[itr + 1]))
    return alpha[1:nlev + 1].copy(), beta[1:nlev + 1].copy(), norm1, nlev
