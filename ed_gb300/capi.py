"""ctypes binding of libqs3g.so (include/qs3g.h).

This is the host-side view of the C ABI used by the tests and bench.py.  It
mirrors the QS3 module procedures it replaces: ``Handle.hv`` is
ham_to_vec_wave_vector (ham2vec_v3.f90:37-72), ``Handle.trlan`` is
lancz_eigen_val_complex (eigen_solver.f90:69-261), ``Handle.dsf`` is
calcu_Sq_a + calcu_DSF_wavevector (get_expectation_values.f90:281-605) and
``cfrac`` is DSFLan (source_DSFLan/main.f90).  Every call checks the status
code and raises :class:`QS3GError` with the library's message.

There is no CPU fallback: if the CUDA library cannot be loaded, the import of
this module's functions raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libqs3g.so")

OK, EINVAL, ENOMEM, ENOTCONV, EITERCAP, ECUDA, ESTATE, ERANGE, ENOTSUP, EBREAKDOWN = range(10)
HOST, DEVICE = 0, 1

EXPORTS = [
    "qs3g_create", "qs3g_destroy", "qs3g_build_sector", "qs3g_build_sector_u1", "qs3g_get_sector", "qs3g_hv", "qs3g_hv32",
    "qs3g_connection_table", "qs3g_connection_table_rows", "qs3g_trlan", "qs3g_lanczos", "qs3g_dsf",
    "qs3g_cfrac", "qs3g_last_error", "qs3g_kernel_launches", "qs3g_set_stream", "qs3g_sync",
    "qs3g_sq_a", "qs3g_cfrac_noalloc", "qs3g_correlations",
    "qs3g_write_wf", "qs3g_read_wf", "qs3g_write_energy", "qs3g_read_energy",
    "qs3g_write_alpha_beta", "qs3g_read_alpha_beta", "qs3g_format_real",
    "qs3g_full_hamiltonian", "qs3g_full_diag",
    "qs3g_mlp_create", "qs3g_mlp_destroy", "qs3g_mlp_params", "qs3g_mlp_add_sample", "qs3g_mlp_clear",
    "qs3g_mlp_loss_grad", "qs3g_mlp_train", "qs3g_mlp_align", "qs3g_mlp_predict", "qs3g_trlan_batch",
    "qs3g_trlan_lockstep", "qs3g_hv_schedule", "qs3g_hv_real", "qs3g_set_time_limit", "qs3g_trlan_stats",
    "qs3g_build_sector_i32", "qs3g_get_sector_i32", "qs3g_load_sector", "qs3g_load_sector_i32",
    "qs3g_hv32_real", "qs3g_hv_cache", "qs3g_hv_df",
]

MLP_NPARAMS = 35329
REAL = 8  # QS3G_REAL: added to a trlan precision for real Krylov vectors

_lib = None
_lock = threading.Lock()


class QS3GError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"qs3g error {code}: {msg}")
        self.code = code


def load(path: str | None = None):
    """Load the shared library (building it first if it is missing)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            from . import build as _b
            _b.build()
        L = C.CDLL(p)
        vp, ip, dp, i64p = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_int64)
        L.qs3g_last_error.restype = C.c_char_p
        L.qs3g_last_error.argtypes = [vp]
        L.qs3g_kernel_launches.restype = C.c_int64
        for name in EXPORTS:
            if name not in ("qs3g_last_error", "qs3g_kernel_launches"):
                getattr(L, name).restype = C.c_int
        L.qs3g_destroy.argtypes = [vp]
        _lib = L
        return L


def _i(v):
    return C.byref(C.c_int(int(v)))


def _d(v):
    return C.byref(C.c_double(float(v)))


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _check(rc, h=None):
    if rc != OK:
        msg = load().qs3g_last_error(h).decode(errors="replace")
        raise QS3GError(rc, msg)


def kernel_launches() -> int:
    return int(load().qs3g_kernel_launches())


class Handle:
    """One qs3g handle: lattice, bonds and the current sector."""

    def __init__(self, NOS, LX, LY, LZ, bonds, Jxy, Jz):
        L = load()
        bonds = np.ascontiguousarray(np.asarray(bonds, dtype=np.int32).reshape(-1, 2))
        self.NOS, self.LX, self.LY, self.LZ = int(NOS), int(LX), int(LY), int(LZ)
        self.NOxxz = bonds.shape[0]
        sJ = np.ascontiguousarray(np.concatenate([np.asarray(Jxy, np.float64) * 0.5,
                                                  np.asarray(Jz, np.float64) * 0.25]))
        h = C.c_void_p()
        rc = L.qs3g_create(C.byref(h), _i(self.NOS), _i(self.LX), _i(self.LY), _i(self.LZ),
                           _i(self.NOxxz), _ptr(bonds.reshape(-1)), _ptr(sJ))
        _check(rc, None)
        self.h = h
        self.D = None
        self.nod = None

    def close(self):
        if getattr(self, "h", None):
            load().qs3g_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_stream(self, stream_ptr: int):
        """Queue the handle's work on a caller-owned cudaStream_t (e.g. torch's)."""
        _check(load().qs3g_set_stream(self.h, C.c_void_p(stream_ptr)), self.h)

    def sync(self):
        _check(load().qs3g_sync(self.h), self.h)

    def build_sector(self, nod, K=(0, 0, 0)):
        D = C.c_int64()
        _check(load().qs3g_build_sector(self.h, _i(nod), _i(K[0]), _i(K[1]), _i(K[2]), C.byref(D)), self.h)
        self.D = int(D.value)
        self.nod = int(nod)
        return self.D

    def build_sector_u1(self, nod):
        """All C(NOS, nod) configurations, no translations (qs3g_build_sector_u1)."""
        D = C.c_int64()
        _check(load().qs3g_build_sector_u1(self.h, _i(nod), C.byref(D)), self.h)
        self.D = int(D.value)
        self.nod = int(nod)
        return self.D

    def build_sector_i32(self, nod, K=(0, 0, 0)):
        """qs3g_build_sector_i32: THS as a default-kind (32-bit) integer."""
        D = C.c_int()
        _check(load().qs3g_build_sector_i32(self.h, _i(nod), _i(K[0]), _i(K[1]), _i(K[2]), C.byref(D)), self.h)
        self.D = int(D.value)
        self.nod = int(nod)
        return self.D

    def load_sector(self, nod, K, list_s, list_r, i32=False):
        """qs3g_load_sector(_i32): adopt the caller's (list_s, list_r) of the (nod, K) sector."""
        ls = np.ascontiguousarray(list_s, np.int32 if i32 else np.int64)
        lr = np.ascontiguousarray(list_r, np.float64)
        if ls.shape != lr.shape or ls.ndim != 1:
            raise ValueError("list_s and list_r must be 1-D of the same length")
        if i32:
            rc = load().qs3g_load_sector_i32(self.h, _i(nod), _i(K[0]), _i(K[1]), _i(K[2]), _i(len(ls)), _ptr(ls),
                                             _ptr(lr))
        else:
            n = C.c_int64(len(ls))
            rc = load().qs3g_load_sector(self.h, _i(nod), _i(K[0]), _i(K[1]), _i(K[2]), C.byref(n), _ptr(ls),
                                         _ptr(lr))
        _check(rc, self.h)
        self.D = len(ls)
        self.nod = int(nod)
        return self.D

    def get_sector_i32(self):
        ls = np.zeros(self.D, np.int32)
        lr = np.zeros(self.D, np.float64)
        _check(load().qs3g_get_sector_i32(self.h, _ptr(ls), _ptr(lr)), self.h)
        return ls, lr

    def get_sector(self):
        ls = np.zeros(self.D, np.int64)
        lr = np.zeros(self.D, np.float64)
        _check(load().qs3g_get_sector(self.h, _ptr(ls), _ptr(lr)), self.h)
        return ls, lr

    def hv(self, x):
        x = np.ascontiguousarray(x, dtype=np.complex128)
        assert x.shape == (self.D,)
        y = np.zeros(self.D, np.complex128)
        _check(load().qs3g_hv(self.h, _ptr(y), _ptr(x), _i(HOST)), self.h)
        return y

    def hv_host_into(self, x, y):
        """y = H x through the host-pointer form (x, y: complex128 arrays, e.g. pinned)."""
        assert x.dtype == np.complex128 and y.dtype == np.complex128
        assert x.flags.c_contiguous and y.flags.c_contiguous
        _check(load().qs3g_hv(self.h, _ptr(y), _ptr(x), _i(HOST)), self.h)

    def connection_table_count(self):
        nnz = C.c_int64(0)
        _check(load().qs3g_connection_table(self.h, None, None, None, None, C.byref(nnz)), self.h)
        return int(nnz.value)

    def hv_device(self, x_ptr: int, y_ptr: int):
        """y = H x for device pointers (complex128), on the handle's stream."""
        _check(load().qs3g_hv(self.h, C.c_void_p(y_ptr), C.c_void_p(x_ptr), _i(DEVICE)), self.h)

    def hv32(self, x):
        x = np.ascontiguousarray(x, dtype=np.complex64)
        y = np.zeros(self.D, np.complex64)
        _check(load().qs3g_hv32(self.h, _ptr(y), _ptr(x), _i(HOST)), self.h)
        return y

    def hv_real(self, x):
        """y = H x for a real vector x (sectors whose H is real symmetric)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        assert x.shape == (self.D,)
        y = np.zeros(self.D, np.float64)
        _check(load().qs3g_hv_real(self.h, _ptr(y), _ptr(x), _i(HOST)), self.h)
        return y

    def hv32_real(self, x, shift=0.0):
        """y = (H - shift) x in FP32 for a real vector x (sectors whose H is real symmetric)."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        assert x.shape == (self.D,)
        y = np.zeros(self.D, np.float32)
        sh = C.c_float(float(shift))
        _check(load().qs3g_hv32_real(self.h, _ptr(y), _ptr(x), C.byref(sh), _i(HOST)), self.h)
        return y

    def hv32_real_device(self, x_ptr: int, y_ptr: int, shift=0.0):
        sh = C.c_float(float(shift))
        _check(load().qs3g_hv32_real(self.h, C.c_void_p(y_ptr), C.c_void_p(x_ptr), C.byref(sh), _i(DEVICE)), self.h)

    def hv_real_device(self, x_ptr: int, y_ptr: int):
        _check(load().qs3g_hv_real(self.h, C.c_void_p(y_ptr), C.c_void_p(x_ptr), _i(DEVICE)), self.h)

    def hv32_device(self, x_ptr: int, y_ptr: int):
        _check(load().qs3g_hv32(self.h, C.c_void_p(y_ptr), C.c_void_p(x_ptr), _i(DEVICE)), self.h)

    def connection_table(self, rows=None):
        L = load()
        nnz = C.c_int64(0)
        if rows is None:
            _check(L.qs3g_connection_table(self.h, None, None, None, None, C.byref(nnz)), self.h)
        else:
            r0, r1 = C.c_int64(rows[0] + 1), C.c_int64(rows[1])
            _check(L.qs3g_connection_table_rows(self.h, C.byref(r0), C.byref(r1), None, None, None,
                                                None, C.byref(nnz)), self.h)
        n = int(nnz.value)
        row = np.zeros(n, np.int64)
        col = np.zeros(n, np.int64)
        ell = np.zeros((n, 3), np.int32)
        bond = np.zeros(n, np.int32)
        if n:
            if rows is None:
                _check(L.qs3g_connection_table(self.h, _ptr(row), _ptr(col), _ptr(ell), _ptr(bond),
                                               C.byref(nnz)), self.h)
            else:
                _check(L.qs3g_connection_table_rows(self.h, C.byref(r0), C.byref(r1), _ptr(row),
                                                    _ptr(col), _ptr(ell), _ptr(bond), C.byref(nnz)),
                       self.h)
        return row, col, ell, bond

    def trlan(self, NOE, NOK, NOM, maxitr=10000, tol=1e-12, precision=0, conv_mode=0, seed=1,
              start=None, want_psi=True, allow_unconverged=False, real=False):
        """qs3g_trlan; real=True adds QS3G_REAL (real Krylov vectors)."""
        if real:
            precision |= REAL
        ene = np.zeros(NOE)
        psi = np.zeros((NOE, self.D), np.complex128) if want_psi else None
        resid = np.zeros(NOE)
        iters = C.c_int(0)
        st = None if start is None else np.ascontiguousarray(start, np.complex128)
        sd = C.c_uint64(int(seed))
        rc = load().qs3g_trlan(self.h, _i(NOE), _i(NOK), _i(NOM), _i(maxitr), _d(tol), _i(precision),
                               _i(conv_mode), _i(0 if st is None else 1), C.byref(sd), _ptr(st),
                               _ptr(ene), _ptr(psi), C.byref(iters), _ptr(resid))
        if rc == ENOTCONV and allow_unconverged:
            pass
        else:
            _check(rc, self.h)
        return dict(ene=ene, psi=psi, iters=int(iters.value), resid=resid, converged=(rc == OK))

    def hv_df(self, x):
        """H x from the cached connection table in double-float arithmetic."""
        x = np.ascontiguousarray(x, np.complex128)
        y = np.empty_like(x)
        _check(load().qs3g_hv_df(self.h, _ptr(y), _ptr(x), _i(HOST)), self.h)
        return y

    def hv_df_device(self, x_ptr: int, y_ptr: int):
        _check(load().qs3g_hv_df(self.h, C.c_void_p(y_ptr), C.c_void_p(x_ptr), _i(DEVICE)), self.h)

    def hv_cache(self, on=True):
        """Cache (or drop) the sector's connection table on the device; returns its bytes."""
        nb = C.c_int64(0)
        _check(load().qs3g_hv_cache(self.h, _i(1 if on else 0), C.byref(nb)), self.h)
        return int(nb.value)

    def set_time_limit(self, seconds):
        """Wall-clock limit of later trlan calls on this handle (0 = none)."""
        _check(load().qs3g_set_time_limit(self.h, _d(seconds)), self.h)

    def trlan_stats(self):
        """What the last trlan call did: H*v on complex(4) / complex(8) vectors, restarts, seconds."""
        a, b, r, to = C.c_int(0), C.c_int(0), C.c_int(0), C.c_int(0)
        sec = C.c_double(0.0)
        _check(load().qs3g_trlan_stats(self.h, C.byref(a), C.byref(b), C.byref(r), C.byref(sec), C.byref(to)),
               self.h)
        return dict(hv_fp32=int(a.value), hv_fp64=int(b.value), restarts=int(r.value), seconds=float(sec.value),
                    timed_out=bool(to.value))

    def lanczos(self, maxitr=10000, minitr=20, itrint=5, tol=1e-14, seed=1, start=None):
        ene = np.zeros(1)
        psi = np.zeros(self.D, np.complex128)
        iters = C.c_int(0)
        st = None if start is None else np.ascontiguousarray(start, np.complex128)
        sd = C.c_uint64(int(seed))
        _check(load().qs3g_lanczos(self.h, _i(maxitr), _i(minitr), _i(itrint), _d(tol),
                                   _i(0 if st is None else 1), C.byref(sd), _ptr(st), _ptr(ene),
                                   _ptr(psi), C.byref(iters)), self.h)
        return dict(ene=float(ene[0]), psi=psi, iters=int(iters.value))

    def dsf(self, psi, ene1, spsmsz, qvecs, Spos, itr_dsf, rfield=0.0):
        qv = np.ascontiguousarray(np.asarray(qvecs, np.float64).reshape(-1, 3))
        nq = qv.shape[0]
        sp = np.ascontiguousarray(np.asarray(Spos, np.float64).reshape(-1))
        alpha = np.zeros((nq, itr_dsf))
        beta2 = np.zeros((nq, itr_dsf))
        norm1 = np.zeros(nq)
        E0 = np.zeros(nq)
        nlev = np.zeros(nq, np.int32)
        psi = np.ascontiguousarray(psi, np.complex128)
        _check(load().qs3g_dsf(self.h, _ptr(psi), _d(ene1), _i(spsmsz), _i(nq), _ptr(qv.reshape(-1)),
                               _ptr(sp), _i(itr_dsf), _d(rfield), _ptr(alpha), _ptr(beta2),
                               _ptr(norm1), _ptr(E0), _ptr(nlev)), self.h)
        return dict(alpha=alpha, beta2=beta2, norm1=norm1, E0=E0, nlev=nlev)


def _sq_a(h, psi, spsmsz, qvec, Spos):
    psi = np.ascontiguousarray(psi, np.complex128)
    qv = np.ascontiguousarray(np.asarray(qvec, np.float64).reshape(3))
    sp = np.ascontiguousarray(np.asarray(Spos, np.float64).reshape(-1))
    Dn = C.c_int64(0)
    _check(load().qs3g_sq_a(h.h, _ptr(psi), _i(spsmsz), _ptr(qv), _ptr(sp), C.byref(Dn), None, None), h.h)
    n = int(Dn.value)
    ls = np.zeros(n, np.int64)
    fn = np.zeros(n, np.complex128)
    _check(load().qs3g_sq_a(h.h, _ptr(psi), _i(spsmsz), _ptr(qv), _ptr(sp), C.byref(Dn), _ptr(ls), _ptr(fn)),
           h.h)
    return ls, fn


Handle.sq_a = lambda self, psi, spsmsz, qvec, Spos: _sq_a(self, psi, spsmsz, qvec, Spos)


def _correlations(h, psi):
    """(szsz, spsm, lm): szsz[a-1, b-1] = <Sz_a Sz_b>, spsm[a-1, b-1] = <S+_a S-_b>, lm = <Sz_i>."""
    psi = np.ascontiguousarray(psi, np.complex128)
    n = h.NOS
    zz = np.zeros(n * n)
    pm = np.zeros(n * n, np.complex128)
    lm = np.zeros(n)
    _check(load().qs3g_correlations(h.h, _ptr(psi), _ptr(zz), _ptr(pm), _ptr(lm)), h.h)
    # flat index (a-1) + (b-1)*NOS  ->  [a-1, b-1]
    return zz.reshape(n, n).T.copy(), pm.reshape(n, n).T.copy(), lm


Handle.correlations = _correlations


def _cfrac_args(alpha, beta2, nlev, norm1, E0, omega):
    """Shape-checked contiguous copies of the continued-fraction inputs: alpha and
    beta2 (nq, ldab), nlev / norm1 / E0 with nq entries (the C side reads nq of
    each), omega 1-D."""
    alpha = np.ascontiguousarray(np.atleast_2d(alpha), np.float64)
    beta2 = np.ascontiguousarray(np.atleast_2d(beta2), np.float64)
    nq = alpha.shape[0]
    nlev = np.ascontiguousarray(np.atleast_1d(nlev), np.int32)
    norm1 = np.ascontiguousarray(np.atleast_1d(norm1), np.float64)
    E0 = np.ascontiguousarray(np.atleast_1d(E0), np.float64)
    omega = np.ascontiguousarray(omega, np.float64)
    if beta2.shape != alpha.shape:
        raise ValueError(f"beta2 has shape {beta2.shape}, alpha {alpha.shape}")
    for name, a in (("nlev", nlev), ("norm1", norm1), ("E0", E0)):
        if a.ndim != 1 or a.size != nq:
            raise ValueError(f"{name} needs {nq} entries (one per spectrum), got shape {a.shape}")
    if omega.ndim != 1:
        raise ValueError("omega must be one-dimensional")
    return alpha, beta2, nlev, norm1, E0, omega


def cfrac(alpha, beta2, nlev, norm1, E0, eta, omega, compat=True):
    """DSFLan continued fraction for nq spectra: alpha/beta2 are (nq, ldab)."""
    alpha, beta2, nlev, norm1, E0, omega = _cfrac_args(alpha, beta2, nlev, norm1, E0, omega)
    nq, ld = alpha.shape
    S = np.zeros((nq, len(omega)))
    _check(load().qs3g_cfrac(_i(nq), _i(ld), _ptr(nlev), _ptr(alpha), _ptr(beta2), _ptr(norm1),
                             _ptr(E0), _d(eta), _i(len(omega)), _ptr(omega), _i(1 if compat else 0),
                             _ptr(S)))
    return S


def cfrac_noalloc(alpha, beta2, nlev, norm1, E0, eta, omega, compat=True):
    """qs3g_cfrac_noalloc: the same continued fraction, staged in the library's
    static device array instead of allocated buffers (for callers that cannot
    allocate device memory)."""
    alpha, beta2, nlev, norm1, E0, omega = _cfrac_args(alpha, beta2, nlev, norm1, E0, omega)
    nq, ld = alpha.shape
    S = np.zeros((nq, len(omega)))
    _check(load().qs3g_cfrac_noalloc(_i(nq), _i(ld), _ptr(nlev), _ptr(alpha), _ptr(beta2), _ptr(norm1),
                                     _ptr(E0), _d(eta), _i(len(omega)), _ptr(omega),
                                     _i(1 if compat else 0), _ptr(S)))
    return S


def cfrac_noalloc_doubles(nq, ldab, nomega):
    """Doubles of the static area one qs3g_cfrac_noalloc call stages (each region
    rounded up to 32 doubles): alpha and beta2 (nq*ldab each), norm1 and E0 (nq
    each), omega, S (nq*nomega) and nlev (ceil(nq/2) doubles of int32 pairs).
    The call is accepted when this is at most 524,288."""
    up32 = lambda n: (n + 31) // 32 * 32
    return (2 * up32(nq * ldab) + 2 * up32(nq) + up32(nomega) + up32(nq * nomega) + up32((nq + 1) // 2))


def _full_hamiltonian(h):
    """Dense H(i, id) of the current sector (make_full_hamiltonian), shape (D, D)."""
    H = np.zeros((h.D, h.D), np.complex128, order="F")
    _check(load().qs3g_full_hamiltonian(h.h, _ptr(H)), h.h)
    return H


def _full_diag(h, want_psi=True):
    """All eigenpairs (ALG = 3): (ene[D], psi[D, D] with eigenvectors as columns)."""
    ene = np.zeros(h.D)
    psi = np.zeros((h.D, h.D), np.complex128, order="F") if want_psi else None
    _check(load().qs3g_full_diag(h.h, _ptr(ene), _ptr(psi)), h.h)
    return ene, psi


Handle.full_hamiltonian = _full_hamiltonian
Handle.full_diag = _full_diag


def _hv_schedule(h, mode=None):
    """Set (0 auto, 1 warp per row, 2 thread per row) and/or read the
    general-lattice H*v schedule of the current sector: (complex(8), complex(4))."""
    chosen = (C.c_int * 2)()
    _check(load().qs3g_hv_schedule(h.h, None if mode is None else _i(mode), chosen), h.h)
    return int(chosen[0]), int(chosen[1])


Handle.hv_schedule = _hv_schedule


def trlan_batch(handles, NOE, NOK, NOM, maxitr=10000, tol=1e-10, precision=1, conv_mode=1, seed=1,
                nthreads=8):
    """qs3g_trlan_batch over handles with built sectors: (ene[n, NOE], iters[n], resid[n, NOE], status[n])."""
    n = len(handles)
    arr = (C.c_void_p * max(1, n))(*[h.h.value if isinstance(h.h, C.c_void_p) else h.h for h in handles])
    ene = np.zeros((n, NOE))
    resid = np.zeros((n, NOE))
    iters = np.zeros(n, np.int32)
    status = np.zeros(n, np.int32)
    rc = load().qs3g_trlan_batch(_i(n), arr, _i(NOE), _i(NOK), _i(NOM), _i(maxitr), _d(tol), _i(precision),
                                 _i(conv_mode), C.byref(C.c_uint64(seed)), _i(nthreads), _ptr(ene), _ptr(iters),
                                 _ptr(resid), _ptr(status))
    if rc not in (OK, ENOTCONV):
        _check(rc, None)
    return ene, iters, resid, status


def trlan_lockstep(handles, NOE, NOK, NOM, maxitr=10000, tol=1e-10, precision=1, conv_mode=1, seed=1):
    """qs3g_trlan_lockstep over chain handles with built sectors: (ene, iters, resid, status)."""
    n = len(handles)
    arr = (C.c_void_p * max(1, n))(*[h.h.value if isinstance(h.h, C.c_void_p) else h.h for h in handles])
    ene = np.zeros((n, NOE))
    resid = np.zeros((n, NOE))
    iters = np.zeros(n, np.int32)
    status = np.zeros(n, np.int32)
    rc = load().qs3g_trlan_lockstep(_i(n), arr, _i(NOE), _i(NOK), _i(NOM), _i(maxitr), _d(tol), _i(precision),
                                    _i(conv_mode), C.byref(C.c_uint64(seed)), _ptr(ene), _ptr(iters), _ptr(resid),
                                    _ptr(status))
    if rc not in (OK, ENOTCONV):
        _check(rc, None)
    return ene, iters, resid, status


# ---------------------------------------------------------------- learned start
def band_minimum(J1xy, J2xy):
    """Wave number of the single-magnon band minimum of J1xy cos q + J2xy cos 2q (J1xy > 0)."""
    if J2xy <= 0.25 * J1xy:
        return float(np.pi)
    return float(np.arccos(-J1xy / (4.0 * J2xy)))


class Mlp:
    """The learned start-vector network (qs3g_mlp_*)."""

    def __init__(self, seed=1):
        self.h = C.c_void_p()
        _check(load().qs3g_mlp_create(C.byref(self.h), C.byref(C.c_uint64(seed))), None)

    def close(self):
        if self.h:
            load().qs3g_mlp_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self):
        p = np.zeros(MLP_NPARAMS)
        _check(load().qs3g_mlp_params(self.h, _ptr(p), None), None)
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float64)
        assert p.shape == (MLP_NPARAMS,)
        _check(load().qs3g_mlp_params(self.h, None, _ptr(p)), None)

    def add_sample(self, handle, psi, delta, j2, q0):
        psi = np.ascontiguousarray(psi, np.complex128)
        cond = np.array([delta, j2, q0], np.float64)
        _check(load().qs3g_mlp_add_sample(self.h, handle.h, _ptr(psi), _ptr(cond)), handle.h)

    def clear(self):
        _check(load().qs3g_mlp_clear(self.h), None)

    def loss_grad(self):
        loss = C.c_double()
        g = np.zeros(MLP_NPARAMS)
        _check(load().qs3g_mlp_loss_grad(self.h, C.byref(loss), _ptr(g)), None)
        return loss.value, g

    def train(self, steps, batch, lr, seed=1):
        losses = np.zeros(max(1, steps))
        _check(load().qs3g_mlp_train(self.h, _i(steps), C.byref(C.c_int64(batch)), C.byref(C.c_double(lr)),
                                     C.byref(C.c_uint64(seed)), _ptr(losses)), None)
        return losses[:steps]

    def align(self):
        n = C.c_int()
        _check(load().qs3g_mlp_align(self.h, C.byref(n)), None)
        return n.value

    def predict(self, handle, delta, j2, q0):
        cond = np.array([delta, j2, q0], np.float64)
        v = np.zeros(handle.D, np.complex128)
        _check(load().qs3g_mlp_predict(self.h, handle.h, _ptr(cond), _ptr(v), _i(HOST)), handle.h)
        return v

    def predict_device(self, handle, delta, j2, q0, v_ptr: int):
        """The prediction into a device array of handle.D complex(8) values."""
        cond = np.array([delta, j2, q0], np.float64)
        _check(load().qs3g_mlp_predict(self.h, handle.h, _ptr(cond), C.c_void_p(v_ptr), _i(DEVICE)), handle.h)


# ---------------------------------------------------------------- result files
def _path(p):
    return os.fsencode(p)


def write_wf(path, psi):
    """wf<i>.bin: psi as one Fortran unformatted record of complex(8)."""
    psi = np.ascontiguousarray(psi, np.complex128)
    _check(load().qs3g_write_wf(_path(path), C.byref(C.c_int64(psi.size)), _ptr(psi)), None)


def read_wf(path, dim):
    psi = np.zeros(int(dim), np.complex128)
    _check(load().qs3g_read_wf(_path(path), C.byref(C.c_int64(int(dim))), _ptr(psi)), None)
    return psi


def write_energy(path, ene):
    ene = np.ascontiguousarray(ene, np.float64)
    _check(load().qs3g_write_energy(_path(path), _i(ene.size), _ptr(ene)), None)


def read_energy(path, noe):
    ene = np.zeros(int(noe))
    _check(load().qs3g_read_energy(_path(path), _i(noe), _ptr(ene)), None)
    return ene


def write_alpha_beta(path, alpha, beta2, norm1, E0, sztot, ex_i=1, itr=1, append=True):
    """alpha_beta_values_*.d lines (3I6, 8e23.15) for levels 1..len(alpha)."""
    alpha = np.ascontiguousarray(alpha, np.float64)
    beta2 = np.ascontiguousarray(beta2, np.float64)
    assert alpha.shape == beta2.shape
    _check(load().qs3g_write_alpha_beta(_path(path), _i(alpha.size), _i(ex_i), _i(itr), _ptr(alpha), _ptr(beta2),
                                        C.byref(C.c_double(norm1)), C.byref(C.c_double(E0)),
                                        C.byref(C.c_double(sztot)), _i(1 if append else 0)), None)


def read_alpha_beta(path, cap=4000):
    """(alpha, beta2, norm1, E0, sztot) as DSFLan's list-directed read sees them."""
    alpha = np.zeros(cap)
    beta2 = np.zeros(cap)
    n1, e0, sz = C.c_double(), C.c_double(), C.c_double()
    n = C.c_int()
    _check(load().qs3g_read_alpha_beta(_path(path), _i(cap), _ptr(alpha), _ptr(beta2), C.byref(n1), C.byref(e0),
                                       C.byref(sz), C.byref(n)), None)
    k = n.value
    return alpha[:k].copy(), beta2[:k].copy(), n1.value, e0.value, sz.value


def format_real(x, w, d, kind="E"):
    """Fortran Ew.d (kind 'E') or ESw.d (kind 'ES') of x."""
    out = C.create_string_buffer(w + 1)
    _check(load().qs3g_format_real(C.byref(C.c_double(x)), _i(1 if kind == "ES" else 0), _i(w), _i(d), out), None)
    return out.value.decode()
