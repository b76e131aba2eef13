"""ctypes front end of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

This module loads ``oracle/_build/libqs3oracle.so`` (compiled from
``qs3_oracle.cpp`` by :func:`build`) and wraps its functions with numpy
arrays.  Only the tests, ``__graft_entry__.smoke()`` and the CPU legs of
``bench.py`` use it, and only to compare against or as the CPU baseline;
the product library never imports it.

Each wrapper names the QS3 routine it restates (paths relative to the
QS-Cube/ED source tree).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libqs3oracle.so")
SRC = os.path.join(HERE, "qs3_oracle.cpp")

_lib = None
_lock = threading.Lock()

i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (OpenMP, no FMA contraction)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(SRC)):
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           SRC, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        build()
        L = C.CDLL(LIB_PATH)
        L.ora_model_new.restype = C.c_void_p
        L.ora_model_new.argtypes = [C.c_int] * 5 + [i32p, f64p, C.c_int]
        L.ora_model_free.argtypes = [C.c_void_p]
        L.ora_binom.restype = C.c_int64
        L.ora_binom.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.ora_wavevector.argtypes = [C.c_int] * 6 + [f64p]
        L.ora_explist.argtypes = [f64p, C.c_int, C.c_int, C.c_int, f64p]
        L.ora_list_fly.argtypes = [C.c_void_p, C.c_int64, C.c_int, i32p]
        L.ora_inv_list.restype = C.c_int64
        L.ora_inv_list.argtypes = [C.c_void_p, i32p, C.c_int]
        L.ora_representative.restype = C.c_int64
        L.ora_representative.argtypes = [C.c_void_p, C.c_int, i32p, i32p]
        L.ora_j_flip.argtypes = [C.c_int, C.c_int, i32p, C.c_int, i32p]
        L.ora_checkstate.restype = C.c_double
        L.ora_checkstate.argtypes = [C.c_void_p, C.c_int64, C.c_int, f64p]
        L.ora_build_sector.restype = C.c_int64
        L.ora_build_sector.argtypes = [C.c_void_p, C.c_int, f64p, C.c_void_p, C.c_void_p,
                                       C.c_int64, C.c_int]
        L.ora_hv.argtypes = [C.c_void_p, C.c_int, C.c_int64, i64p, f64p, f64p, f64p, f64p,
                             C.c_int64, C.c_int64, C.c_int]
        L.ora_connection_table.restype = C.c_int64
        L.ora_connection_table.argtypes = [C.c_void_p, C.c_int, C.c_int64, i64p, C.c_void_p,
                                           C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                                           C.c_int]
        L.ora_connection_table_rows.restype = C.c_int64
        L.ora_connection_table_rows.argtypes = [C.c_void_p, C.c_int, C.c_int64, i64p, C.c_int64,
                                                C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                                C.c_void_p, C.c_int64, C.c_int]
        L.ora_sq_a.restype = C.c_int
        L.ora_sq_a.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int64, i64p, f64p, C.c_int,
                               C.c_int64, i64p, f64p, f64p, f64p, f64p, f64p, f64p, C.c_int]
        L.ora_corr.restype = C.c_int
        L.ora_corr.argtypes = [C.c_void_p, C.c_int, C.c_int64, i64p, f64p, f64p, f64p, i32p,
                               C.c_int, f64p, f64p, C.c_int]
        L.ora_count_offdiag.restype = C.c_int64
        L.ora_count_offdiag.argtypes = [C.c_void_p, C.c_int, C.c_int64, i64p, C.c_int64, C.c_int64,
                                        C.c_int]
        L.ora_chain_sector.restype = C.c_int64
        L.ora_chain_sector.argtypes = [C.c_void_p, C.c_int, f64p, C.c_void_p, C.c_void_p,
                                       C.c_int64, C.c_int]
        L.ora_u1_hv.argtypes = [C.c_void_p, C.c_int, f64p, f64p, C.c_int64, C.c_int64, C.c_int]
        L.ora_u1_corr.restype = C.c_int
        L.ora_u1_corr.argtypes = [C.c_void_p, C.c_int, f64p, f64p, f64p, f64p, C.c_int]
        L.ora_u1_sq_a.restype = C.c_int
        L.ora_u1_sq_a.argtypes = [C.c_void_p, C.c_int, C.c_int, f64p, f64p, f64p, f64p]
        L.ora_cfrac.restype = C.c_int
        L.ora_cfrac.argtypes = [C.c_int, f64p, f64p, C.c_double, C.c_double, C.c_double,
                                C.c_int, f64p, C.c_int, f64p]
        _lib = L
        return L


def _c(a):
    return np.ascontiguousarray(a).view(np.float64) if np.iscomplexobj(a) else a


def wavevector(K, Ls):
    """rk = 2*pi*K/L (input_param.f90:76-78)."""
    out = np.zeros(3)
    lib().ora_wavevector(int(K[0]), int(K[1]), int(K[2]), int(Ls[0]), int(Ls[1]), int(Ls[2]), out)
    return out


def explist(rk, Ls):
    """explist(0:LX,0:LY,0:LZ) (input_param.f90:87-89), Fortran order, complex."""
    LX, LY, LZ = Ls
    out = np.zeros(2 * (LX + 1) * (LY + 1) * (LZ + 1))
    lib().ora_explist(np.ascontiguousarray(rk, dtype=np.float64), LX, LY, LZ, out)
    return out.view(np.complex128)


class Model:
    """Module globals of input_param (NOS, LX/LY/LZ, p_xxz, sJint, shift tables, combination)."""

    def __init__(self, NOS, LX, LY, LZ, bonds, Jxy, Jz, kmax=None):
        bonds = np.asarray(bonds, dtype=np.int32).reshape(-1, 2)
        self.NOS, self.LX, self.LY, self.LZ = int(NOS), int(LX), int(LY), int(LZ)
        self.NOxxz = bonds.shape[0]
        self.bonds = bonds.copy()
        self.Jxy = np.asarray(Jxy, dtype=np.float64).copy()
        self.Jz = np.asarray(Jz, dtype=np.float64).copy()
        self.kmax = int(kmax) if kmax is not None else min(self.NOS, 16)
        J = np.concatenate([self.Jxy, self.Jz])
        self.h = lib().ora_model_new(self.NOS, self.LX, self.LY, self.LZ, self.NOxxz,
                                     np.ascontiguousarray(bonds.reshape(-1)), J, self.kmax)
        if not self.h:
            raise ValueError("oracle: invalid model")

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ora_model_free(self.h)
            self.h = None

    @property
    def Ls(self):
        return (self.LX, self.LY, self.LZ)

    def binom(self, n, k):
        return lib().ora_binom(self.h, n, k)

    def list_fly(self, t, nod):
        n = np.zeros(nod, dtype=np.int32)
        lib().ora_list_fly(self.h, int(t), nod, n)
        return n

    def inv_list(self, n):
        n = np.ascontiguousarray(n, dtype=np.int32)
        return lib().ora_inv_list(self.h, n, len(n))

    def representative(self, n):
        n = np.array(n, dtype=np.int32)
        ell = np.zeros(3, dtype=np.int32)
        t = lib().ora_representative(self.h, len(n), n, ell)
        return t, n, ell

    def checkstate(self, s, nod, rk):
        return lib().ora_checkstate(self.h, int(s), nod, np.ascontiguousarray(rk, np.float64))

    def build_sector(self, nod, K, nthreads=0):
        """allocate_lists_omp_SQ (state_lists.f90:225-292) -> (list_s, list_r)."""
        rk = wavevector(K, self.Ls)
        D = lib().ora_build_sector(self.h, nod, rk, None, None, 0, nthreads)
        if D < 0:
            raise ValueError("oracle: sector too large")
        ls = np.zeros(D, dtype=np.int64)
        lr = np.zeros(D, dtype=np.float64)
        D2 = lib().ora_build_sector(self.h, nod, rk, ls.ctypes.data, lr.ctypes.data, D, nthreads)
        assert D2 == D
        return Sector(self, nod, K, ls, lr)


class Sector:
    """A (NOD, K) sector: list_s, list_r, explist."""

    def __init__(self, model, nod, K, list_s, list_r, rk=None):
        self.model = model
        self.nod = int(nod)
        self.K = tuple(int(k) for k in K)
        self.list_s = np.ascontiguousarray(list_s, dtype=np.int64)
        self.list_r = np.ascontiguousarray(list_r, dtype=np.float64)
        self.rk = wavevector(self.K, model.Ls) if rk is None else np.asarray(rk, np.float64)
        self.explist = explist(self.rk, model.Ls)

    @property
    def D(self):
        return len(self.list_s)

    def hv(self, x, rows=None, nthreads=0):
        """ham_to_vec_wave_vector (ham2vec_v3.f90:37-72)."""
        x = np.ascontiguousarray(x, dtype=np.complex128)
        y = np.zeros(self.D, dtype=np.complex128)
        r0, r1 = (0, self.D) if rows is None else rows
        lib().ora_hv(self.model.h, self.nod, self.D, self.list_s, self.list_r,
                     self.explist.view(np.float64), x.view(np.float64), y.view(np.float64),
                     r0, r1, nthreads)
        return y

    def connection_table(self, nthreads=0, rows=None):
        """Connection table of ham_to_vec_wave_vector, optionally of rows [r0, r1) only
        (0-based rows, columns and bonds)."""
        L = lib()
        r0, r1 = (0, self.D) if rows is None else (int(rows[0]), int(rows[1]))
        nnz = L.ora_connection_table_rows(self.model.h, self.nod, self.D, self.list_s, r0, r1,
                                          None, None, None, None, 0, nthreads)
        if nnz < 0:
            raise ValueError("oracle: bad row range")
        row = np.zeros(nnz, np.int64)
        col = np.zeros(nnz, np.int64)
        ell = np.zeros((nnz, 3), np.int32)
        bond = np.zeros(nnz, np.int32)
        n2 = L.ora_connection_table_rows(self.model.h, self.nod, self.D, self.list_s, r0, r1,
                                         row.ctypes.data, col.ctypes.data, ell.ctypes.data,
                                         bond.ctypes.data, nnz, nthreads)
        assert n2 == nnz
        return row, col, ell, bond

    def sparse(self, nthreads=0):
        """H of the sector as a scipy CSR matrix: one entry per connection-table hop with the
        coefficient sJint(j,2) * list_r(id) / list_r(i) * explist(ell) of ham2vec_v3.f90:61-65
        (entries of the same (row, col) summed), plus the diagonal of :60,67 read off one
        oracle H*v of the all-ones vector.  For solver checks at sizes where dense() is too slow."""
        import scipy.sparse as sp
        m = self.model
        D = self.D
        row, col, ell, bond = self.connection_table(nthreads)
        ex1 = m.LX + 1
        ex2 = ex1 * (m.LY + 1)
        e = self.explist[ell[:, 0] + ex1 * ell[:, 1] + ex2 * ell[:, 2]]
        c = (0.5 * m.Jxy[bond]) * self.list_r[col] / self.list_r[row]
        off = sp.csr_matrix((c * e, (row, col)), shape=(D, D))
        ones = np.ones(D, np.complex128)
        diag = (self.hv(ones, nthreads=nthreads) - off @ ones).real
        return (off + sp.diags(diag)).tocsr()

    def dense(self):
        """make_full_hamiltonian (ham2vec_v3.f90:5-35) built column by column through hv."""
        D = self.D
        H = np.zeros((D, D), dtype=np.complex128)
        e = np.zeros(D, dtype=np.complex128)
        for j in range(D):
            e[:] = 0
            e[j] = 1.0
            H[:, j] = self.hv(e)
        return H

    def corr(self, v, ss=None, nthreads=0):
        """get_cf_2_wave_vector / calcu_cf_trans_2 for all NOS*NOS ordered pairs.

        Returns (szsz, spsm) as (NOS, NOS) arrays S[a-1, b-1] for the FILECF line
        'a b' (list_expe_ss(2) = a, list_expe_ss(1) = b): <Sz_a Sz_b> and <S+_a S-_b>.
        """
        NOS = self.model.NOS
        if ss is None:
            a, b = np.meshgrid(np.arange(1, NOS + 1), np.arange(1, NOS + 1), indexing="ij")
            ss = np.stack([b.reshape(-1), a.reshape(-1)], axis=1)  # (ss1, ss2) per line
        ss = np.ascontiguousarray(np.asarray(ss, dtype=np.int32).reshape(-1))
        szsz = np.zeros(NOS * NOS)
        spsm = np.zeros(NOS * NOS, dtype=np.complex128)
        v = np.ascontiguousarray(v, dtype=np.complex128)
        rc = lib().ora_corr(self.model.h, self.nod, self.D, self.list_s, self.list_r,
                            self.explist.view(np.float64), v.view(np.float64), ss, NOS * NOS,
                            szsz, spsm.view(np.float64), nthreads)
        if rc != 0:
            raise ValueError("oracle: corr failed")
        # flat index p = ss1 + (ss2-1)*NOS - 1 = (a-1)*NOS + (b-1)
        return szsz.reshape(NOS, NOS), spsm.reshape(NOS, NOS)


def count_offdiag_rows(sec: Sector, r0, r1, nthreads=0):
    """nnz_off of rows [r0, r1) (connection-table entries)."""
    return int(lib().ora_count_offdiag(sec.model.h, sec.nod, sec.D, sec.list_s, int(r0), int(r1),
                                       nthreads))


def chain_sector_lists(L, nod, K=0, nthreads=0, bonds=None):
    """(list_s, list_r) of a chain sector by anchored enumeration (no bonds needed)."""
    if bonds is None:
        bonds = np.array([[1, 2]], np.int32)
    m = Model(L, L, 1, 1, bonds, np.ones(len(bonds)), np.ones(len(bonds)), kmax=nod + 2)
    rk = wavevector((K, 0, 0), m.Ls)
    D = lib().ora_chain_sector(m.h, nod, rk, None, None, 0, nthreads)
    if D < 0:
        raise ValueError("oracle: chain sector unsupported")
    ls = np.zeros(D, np.int64)
    lr = np.zeros(D)
    lib().ora_chain_sector(m.h, nod, rk, ls.ctypes.data, lr.ctypes.data, D, nthreads)
    return ls, lr


def sq_a(spsmsz, gs: Sector, new: Sector, qvec, Spos, psi, nthreads=0):
    """calcu_Sq_a (get_expectation_values.f90:281-377)."""
    m = gs.model
    fn = np.zeros(new.D, dtype=np.complex128)
    psi = np.ascontiguousarray(psi, dtype=np.complex128)
    rc = lib().ora_sq_a(m.h, spsmsz, gs.nod, gs.D, gs.list_s, gs.list_r, new.nod, new.D,
                        new.list_s, new.list_r, new.explist.view(np.float64),
                        np.ascontiguousarray(qvec, np.float64),
                        np.ascontiguousarray(np.asarray(Spos, np.float64).reshape(-1)),
                        psi.view(np.float64), fn.view(np.float64), nthreads)
    if rc != 0:
        raise ValueError("oracle: sq_a unsupported arguments")
    return fn


def u1_hv(model: Model, nod, x, nthreads=0):
    """ham_to_vec_wave_vector of the U(1)-only variant (source_only_u1/ham2vec_v3.f90:35-65)."""
    D = model.binom(model.NOS, nod)
    x = np.ascontiguousarray(x, dtype=np.complex128)
    assert x.shape == (D,)
    y = np.zeros(D, dtype=np.complex128)
    lib().ora_u1_hv(model.h, nod, x.view(np.float64), y.view(np.float64), 0, D, nthreads)
    return y


def u1_dense(model: Model, nod):
    """Dense H of the U(1)-only basis (colex order) from unit vectors; small D only."""
    D = model.binom(model.NOS, nod)
    H = np.zeros((D, D), dtype=np.complex128)
    for j in range(D):
        e = np.zeros(D, dtype=np.complex128)
        e[j] = 1.0
        H[:, j] = u1_hv(model, nod, e)
    return H


def u1_corr(model: Model, nod, v, nthreads=0):
    """calcu_cf / calcu_lm of the U(1)-only variant for all ordered pairs.

    Returns (szsz, spsm, lm) with S[a-1, b-1] for list_ij = (a, b).
    """
    n = model.NOS
    v = np.ascontiguousarray(v, dtype=np.complex128)
    zz = np.zeros(n * n)
    pm = np.zeros(n * n, dtype=np.complex128)
    lm = np.zeros(n)
    rc = lib().ora_u1_corr(model.h, nod, v.view(np.float64), zz, pm.view(np.float64), lm, nthreads)
    if rc != 0:
        raise ValueError("oracle: u1_corr unsupported arguments")
    return zz.reshape(n, n).T.copy(), pm.reshape(n, n).T.copy(), lm


def u1_sq_a(model: Model, spsmsz, nod, qvec, Spos, psi):
    """calcu_Sq_a of the U(1)-only variant (source_only_u1/get_expectation_values.f90:100-179)."""
    nodn = nod - 1 if spsmsz == 1 else (nod + 1 if spsmsz == 2 else nod)
    fn = np.zeros(model.binom(model.NOS, nodn), dtype=np.complex128)
    psi = np.ascontiguousarray(psi, dtype=np.complex128)
    rc = lib().ora_u1_sq_a(model.h, spsmsz, nod, np.ascontiguousarray(qvec, np.float64),
                           np.ascontiguousarray(np.asarray(Spos, np.float64).reshape(-1)),
                           psi.view(np.float64), fn.view(np.float64))
    if rc != 0:
        raise ValueError("oracle: u1_sq_a unsupported arguments")
    return fn


def cfrac(alpha, beta, norm1, E0, eta, omega, compat=True):
    """DSFLan continued fraction (source_DSFLan/main.f90:52-84)."""
    alpha = np.ascontiguousarray(alpha, np.float64)
    beta = np.ascontiguousarray(beta, np.float64)
    omega = np.ascontiguousarray(omega, np.float64)
    S = np.zeros(len(omega))
    rc = lib().ora_cfrac(len(alpha), alpha, beta, float(norm1), float(E0), float(eta),
                         len(omega), omega, 1 if compat else 0, S)
    if rc != 0:
        raise ValueError("oracle: cfrac needs at least one level")
    return S
