// qs3_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A CPU restatement of the QS3 (QS-Cube/ED) hot-path loops, used as the
// checker for the GB300 library.  Only tests/, __graft_entry__.smoke() and the
// cpu_baseline / reference legs of bench.py may load this file's library.  It
// is never linked into, called by or shipped with the product path.
//
// Parity status: the reference is Fortran and no Fortran compiler exists in
// the build image, and the reference ships no tests or golden outputs, so this
// restatement cannot be pinned against the reference binary ("parity
// unpinned" against QS3.exe itself).  It is pinned instead against known
// answers that follow from the physics (dense exact diagonalisation written
// independently in numpy, free-fermion XX chains, single-magnon dispersion,
// SU(2) multiplets, the sector sum rule); see tests/test_oracle_*.py.
//
// Each function names the reference routine it follows.  Deliberate
// deviations from the Fortran:
//   * 64-bit integers for ranks, dimensions and binomials (the reference uses
//     default 32-bit integer and overflows for C(1000,4));
//   * the S^z(q) start-vector scatter (spsmsz==3) is race-free here (the
//     reference updates fn(lp) without an atomic);
//   * scatter accumulation runs in per-thread buffers reduced in thread order,
//     so the result is deterministic (the reference's OpenMP atomics are not).
//
// Conventions: sites are 1-based as in Fortran; a configuration is the sorted
// list n[0..NOD-1] of down-spin sites; ranks ("list_s" values) are the 1-based
// colex ranks of inv_list; rows are 0-based; complex numbers are interleaved
// (re, im) doubles, i.e. Fortran complex(8).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct Model {
  int NOS = 0, LX = 0, LY = 0, LZ = 0, NOxxz = 0, KMAX = 0;
  std::vector<int> p1, p2;            // bond ends, 1-based, p1 <= p2
  std::vector<double> sJxy, sJz;      // sJint(:,2) = Jxy/2, sJint(:,3) = Jz/4
  std::vector<int> shx, shy, shz;     // shift tables, index 1..NOS
  std::vector<int64_t> comb;          // C(n,k), n in [0,NOS], k in [0,KMAX]
  int64_t C(int n, int k) const {
    if (n < 0 || k < 0 || n < k || k > KMAX) return 0;
    return comb[(size_t)n * (KMAX + 1) + k];
  }
};

struct cplx { double re, im; };

static inline cplx cmul(cplx a, cplx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }

// f_combination (state_lists.f90:17-33), in 64-bit with overflow saturation.
static int64_t f_combination(int n, int k) {
  if (n < k) return 0;
  __int128 v = 1;
  for (int i = 1; i <= k; ++i) {
    v = v * (n - k + i);
    v = v / i;
    if (v > (__int128)INT64_MAX) return INT64_MAX;
  }
  return (int64_t)v;
}

// insertion_sort (state_lists.f90:115-129)
static inline void insertion_sort(int* a, int nod) {
  for (int i = 1; i < nod; ++i) {
    int t = a[i];
    int j = i - 1;
    while (j >= 0 && a[j] > t) { a[j + 1] = a[j]; --j; }
    a[j + 1] = t;
  }
}

// inv_list (state_lists.f90:131-139): colex rank, 1-based.
static inline int64_t inv_list(const Model& m, const int* n, int nod) {
  int64_t t = n[0];
  for (int i = 2; i <= nod; ++i) t += m.C(n[i - 1] - 1, i);
  return t;
}

// list_fly + binary_search (state_lists.f90:294-331): unrank t into n[].
static inline void list_fly(const Model& m, int64_t t, int nod, int* n) {
  int64_t s = t;
  int hi = m.NOS - 1;
  for (int i = nod; i >= 2; --i) {
    // smallest j0 in [i, hi] with C(j0, i) >= s (binary_search's bmin)
    int lo = i, h = hi;
    while (lo <= h) {
      int b = lo + (h - lo) / 2;
      int64_t c = m.C(b, i);
      if (s < c) h = b - 1;
      else if (c < s) lo = b + 1;
      else { lo = b; break; }
    }
    int j0 = lo;
    n[i - 1] = j0;
    s -= m.C(j0 - 1, i);
    hi = j0 - 1;
  }
  n[0] = (int)s;
}

// j_flip_ni (state_lists.f90:333-362): flip the antiparallel pair (i<j) and
// return the sorted result.
static inline void j_flip_ni(int i, int j, const int* n, int nod, int* nd) {
  bool jdown = false;
  for (int k = 0; k < nod; ++k) if (n[k] == j) { jdown = true; break; }
  int w = 0;
  if (!jdown) {  // S+_i S-_j : remove i, insert j
    bool ins = false;
    for (int k = 0; k < nod; ++k) {
      if (n[k] == i) continue;
      if (!ins && n[k] > j) { nd[w++] = j; ins = true; }
      nd[w++] = n[k];
    }
    if (!ins) nd[w++] = j;
  } else {       // S-_i S+_j : remove j, insert i
    bool ins = false;
    for (int k = 0; k < nod; ++k) {
      if (n[k] == j) continue;
      if (!ins && n[k] > i) { nd[w++] = i; ins = true; }
      nd[w++] = n[k];
    }
    if (!ins) nd[w++] = i;
  }
}

// representative_SQ (state_lists.f90:384-416).  n is replaced by the
// representative; ell receives the translation (i,j,k) of the last strict
// decrease in loop order (0,0,0 if n was already minimal).
static inline int64_t representative(const Model& m, int nod, int* n, int* ell) {
  int nd[64];
  ell[0] = ell[1] = ell[2] = 0;
  for (int a = 0; a < nod; ++a) nd[a] = n[a];
  for (int k = 1; k <= m.LZ; ++k) {
    for (int a = 0; a < nod; ++a) nd[a] = m.shz[nd[a]];
    for (int j = 1; j <= m.LY; ++j) {
      for (int a = 0; a < nod; ++a) nd[a] = m.shy[nd[a]];
      for (int i = 1; i <= m.LX; ++i) {
        for (int a = 0; a < nod; ++a) nd[a] = m.shx[nd[a]];
        insertion_sort(nd, nod);
        for (int l = nod - 1; l >= 0; --l) {
          if (nd[l] > n[l]) break;
          if (nd[l] < n[l]) {
            ell[0] = i; ell[1] = j; ell[2] = k;
            for (int a = 0; a <= l; ++a) n[a] = nd[a];
            break;
          }
        }
      }
    }
  }
  return inv_list(m, n, nod);
}

// findstate (state_lists.f90:364-382): 0-based row or -1.
static inline int64_t findstate(int64_t s, const int64_t* list_s, int64_t D) {
  int64_t lo = 0, hi = D - 1;
  while (lo <= hi) {
    int64_t b = lo + (hi - lo) / 2;
    if (s < list_s[b]) hi = b - 1;
    else if (s > list_s[b]) lo = b + 1;
    else return b;
  }
  return -1;
}

// checkstate_SQ (state_lists.f90:66-112): returns ro (0 if not a representative).
static double checkstate(const Model& m, int64_t s, int nod, double pkx, double pky, double pkz) {
  int n[64], np[64];
  list_fly(m, s, nod, n);
  for (int a = 0; a < nod; ++a) np[a] = n[a];
  double cre = 0.0, cim = 0.0;
  int count = 0;
  for (int k = 1; k <= m.LZ; ++k) {
    for (int a = 0; a < nod; ++a) np[a] = m.shz[np[a]];
    double p1 = pkz * (double)k;
    for (int j = 1; j <= m.LY; ++j) {
      for (int a = 0; a < nod; ++a) np[a] = m.shy[np[a]];
      double p2 = pky * (double)j + p1;
      for (int i = 1; i <= m.LX; ++i) {
        for (int a = 0; a < nod; ++a) np[a] = m.shx[np[a]];
        insertion_sort(np, nod);
        int l;
        for (l = nod - 1; l >= 0; --l) {
          if (np[l] < n[l]) return 0.0;
          if (np[l] > n[l]) break;
        }
        if (l < 0) {
          double ph = pkx * (double)i + p2;
          // exp((0,-1)*ph) = (cos ph, -sin ph)
          cre += std::cos(ph);
          cim += -std::sin(ph);
          ++count;
        }
      }
    }
  }
  double a = std::hypot(cre, cim);
  return (a * a) * (double)m.NOS / (double)count;
}

static inline bool contains(const int* n, int nod, int s) {
  for (int a = 0; a < nod; ++a) if (n[a] == s) return true;
  return false;
}

static inline int nthreads_or_default(int nt) {
#ifdef _OPENMP
  return nt > 0 ? nt : omp_get_max_threads();
#else
  (void)nt;
  return 1;
#endif
}

}  // namespace

extern "C" {

// Model set-up: read_ip (input_param.f90:58-117) bond handling and the shift
// tables mk_shift_{x,y,z}_SQ (state_lists.f90:36-64).  p_xxz is p_xxz(1:2,b)
// interleaved; Jint holds Jxy[NOxxz] followed by Jz[NOxxz] (Jint(:,2:3)).
void* ora_model_new(int NOS, int LX, int LY, int LZ, int NOxxz, const int* p_xxz,
                    const double* Jint, int kmax) {
  if (NOS <= 0 || LX <= 0 || LY <= 0 || LZ <= 0 || LX * LY * LZ != NOS || kmax < 1 || kmax > 60)
    return nullptr;
  Model* m = new Model();
  m->NOS = NOS; m->LX = LX; m->LY = LY; m->LZ = LZ; m->NOxxz = NOxxz; m->KMAX = kmax;
  m->p1.resize(NOxxz); m->p2.resize(NOxxz); m->sJxy.resize(NOxxz); m->sJz.resize(NOxxz);
  for (int b = 0; b < NOxxz; ++b) {
    int a = p_xxz[2 * b], c = p_xxz[2 * b + 1];
    if (a < 1 || a > NOS || c < 1 || c > NOS) { delete m; return nullptr; }
    if (a > c) std::swap(a, c);
    m->p1[b] = a; m->p2[b] = c;
    m->sJxy[b] = Jint[b] * 0.5;
    m->sJz[b] = Jint[NOxxz + b] * 0.25;
  }
  m->shx.assign(NOS + 1, 0); m->shy.assign(NOS + 1, 0); m->shz.assign(NOS + 1, 0);
  for (int z = 1; z <= LZ; ++z)
    for (int y = 1; y <= LY; ++y)
      for (int x = 1; x <= LX; ++x) {
        int s = x + LX * ((y - 1) + LY * (z - 1));
        m->shx[s] = (x % LX) + 1 + LX * (y - 1) + LX * LY * (z - 1);
        m->shy[s] = x + LX * (y % LY) + LX * LY * (z - 1);
        m->shz[s] = x + LX * (y - 1) + LX * LY * (z % LZ);
      }
  m->comb.assign((size_t)(NOS + 1) * (kmax + 1), 0);
  for (int n = 0; n <= NOS; ++n)
    for (int k = 0; k <= kmax; ++k) m->comb[(size_t)n * (kmax + 1) + k] = f_combination(n, k);
  return m;
}

void ora_model_free(void* h) { delete (Model*)h; }

int64_t ora_binom(void* h, int n, int k) { return ((Model*)h)->C(n, k); }

// rk = 2*pi*K/L (input_param.f90:76-78)
void ora_wavevector(int KX, int KY, int KZ, int LX, int LY, int LZ, double* rk3) {
  const double PI = std::acos(-1.0);
  rk3[0] = 2.0 * PI * (double)KX / (double)LX;
  rk3[1] = 2.0 * PI * (double)KY / (double)LY;
  rk3[2] = 2.0 * PI * (double)KZ / (double)LZ;
}

// explist(0:LX,0:LY,0:LZ) = exp(i*(rkx*i + rky*j + rkz*k)) (input_param.f90:87-89)
void ora_explist(const double* rk3, int LX, int LY, int LZ, double* out) {
  for (int k = 0; k <= LZ; ++k)
    for (int j = 0; j <= LY; ++j)
      for (int i = 0; i <= LX; ++i) {
        double ph = rk3[0] * (double)i + rk3[1] * (double)j + rk3[2] * (double)k;
        size_t idx = (size_t)i + (size_t)(LX + 1) * ((size_t)j + (size_t)(LY + 1) * k);
        out[2 * idx] = std::cos(ph);
        out[2 * idx + 1] = std::sin(ph);
      }
}

void ora_list_fly(void* h, int64_t t, int nod, int* n) { list_fly(*(Model*)h, t, nod, n); }
int64_t ora_inv_list(void* h, const int* n, int nod) { return inv_list(*(Model*)h, n, nod); }
int64_t ora_representative(void* h, int nod, int* n, int* ell) {
  return representative(*(Model*)h, nod, n, ell);
}
void ora_j_flip(int i, int j, const int* n, int nod, int* nd) { j_flip_ni(i, j, n, nod, nd); }
double ora_checkstate(void* h, int64_t s, int nod, const double* rk3) {
  return checkstate(*(Model*)h, s, nod, rk3[0], rk3[1], rk3[2]);
}

// allocate_lists_omp_SQ (state_lists.f90:225-292): scan every rank 1..C(NOS,NOD)
// with checkstate_SQ, keep ro > 1e-15, list sorted by rank, list_r = sqrt(ro).
// With list_s == nullptr only the count is returned.  Returns -1 on overflow
// or when cap is too small.
int64_t ora_build_sector(void* h, int nod, const double* rk3, int64_t* list_s, double* list_r,
                         int64_t cap, int nthreads) {
  const Model& m = *(Model*)h;
  if (nod < 1 || nod > m.NOS || nod > m.KMAX || nod > 64) return -1;
  int64_t ths = m.C(m.NOS, nod);
  if (ths == INT64_MAX) return -1;
  int nt = nthreads_or_default(nthreads);
  const int64_t chunk = 1 << 14;
  int64_t nchunks = (ths + chunk - 1) / chunk;
  std::vector<std::vector<int64_t>> cs(nchunks);
  std::vector<std::vector<double>> cr(nchunks);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
  for (int64_t c = 0; c < nchunks; ++c) {
    int64_t a = c * chunk + 1, b = std::min(ths, (c + 1) * chunk);
    for (int64_t s = a; s <= b; ++s) {
      double r = checkstate(m, s, nod, rk3[0], rk3[1], rk3[2]);
      if (r > 1.0e-15) { cs[c].push_back(s); cr[c].push_back(r); }
    }
  }
  int64_t D = 0;
  for (auto& v : cs) D += (int64_t)v.size();
  if (!list_s) return D;
  if (D > cap) return -1;
  int64_t w = 0;
  for (int64_t c = 0; c < nchunks; ++c)
    for (size_t q = 0; q < cs[c].size(); ++q) {
      list_s[w] = cs[c][q];
      list_r[w] = std::sqrt(cr[c][q]);
      ++w;
    }
  return D;
}

// ham_to_vec_wave_vector (ham2vec_v3.f90:37-72) over rows [row0, row1).
// v0/v1/explist are complex(8) interleaved.
void ora_hv(void* h, int nod, int64_t D, const int64_t* list_s, const double* list_r,
            const double* explist, const double* v1, double* v0, int64_t row0, int64_t row1,
            int nthreads) {
  const Model& m = *(Model*)h;
  const cplx* x = (const cplx*)v1;
  cplx* y = (cplx*)v0;
  const cplx* ex = (const cplx*)explist;
  const size_t ex1 = (size_t)m.LX + 1, ex2 = ex1 * ((size_t)m.LY + 1);
  int nt = nthreads_or_default(nthreads);
  if (row1 > D) row1 = D;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nt)
  for (int64_t i = row0; i < row1; ++i) {
    int st[64], ni[64], ell[3];
    cplx acc = {0.0, 0.0};
    list_fly(m, list_s[i], nod, st);
    const cplx xi = x[i];
    for (int j = 0; j < m.NOxxz; ++j) {
      bool f1 = contains(st, nod, m.p1[j]);
      bool f2 = contains(st, nod, m.p2[j]);
      if (f1 != f2) {
        acc.re = acc.re - m.sJz[j] * xi.re;
        acc.im = acc.im - m.sJz[j] * xi.im;
        j_flip_ni(m.p1[j], m.p2[j], st, nod, ni);
        int64_t s = representative(m, nod, ni, ell);
        int64_t id = findstate(s, list_s, D);
        if (id >= 0) {
          double c = m.sJxy[j] * list_r[id] / list_r[i];
          cplx e = ex[(size_t)ell[0] + ex1 * (size_t)ell[1] + ex2 * (size_t)ell[2]];
          cplx ce = {c * e.re, c * e.im};
          cplx t = cmul(ce, x[id]);
          acc.re = acc.re + t.re;
          acc.im = acc.im + t.im;
        }
      } else {
        acc.re = acc.re + m.sJz[j] * xi.re;
        acc.im = acc.im + m.sJz[j] * xi.im;
      }
    }
    y[i] = acc;
  }
}

// The connection table of ham_to_vec_wave_vector restricted to rows
// [row0, row1): one entry (row, col, ell, bond) for every antiparallel bond
// whose hop lands on a row of the sector (id > 0 in the Fortran), rows
// ascending, bonds in list order.  Returns nnz, or -1 when cap is too small
// (pass row == nullptr to count only).
int64_t ora_connection_table_rows(void* h, int nod, int64_t D, const int64_t* list_s, int64_t row0,
                                  int64_t row1, int64_t* row, int64_t* col, int* ell3, int* bond,
                                  int64_t cap, int nthreads) {
  const Model& m = *(Model*)h;
  int nt = nthreads_or_default(nthreads);
  if (row1 > D) row1 = D;
  if (row0 < 0 || row0 > row1) return -1;
  const int64_t nr = row1 - row0;
  std::vector<int64_t> cnt(nr + 1, 0);
#pragma omp parallel for schedule(dynamic, 64) num_threads(nt)
  for (int64_t r = 0; r < nr; ++r) {
    int st[64], ni[64], ell[3];
    list_fly(m, list_s[row0 + r], nod, st);
    int64_t c = 0;
    for (int j = 0; j < m.NOxxz; ++j) {
      bool f1 = contains(st, nod, m.p1[j]);
      bool f2 = contains(st, nod, m.p2[j]);
      if (f1 != f2) {
        j_flip_ni(m.p1[j], m.p2[j], st, nod, ni);
        int64_t s = representative(m, nod, ni, ell);
        if (findstate(s, list_s, D) >= 0) ++c;
      }
    }
    cnt[r + 1] = c;
  }
  for (int64_t r = 0; r < nr; ++r) cnt[r + 1] += cnt[r];
  int64_t nnz = cnt[nr];
  if (!row) return nnz;
  if (nnz > cap) return -1;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nt)
  for (int64_t r = 0; r < nr; ++r) {
    const int64_t i = row0 + r;
    int st[64], ni[64], ell[3];
    list_fly(m, list_s[i], nod, st);
    int64_t w = cnt[r];
    for (int j = 0; j < m.NOxxz; ++j) {
      bool f1 = contains(st, nod, m.p1[j]);
      bool f2 = contains(st, nod, m.p2[j]);
      if (f1 != f2) {
        j_flip_ni(m.p1[j], m.p2[j], st, nod, ni);
        int64_t s = representative(m, nod, ni, ell);
        int64_t id = findstate(s, list_s, D);
        if (id >= 0) {
          row[w] = i; col[w] = id;
          ell3[3 * w] = ell[0]; ell3[3 * w + 1] = ell[1]; ell3[3 * w + 2] = ell[2];
          bond[w] = j;
          ++w;
        }
      }
    }
  }
  return nnz;
}

// The whole connection table (rows 0..D-1).
int64_t ora_connection_table(void* h, int nod, int64_t D, const int64_t* list_s, int64_t* row,
                             int64_t* col, int* ell3, int* bond, int64_t cap, int nthreads) {
  return ora_connection_table_rows(h, nod, D, list_s, 0, D, row, col, ell3, bond, cap, nthreads);
}

// Number of connection-table entries (off-diagonal hops that land on a row)
// of rows [row0, row1): the nnz_off of the algorithmic byte count.
int64_t ora_count_offdiag(void* h, int nod, int64_t D, const int64_t* list_s, int64_t row0,
                          int64_t row1, int nthreads) {
  const Model& m = *(Model*)h;
  int nt = nthreads_or_default(nthreads);
  int64_t tot = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : tot) num_threads(nt)
  for (int64_t i = row0; i < row1; ++i) {
    int st[64], ni[64], ell[3];
    list_fly(m, list_s[i], nod, st);
    for (int j = 0; j < m.NOxxz; ++j) {
      bool f1 = contains(st, nod, m.p1[j]);
      bool f2 = contains(st, nod, m.p2[j]);
      if (f1 != f2) {
        j_flip_ni(m.p1[j], m.p2[j], st, nod, ni);
        int64_t s = representative(m, nod, ni, ell);
        if (findstate(s, list_s, D) >= 0) ++tot;
      }
    }
  }
  return tot;
}

// Sector lists of a chain (LY = LZ = 1) without scanning all C(NOS, NOD)
// ranks: a representative occupies site 1, so only the C(NOS-1, NOD-1)
// candidates containing site 1 are enumerated; a candidate is kept when no
// rotation that moves another down spin onto site 1 gives a smaller
// configuration (colex), and its norm follows checkstate_SQ summed over its
// self-translations.  Produces the same lists as ora_build_sector (checked
// by the tests at small L); used to set up large chain workloads on the CPU.
int64_t ora_chain_sector(void* h, int nod, const double* rk3, int64_t* list_s, double* list_r,
                         int64_t cap, int nthreads) {
  const Model& m = *(Model*)h;
  if (m.LY != 1 || m.LZ != 1 || nod < 1 || nod > 16 || nod > m.KMAX) return -1;
  const int L = m.NOS;
  const int64_t nc = m.C(L - 1, nod - 1);
  // r by number of self-translations (count = L/p): checkstate restricted to i = p, 2p, ..., L
  std::vector<double> rc(nod + 1, 0.0);
  for (int c = 1; c <= nod; ++c) {
    if (L % c) continue;
    const int per = L / c;
    double cre = 0.0, cim = 0.0;
    const double p1 = rk3[2] * 1.0, p2 = rk3[1] * 1.0 + p1;
    for (int i = per; i <= L; i += per) {
      double ph = rk3[0] * (double)i + p2;
      cre += std::cos(ph);
      cim += -std::sin(ph);
    }
    double a = std::hypot(cre, cim);
    rc[c] = (a * a) * (double)m.NOS / (double)c;
  }
  int nt = nthreads_or_default(nthreads);
  const int64_t chunk = 1 << 16;
  const int64_t nchunks = (nc + chunk - 1) / chunk;
  std::vector<std::vector<int64_t>> cs(nchunks);
  std::vector<std::vector<double>> cr(nchunks);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
  for (int64_t ch = 0; ch < nchunks; ++ch) {
    const int64_t a0 = ch * chunk, a1 = std::min(nc, a0 + chunk);
    // unrank a0 over sites 2..L: a0 = sum_{j>=1} C(q_j, j), q_j = n_j - 2
    int n[64];
    n[0] = 1;
    int64_t rem = a0;
    for (int j = nod - 1; j >= 1; --j) {
      int lo = j - 1, hi = L - 2;
      while (lo < hi) {
        int mid = (lo + hi + 1) / 2;
        if (m.C(mid, j) <= rem) lo = mid; else hi = mid - 1;
      }
      n[j] = lo + 2;
      rem -= m.C(lo, j);
    }
    for (int64_t c = a0; c < a1; ++c) {
      // gaps and reverse-lexicographic keys
      int g[64];
      for (int t = 0; t < nod - 1; ++t) g[t] = n[t + 1] - n[t];
      g[nod - 1] = n[0] + L - n[nod - 1];
      bool rep = true;
      int count = 1;
      for (int q = 1; q < nod && rep; ++q) {
        int cmp = 0;
        for (int t = 1; t <= nod && cmp == 0; ++t) {
          int a = g[((0 - t) % nod + nod) % nod], b = g[((q - t) % nod + nod) % nod];
          cmp = (b > a) ? 1 : (b < a ? -1 : 0);
        }
        if (cmp > 0) rep = false;
        else if (cmp == 0) ++count;
      }
      if (rep && rc[count] > 1.0e-15) {
        cs[ch].push_back(inv_list(m, n, nod));
        cr[ch].push_back(rc[count]);
      }
      // colex successor of n[1..nod-1] over sites 2..L
      for (int j = 1; j < nod; ++j) {
        int lim = (j + 1 < nod) ? n[j + 1] : L + 1;
        if (n[j] + 1 < lim) { n[j] += 1; break; }
        n[j] = j + 1;
      }
    }
  }
  int64_t D = 0;
  for (auto& v : cs) D += (int64_t)v.size();
  if (!list_s) return D;
  if (D > cap) return -1;
  int64_t w = 0;
  for (int64_t ch = 0; ch < nchunks; ++ch)
    for (size_t q = 0; q < cs[ch].size(); ++q) {
      list_s[w] = cs[ch][q];
      list_r[w] = std::sqrt(cr[ch][q]);
      ++w;
    }
  return D;
}

// calcu_Sq_a (get_expectation_values.f90:281-377) with
// search_representative_{Spi,Smi,Szi}_state_SQ (state_lists.f90:488-583).
// Builds fn = S^a(q)|psi> / sqrt(NOS) in the new sector.  Spos is Spos(1:3,i)
// interleaved per site.  Returns 0, or -1 for unsupported arguments.
int ora_sq_a(void* h, int spsmsz, int nod, int64_t D, const int64_t* list_s, const double* list_r,
             int nod_new, int64_t Dn, const int64_t* list_s_new, const double* list_r_new,
             const double* explist_new, const double* qvec3, const double* Spos,
             const double* psi_, double* fn_, int nthreads) {
  const Model& m = *(Model*)h;
  if (spsmsz < 1 || spsmsz > 3) return -1;
  if (spsmsz == 1 && nod <= 1) return -1;
  if (nod < 1 || nod > 63 || nod_new < 1 || nod_new > 64) return -1;
  const cplx* psi = (const cplx*)psi_;
  cplx* fn = (cplx*)fn_;
  const cplx* ex = (const cplx*)explist_new;
  const size_t ex1 = (size_t)m.LX + 1, ex2 = ex1 * ((size_t)m.LY + 1);
  std::vector<cplx> eks(m.NOS + 1);
  for (int i = 1; i <= m.NOS; ++i) {
    double d = qvec3[0] * Spos[3 * (i - 1)] + qvec3[1] * Spos[3 * (i - 1) + 1] +
               qvec3[2] * Spos[3 * (i - 1) + 2];
    eks[i] = {std::cos(d), -std::sin(d)};  // exp((0,-1)*d)
  }
  int nt = nthreads_or_default(nthreads);
  std::vector<std::vector<cplx>> part(nt, std::vector<cplx>(Dn, cplx{0.0, 0.0}));
  for (int i = 1; i <= m.NOS; ++i) {
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int64_t l = 0; l < D; ++l) {
#ifdef _OPENMP
      int tid = omp_get_thread_num();
#else
      int tid = 0;
#endif
      int st[64], bp[64], ell[3];
      list_fly(m, list_s[l], nod, st);
      bool fi = contains(st, nod, i);
      double siz = 1.0;
      if (spsmsz == 1) {
        if (!fi) continue;
        int w = 0;  // remove site i
        for (int a = 0; a < nod; ++a) if (st[a] != i) bp[w++] = st[a];
      } else if (spsmsz == 2) {
        if (fi) continue;
        int w = 0; bool ins = false;  // insert site i
        for (int a = 0; a < nod; ++a) {
          if (!ins && st[a] > i) { bp[w++] = i; ins = true; }
          bp[w++] = st[a];
        }
        if (!ins) bp[w++] = i;
      } else {
        siz = fi ? -0.5 : 0.5;
        for (int a = 0; a < nod; ++a) bp[a] = st[a];
      }
      int64_t s = representative(m, nod_new, bp, ell);
      int64_t lp = findstate(s, list_s_new, Dn);
      if (lp < 0) continue;
      // psi(l)*list_r_new(lp)/list_r(l), evaluated left to right as in Fortran
      const double rn = list_r_new[lp], ro = list_r[l];
      cplx pv = {(psi[l].re * rn) / ro, (psi[l].im * rn) / ro};
      if (spsmsz == 3) pv = {((siz * psi[l].re) * rn) / ro, ((siz * psi[l].im) * rn) / ro};
      cplx e = ex[(size_t)ell[0] + ex1 * (size_t)ell[1] + ex2 * (size_t)ell[2]];
      cplx ce = {e.re, -e.im};
      cplx t = cmul(cmul(pv, eks[i]), ce);
      part[tid][lp].re += t.re;
      part[tid][lp].im += t.im;
    }
  }
  double sc = 1.0 / std::sqrt((double)m.NOS);
  for (int64_t lp = 0; lp < Dn; ++lp) {
    cplx a = {0.0, 0.0};
    for (int t = 0; t < nt; ++t) { a.re += part[t][lp].re; a.im += part[t][lp].im; }
    fn[lp] = {sc * a.re, sc * a.im};
  }
  return 0;
}

// get_cf_2_wave_vector + mk_list_ij + calcu_cf_trans_2
// (get_expectation_values.f90:97-131,234-279; ham2vec_v3.f90:111-174) for one
// vector.  ss holds list_expe_ss(1:2,j) interleaved for j = 1..NOS*NOS, in the
// order of the reference's FILECF.  Outputs are indexed like the reference's
// expe_szsz(1:NOS**2) / expe_spsm(1:NOS**2): p = ss1 + (ss2-1)*NOS - 1.
int ora_corr(void* h, int nod, int64_t D, const int64_t* list_s, const double* list_r,
             const double* explist, const double* v_, const int* ss, int nocf, double* szsz,
             double* spsm_, int nthreads) {
  const Model& m = *(Model*)h;
  const int NOS = m.NOS;
  if (nocf != NOS * NOS) return -1;
  const cplx* v = (const cplx*)v_;
  cplx* spsm = (cplx*)spsm_;
  const cplx* ex = (const cplx*)explist;
  const size_t ex1 = (size_t)m.LX + 1, ex2 = ex1 * ((size_t)m.LY + 1);
  int nt = nthreads_or_default(nthreads);
  for (int p = 0; p < NOS * NOS; ++p) { szsz[p] = 0.0; spsm[p] = {0.0, 0.0}; }
  int64_t jmax = (int64_t)NOS * NOS, no_tot = 0;
  std::vector<int> lij(2 * (size_t)NOS + 2);
  for (int64_t jj = 0; jj < jmax; ++jj) {
    if (no_tot == jmax) break;
    // mk_list_ij
    int r[2] = {ss[2 * jj], ss[2 * jj + 1]};
    int noij = 1;
    lij[0] = r[0]; lij[1] = r[1];
    int rd[2] = {r[0], r[1]};
    bool done = false;
    for (int k = 1; k <= m.LZ && !done; ++k) {
      rd[0] = m.shz[rd[0]]; rd[1] = m.shz[rd[1]];
      for (int j = 1; j <= m.LY && !done; ++j) {
        rd[0] = m.shy[rd[0]]; rd[1] = m.shy[rd[1]];
        for (int i = 1; i <= m.LX && !done; ++i) {
          rd[0] = m.shx[rd[0]]; rd[1] = m.shx[rd[1]];
          int l;
          for (l = 1; l >= 0; --l) {
            if (rd[l] < r[l]) { noij = 0; done = true; break; }
            if (rd[l] > r[l]) {
              lij[2 * noij] = rd[0]; lij[2 * noij + 1] = rd[1];
              ++noij;
              break;
            }
          }
          if (!done && l < 0) done = true;
        }
      }
    }
    if (noij == 0) continue;
    no_tot += noij;
    // calcu_cf_trans_2
    double ezz = 0.0;
    double spre = 0.0, spim = 0.0;
    if (lij[0] == lij[1]) {
      ezz = 0.25;
#pragma omp parallel for reduction(+ : spre) schedule(static) num_threads(nt)
      for (int64_t i = 0; i < D; ++i) {
        int st[64];
        list_fly(m, list_s[i], nod, st);
        double w = v[i].re * v[i].re + v[i].im * v[i].im;
        for (int q = 0; q < noij; ++q) {
          if (contains(st, nod, lij[2 * q])) continue;
          spre += w;
        }
      }
    } else {
#pragma omp parallel for reduction(+ : ezz, spre, spim) schedule(static) num_threads(nt)
      for (int64_t i = 0; i < D; ++i) {
        int st[64], ni[64], ell[3];
        list_fly(m, list_s[i], nod, st);
        double w = v[i].re * v[i].re + v[i].im * v[i].im;
        for (int q = 0; q < noij; ++q) {
          int a = lij[2 * q], b = lij[2 * q + 1];
          bool f1 = contains(st, nod, a), f2 = contains(st, nod, b);
          if (!f1 && f2) {
            ezz -= w;
          } else if (f1 && !f2) {
            ezz -= w;
            j_flip_ni(std::min(a, b), std::max(a, b), st, nod, ni);
            int64_t s = representative(m, nod, ni, ell);
            int64_t id = findstate(s, list_s, D);
            if (id >= 0) {
              double c = list_r[id] / list_r[i];
              cplx e = ex[(size_t)ell[0] + ex1 * (size_t)ell[1] + ex2 * (size_t)ell[2]];
              cplx ce = {c * e.re, c * e.im};
              cplx cv = {v[i].re, -v[i].im};
              cplx t = cmul(cmul(ce, cv), v[id]);
              spre += t.re; spim += t.im;
            }
          } else {
            ezz += w;
          }
        }
      }
      ezz = ezz / noij * 0.25;
    }
    spre /= noij; spim /= noij;
    for (int q = 0; q < noij; ++q) {
      size_t p = (size_t)lij[2 * q] + (size_t)(lij[2 * q + 1] - 1) * NOS - 1;
      szsz[p] = ezz;
      spsm[p] = {spre, spim};
    }
  }
  return 0;
}

// ---------------------------------------------------------------- U(1)-only variant
// ham_to_vec_wave_vector of source_only_u1/ham2vec_v3.f90:35-65: row i
// (0-based) is list_fly(i+1); every antiparallel bond adds
// sJint(j,2) * v1(inv_list(j_flip_ni(...))) and -sJint(j,3) * v1(i), every
// parallel bond +sJint(j,3) * v1(i), in bond order.
void ora_u1_hv(void* h, int nod, const double* v1, double* v0, int64_t row0, int64_t row1, int nthreads) {
  const Model& m = *(Model*)h;
  const cplx* x = (const cplx*)v1;
  cplx* y = (cplx*)v0;
  const int64_t D = m.C(m.NOS, nod);
  if (row1 > D) row1 = D;
  int nt = nthreads_or_default(nthreads);
#pragma omp parallel for schedule(dynamic, 64) num_threads(nt)
  for (int64_t i = row0; i < row1; ++i) {
    int st[64], ni[64];
    cplx acc = {0.0, 0.0};
    list_fly(m, i + 1, nod, st);
    const cplx xi = x[i];
    for (int j = 0; j < m.NOxxz; ++j) {
      bool f1 = contains(st, nod, m.p1[j]);
      bool f2 = contains(st, nod, m.p2[j]);
      if (f1 != f2) {
        acc.re = acc.re - m.sJz[j] * xi.re;
        acc.im = acc.im - m.sJz[j] * xi.im;
        j_flip_ni(m.p1[j], m.p2[j], st, nod, ni);
        const int64_t id = inv_list(m, ni, nod) - 1;
        acc.re = acc.re + m.sJxy[j] * x[id].re;
        acc.im = acc.im + m.sJxy[j] * x[id].im;
      } else {
        acc.re = acc.re + m.sJz[j] * xi.re;
        acc.im = acc.im + m.sJz[j] * xi.im;
      }
    }
    y[i] = acc;
  }
}

// calcu_cf and calcu_lm of source_only_u1/ham2vec_v3.f90:67-141 for every
// ordered pair (a, b), stored at (a-1) + (b-1)*NOS, and every site.
// Each pair's row sum runs serially in row order.
int ora_u1_corr(void* h, int nod, const double* v_, double* szsz, double* spsm_, double* lm, int nthreads) {
  const Model& m = *(Model*)h;
  const cplx* v = (const cplx*)v_;
  cplx* spsm = (cplx*)spsm_;
  const int NOS = m.NOS;
  const int64_t D = m.C(NOS, nod);
  if (nod < 1 || nod > 63) return -1;
  int nt = nthreads_or_default(nthreads);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
  for (int p = 0; p < NOS * NOS; ++p) {
    const int a = p % NOS + 1, b = p / NOS + 1;
    int st[64], ni[64];
    double zz = 0.0;
    cplx pm = {0.0, 0.0};
    if (a == b) {
      zz = 0.25;
      for (int64_t i = 0; i < D; ++i) {
        list_fly(m, i + 1, nod, st);
        if (contains(st, nod, a)) continue;
        pm.re += v[i].re * v[i].re + v[i].im * v[i].im;
      }
    } else {
      for (int64_t i = 0; i < D; ++i) {
        list_fly(m, i + 1, nod, st);
        const bool f1 = contains(st, nod, a), f2 = contains(st, nod, b);
        const double w = v[i].re * v[i].re + v[i].im * v[i].im;
        if (!f1 && f2) {
          zz -= w;
        } else if (f1 && !f2) {
          zz -= w;
          j_flip_ni(std::min(a, b), std::max(a, b), st, nod, ni);
          const int64_t id = inv_list(m, ni, nod) - 1;
          const cplx t = cmul({v[i].re, -v[i].im}, v[id]);
          pm.re += t.re;
          pm.im += t.im;
        } else {
          zz += w;
        }
      }
      zz *= 0.25;
    }
    szsz[p] = zz;
    spsm[p] = pm;
  }
  if (lm) {
    for (int s = 1; s <= NOS; ++s) {
      int st[64];
      double e = 0.0;
      for (int64_t i = 0; i < D; ++i) {
        list_fly(m, i + 1, nod, st);
        const double w = v[i].re * v[i].re + v[i].im * v[i].im;
        e += contains(st, nod, s) ? -w : w;
      }
      lm[s - 1] = e * 0.5;
    }
  }
  return 0;
}

// calcu_Sq_a of source_only_u1/get_expectation_values.f90:100-179 (scatter
// form, site loop outermost): fn(lp) += psi(l) * exp(-i q.R_i), then
// fn /= sqrt(NOS).  fn has C(NOS, nod') elements.  Returns 0, or -1 for
// unsupported arguments.
int ora_u1_sq_a(void* h, int spsmsz, int nod, const double* qvec3, const double* Spos, const double* psi_,
                double* fn_) {
  const Model& m = *(Model*)h;
  const int NOS = m.NOS;
  if (spsmsz < 1 || spsmsz > 3 || nod < 1 || nod > 62) return -1;
  if (spsmsz == 1 && nod <= 1) return -1;
  const int nodn = spsmsz == 1 ? nod - 1 : (spsmsz == 2 ? nod + 1 : nod);
  if (nodn > NOS) return -1;
  const cplx* psi = (const cplx*)psi_;
  cplx* fn = (cplx*)fn_;
  const int64_t D = m.C(NOS, nod), Dn = m.C(NOS, nodn);
  for (int64_t l = 0; l < Dn; ++l) fn[l] = {0.0, 0.0};
  std::vector<cplx> eks(NOS + 1);
  for (int i = 1; i <= NOS; ++i) {
    const double d = qvec3[0] * Spos[3 * (i - 1)] + qvec3[1] * Spos[3 * (i - 1) + 1] +
                     qvec3[2] * Spos[3 * (i - 1) + 2];
    eks[i] = {std::cos(d), -std::sin(d)};
  }
  int st[64], nd[64];
  for (int i = 1; i <= NOS; ++i) {
    for (int64_t l = 0; l < D; ++l) {
      list_fly(m, l + 1, nod, st);
      const bool fi = contains(st, nod, i);
      if (spsmsz == 1 && fi) {          // search_Spi: remove i
        int w = 0;
        for (int k = 0; k < nod; ++k) if (st[k] != i) nd[w++] = st[k];
        const int64_t lp = inv_list(m, nd, nodn) - 1;
        const cplx t = cmul(psi[l], eks[i]);
        fn[lp].re += t.re; fn[lp].im += t.im;
      } else if (spsmsz == 2 && !fi) {  // search_Smi: insert i
        int w = 0;
        bool ins = false;
        for (int k = 0; k < nod; ++k) {
          if (!ins && st[k] > i) { nd[w++] = i; ins = true; }
          nd[w++] = st[k];
        }
        if (!ins) nd[w++] = i;
        const int64_t lp = inv_list(m, nd, nodn) - 1;
        const cplx t = cmul(psi[l], eks[i]);
        fn[lp].re += t.re; fn[lp].im += t.im;
      } else if (spsmsz == 3) {
        const double siz = fi ? -0.5 : 0.5;
        const cplx t = cmul({siz * psi[l].re, siz * psi[l].im}, eks[i]);
        fn[l].re += t.re; fn[l].im += t.im;
      }
    }
  }
  const double sc = 1.0 / std::sqrt((double)NOS);
  for (int64_t l = 0; l < Dn; ++l) { fn[l].re *= sc; fn[l].im *= sc; }
  return 0;
}

// DSFLan continued fraction (source_DSFLan/main.f90:52-84) on an arbitrary
// omega grid.  alpha[0..N-1], beta[0..N-1] are the file's alpha(n), beta(n)
// (beta(1) = 0, beta(n) = beta_n^2).  compat = 1 keeps the reference's deepest
// level exactly (imaginary part not divided by its denominator); compat = 0
// evaluates the continued fraction without that quirk.  Requires N >= 1.
int ora_cfrac(int N, const double* alpha, const double* beta, double norm1, double E0, double eta,
              int nomega, const double* omega, int compat, double* S) {
  if (N < 1) return -1;
  const double pi = std::acos(-1.0);
  for (int o = 0; o < nomega; ++o) {
    double w = omega[o];
    int n = N;  // Fortran n = itr_num - 1 = number of levels
    double kr = w + E0 - alpha[n - 1] - 0.0;  // beta(n+1) is never read from the file
    double bunbo = kr * kr + eta * eta;
    double tr = beta[n - 1] * kr / bunbo;
    double ti = compat ? -beta[n - 1] * eta : -beta[n - 1] * eta / bunbo;
    for (n = N - 1; n >= 2; --n) {
      kr = w + E0 - alpha[n - 1] - tr;
      double ki = eta - ti;
      bunbo = kr * kr + ki * ki;
      tr = beta[n - 1] * kr / bunbo;
      ti = -beta[n - 1] * ki / bunbo;
    }
    kr = w + E0 - alpha[0] - tr;
    double ki = eta - ti;
    bunbo = kr * kr + ki * ki;
    ti = -norm1 * ki / bunbo;
    S[o] = -ti / pi;
  }
  return 0;
}

}  // extern "C"
