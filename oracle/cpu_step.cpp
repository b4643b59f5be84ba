// CPU restatement, in C++, of the reference's phaseless walker step.
//
// Test infrastructure: bench.py times it as the CPU baseline (the reference's
// own C++ needs Boost, HDF5 and MPI and is not built), and tests/ check it
// against the numpy oracle.  The product never loads it.
//
// Per live walker, as DQMC/DQMCWalker.cpp:441-503 (restricted integrals):
//   theta_c = psi_c (Phi_c^T psi_c)^-1 per trial channel (DQMC/RHF.cpp:46-47),
//   force bias fb_g = mult sum_c sum_k rot_c[g][k] theta_c[k] (RHF.cpp:42-61),
//   shifted fields, shift and fbTerm (DQMCWalker.cpp:451-457), the fields in
//   complex<float>,
//   VHS V = sqrt(dt) (i L.Re(x) - L.Im(x)) from the packed FP32 Cholesky
//   triangle, FP32 accumulation (DQMCWalker.cpp:406-421; FP64 on request),
//   det <- B det, det <- det + sum_{k=1..5} V^k det / k! by temp <- V temp / k,
//   det <- B det (DQMCWalker.cpp:424-431, :478-489),
//   new overlap prod_c det(Phi_c^T psi_c)^mult, the phaseless importance
//   function and its [1e-3, 100] window (DQMCWalker.cpp:492-502),
// then the weight cap and the population-control shift
// (DQMC/MixedEstimator.cpp:461-475); every `ortho_every` steps a QR of every
// walker's spin blocks with the overlap divided by prod diag(R)
// (DQMCWalker.cpp:295-326; modified Gram-Schmidt here: the same Q up to column
// signs, which the stored overlap carries), and every `energy_every` steps the
// local energy E_L = ecore + mult sum_c tr(theta_c^T h1 Phi_c) + 1/2 sum_{g <
// ncholEne} [(mult sum_c tr f_cg)^2 - mult sum_c sum_ij f_cg[i,j] f_cg[j,i]],
// f_cg = rot_c[g] theta_c (RHF.cpp:70-131, UHF.cpp:75-140).
//
// Complex matrices are stored as separate real and imaginary planes, column
// major, so the inner loops are unit-stride and vectorise at -O3.  Walkers are
// independent between measurements, so OpenMP threads over walkers stand in
// for the reference's one MPI rank per core.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <complex>
#include <random>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

using cd = std::complex<double>;

struct CpuCase {
  int N, G, Gene;           // orbitals, Cholesky vectors, vectors used by the energy
  int nchan, mult;          // trial channels; multiplicity (2: RHF trial x restricted walker)
  int ncw, nce;             // walker det columns; channel columns (sum of the channels' n)
  int ch_n[2], ch_psi_off[2], ch_col_off[2];
  int nblk;                 // walker spin blocks propagated (1 restricted, 2 unrestricted)
  int blk_c0[2], blk_nc[2];
  int vhs_fp64;             // 1: FP64 VHS from L64 (the FP64 oracle's arithmetic)
  double dt, ecore, pc_re, pc_im;
  const double* phi;        // [nce][N]
  const double* rot;        // [G][nce N]    rot[g][col N + p] = (Phi^T L_g)[col, p]
  const double* rotT;       // [nce N][G]
  const double* h1phi;      // [nce][N]
  const float* L32;         // [G][T]        packed lower triangle, FP32
  const double* L64;        // [G][T]        packed lower triangle, FP64 (vhs_fp64)
  const double* B_re;       // [N][N]        exp(-dt/2 h1'), column major
  const double* B_im;
  const double* mf_re;      // [G]
  const double* mf_im;
};

namespace {

struct Scratch {
  std::vector<double> thr, thi;        // theta planes [nce][N]
  std::vector<double> thTr, thTi;      // theta transposed per channel [N][n]
  std::vector<cd> M, Minv;             // n x n
  std::vector<int> piv;
  std::vector<double> fbr, fbi;        // [G]
  std::vector<float> xr, xi;           // fields [G], complex<float> as the reference
  std::vector<double> xr64, xi64;      // the same unrounded (FP64 VHS)
  std::vector<float> vr32, vi32;       // packed VHS [T]
  std::vector<double> vr64, vi64;
  std::vector<double> Vr, Vi;          // [N][N] column major
  std::vector<double> ar, ai, tr, ti, cr, ci;  // [N][nmax] work blocks
  std::vector<double> fr, fi;          // [n][n]
  std::mt19937_64 gen;
  std::normal_distribution<double> normal{0.0, 1.0};
};

struct State {
  CpuCase c;
  int W = 0;
  std::vector<double> pr, pi;  // [W][ncw][N]
  std::vector<cd> ovlp;        // [W]
  std::vector<double> w;       // [W]
  std::vector<Scratch> scr;
};

void init_scratch(const CpuCase& c, Scratch& s, uint64_t seed) {
  const int N = c.N, T = N * (N + 1) / 2;
  int nmax = 0;
  for (int i = 0; i < c.nchan; ++i) nmax = std::max(nmax, c.ch_n[i]);
  for (int b = 0; b < c.nblk; ++b) nmax = std::max(nmax, c.blk_nc[b]);
  s.thr.assign((size_t)c.nce * N, 0.0);
  s.thi.assign((size_t)c.nce * N, 0.0);
  s.thTr.assign((size_t)N * nmax, 0.0);
  s.thTi.assign((size_t)N * nmax, 0.0);
  s.M.assign((size_t)nmax * nmax, 0.0);
  s.Minv.assign((size_t)nmax * nmax, 0.0);
  s.piv.assign(nmax, 0);
  s.fbr.assign(c.G, 0.0);
  s.fbi.assign(c.G, 0.0);
  s.xr.assign(c.G, 0.f);
  s.xi.assign(c.G, 0.f);
  s.xr64.assign(c.G, 0.0);
  s.xi64.assign(c.G, 0.0);
  s.vr32.assign(T, 0.f);
  s.vi32.assign(T, 0.f);
  s.vr64.assign(T, 0.0);
  s.vi64.assign(T, 0.0);
  s.Vr.assign((size_t)N * N, 0.0);
  s.Vi.assign((size_t)N * N, 0.0);
  for (auto* v : {&s.ar, &s.ai, &s.tr, &s.ti, &s.cr, &s.ci}) v->assign((size_t)N * nmax, 0.0);
  s.fr.assign((size_t)nmax * nmax, 0.0);
  s.fi.assign((size_t)nmax * nmax, 0.0);
  s.gen.seed(seed);
}

// LU with partial pivoting of the n x n complex matrix A (column major, in
// place); returns the determinant.
cd lu(cd* A, int n, int* piv) {
  cd det = 1.0;
  for (int k = 0; k < n; ++k) {
    int p = k;
    double best = std::abs(A[(size_t)k * n + k]);
    for (int i = k + 1; i < n; ++i) {
      const double a = std::abs(A[(size_t)k * n + i]);
      if (a > best) { best = a; p = i; }
    }
    piv[k] = p;
    if (p != k) {
      for (int j = 0; j < n; ++j) std::swap(A[(size_t)j * n + k], A[(size_t)j * n + p]);
      det = -det;
    }
    const cd d = A[(size_t)k * n + k];
    det *= d;
    if (d == 0.0) continue;
    const cd inv = 1.0 / d;
    for (int i = k + 1; i < n; ++i) A[(size_t)k * n + i] *= inv;
    for (int j = k + 1; j < n; ++j) {
      const cd a = A[(size_t)j * n + k];
      if (a == 0.0) continue;
      for (int i = k + 1; i < n; ++i) A[(size_t)j * n + i] -= A[(size_t)k * n + i] * a;
    }
  }
  return det;
}

// inverse from the LU factors (column major)
void lu_inverse(const cd* LU, const int* piv, int n, cd* X) {
  for (int j = 0; j < n; ++j) {
    cd* x = X + (size_t)j * n;
    for (int i = 0; i < n; ++i) x[i] = (i == j) ? 1.0 : 0.0;
    for (int k = 0; k < n; ++k)
      if (piv[k] != k) std::swap(x[k], x[piv[k]]);
    for (int k = 0; k < n; ++k)  // L y = x (unit diagonal)
      for (int i = k + 1; i < n; ++i) x[i] -= LU[(size_t)k * n + i] * x[k];
    for (int k = n - 1; k >= 0; --k) {  // U z = y
      x[k] /= LU[(size_t)k * n + k];
      for (int i = 0; i < k; ++i) x[i] -= LU[(size_t)k * n + i] * x[k];
    }
  }
}

// M = Phi_c^T psi_c (n x n), from walker w's det
void overlap_matrix(const CpuCase& c, const double* pr, const double* pi, int ch, cd* M) {
  const int N = c.N, n = c.ch_n[ch];
  for (int j = 0; j < n; ++j) {
    const double* xr = pr + (size_t)(c.ch_psi_off[ch] + j) * N;
    const double* xi = pi + (size_t)(c.ch_psi_off[ch] + j) * N;
    for (int i = 0; i < n; ++i) {
      const double* ph = c.phi + (size_t)(c.ch_col_off[ch] + i) * N;
      double sr = 0.0, si = 0.0;
      for (int p = 0; p < N; ++p) {
        sr += ph[p] * xr[p];
        si += ph[p] * xi[p];
      }
      M[(size_t)j * n + i] = cd(sr, si);
    }
  }
}

// overlap prod_c det(M_c)^mult, and theta of every channel when want_theta
cd overlap_theta(const CpuCase& c, const double* pr, const double* pi, Scratch& s, bool want_theta) {
  const int N = c.N;
  cd ov = 1.0;
  for (int ch = 0; ch < c.nchan; ++ch) {
    const int n = c.ch_n[ch];
    overlap_matrix(c, pr, pi, ch, s.M.data());
    const cd d = lu(s.M.data(), n, s.piv.data());
    ov *= c.mult == 2 ? d * d : d;
    if (!want_theta) continue;
    lu_inverse(s.M.data(), s.piv.data(), n, s.Minv.data());
    // theta[:, i] = sum_j psi[:, j] Minv[j][i]
    for (int i = 0; i < n; ++i) {
      double* tr = s.thr.data() + (size_t)(c.ch_col_off[ch] + i) * N;
      double* ti = s.thi.data() + (size_t)(c.ch_col_off[ch] + i) * N;
      std::fill(tr, tr + N, 0.0);
      std::fill(ti, ti + N, 0.0);
      for (int j = 0; j < n; ++j) {
        const cd m = s.Minv[(size_t)i * n + j];
        const double mr = m.real(), mi = m.imag();
        const double* xr = pr + (size_t)(c.ch_psi_off[ch] + j) * N;
        const double* xi = pi + (size_t)(c.ch_psi_off[ch] + j) * N;
        for (int p = 0; p < N; ++p) {
          tr[p] += xr[p] * mr - xi[p] * mi;
          ti[p] += xr[p] * mi + xi[p] * mr;
        }
      }
    }
  }
  return ov;
}

// C (N x m) = A (N x N) X (N x m), complex planes, column major
void cgemm(int N, int m, const double* Ar, const double* Ai, const double* Xr, const double* Xi, double* Cr,
           double* Ci) {
  std::fill(Cr, Cr + (size_t)N * m, 0.0);
  std::fill(Ci, Ci + (size_t)N * m, 0.0);
  for (int j = 0; j < m; ++j) {
    double* cr = Cr + (size_t)j * N;
    double* ci = Ci + (size_t)j * N;
    for (int k = 0; k < N; ++k) {
      const double xr = Xr[(size_t)j * N + k], xi = Xi[(size_t)j * N + k];
      const double* ar = Ar + (size_t)k * N;
      const double* ai = Ai + (size_t)k * N;
      for (int p = 0; p < N; ++p) {
        cr[p] += ar[p] * xr - ai[p] * xi;
        ci[p] += ar[p] * xi + ai[p] * xr;
      }
    }
  }
}

// one phaseless step of walker w; returns the importance factor (0 = dies)
double walker_step(State& st, int w, Scratch& s, const double* xi_in, double eshift) {
  const CpuCase& c = st.c;
  const int N = c.N, G = c.G, T = N * (N + 1) / 2;
  double* pr = st.pr.data() + (size_t)w * c.ncw * N;
  double* pi = st.pi.data() + (size_t)w * c.ncw * N;
  overlap_theta(c, pr, pi, s, true);
  // force bias
  std::fill(s.fbr.begin(), s.fbr.end(), 0.0);
  std::fill(s.fbi.begin(), s.fbi.end(), 0.0);
  for (int k = 0; k < c.nce * N; ++k) {
    const double tr = s.thr[k], ti = s.thi[k];
    const double* r = c.rotT + (size_t)k * G;
    for (int g = 0; g < G; ++g) {
      s.fbr[g] += r[g] * tr;
      s.fbi[g] += r[g] * ti;
    }
  }
  // shifted fields
  const double sdt = sqrt(c.dt);
  cd shift = 0.0, fbterm = 0.0;
  for (int g = 0; g < G; ++g) {
    const double field = xi_in ? xi_in[g] : s.normal(s.gen);
    const cd fb(c.mult * s.fbr[g], c.mult * s.fbi[g]);
    const cd mf(c.mf_re[g], c.mf_im[g]);
    const cd fs = -sdt * (cd(0.0, 1.0) * fb - mf);
    const std::complex<float> x = std::complex<float>(field - fs);
    s.xr[g] = x.real();
    s.xi[g] = x.imag();
    s.xr64[g] = (field - fs).real();
    s.xi64[g] = (field - fs).imag();
    shift += (field - fs) * mf;
    fbterm += field * fs - fs * fs / 2.0;
  }
  // VHS, packed, then the full symmetric matrix times sqrt(dt)
  if (c.vhs_fp64) {
    std::fill(s.vr64.begin(), s.vr64.end(), 0.0);
    std::fill(s.vi64.begin(), s.vi64.end(), 0.0);
    for (int g = 0; g < G; ++g) {
      const double xr = s.xr64[g], xi = s.xi64[g];
      const double* L = c.L64 + (size_t)g * T;
      for (int t = 0; t < T; ++t) {
        s.vr64[t] += xr * L[t];
        s.vi64[t] += xi * L[t];
      }
    }
  } else {
    std::fill(s.vr32.begin(), s.vr32.end(), 0.f);
    std::fill(s.vi32.begin(), s.vi32.end(), 0.f);
    for (int g = 0; g < G; ++g) {
      const float xr = s.xr[g], xi = s.xi[g];
      const float* L = c.L32 + (size_t)g * T;
      for (int t = 0; t < T; ++t) {
        s.vr32[t] += xr * L[t];
        s.vi32[t] += xi * L[t];
      }
    }
  }
  for (int i = 0; i < N; ++i)
    for (int j = 0; j <= i; ++j) {
      const int t = i * (i + 1) / 2 + j;
      const double re = c.vhs_fp64 ? -s.vi64[t] : (double)(-s.vi32[t]);
      const double im = c.vhs_fp64 ? s.vr64[t] : (double)s.vr32[t];
      s.Vr[(size_t)j * N + i] = s.Vr[(size_t)i * N + j] = sdt * re;
      s.Vi[(size_t)j * N + i] = s.Vi[(size_t)i * N + j] = sdt * im;
    }
  // B exp-Taylor(V) B on each spin block
  for (int b = 0; b < c.nblk; ++b) {
    const int m = c.blk_nc[b];
    double* dr = pr + (size_t)c.blk_c0[b] * N;
    double* di = pi + (size_t)c.blk_c0[b] * N;
    cgemm(N, m, c.B_re, c.B_im, dr, di, s.ar.data(), s.ai.data());  // a = B det
    std::copy(s.ar.begin(), s.ar.begin() + (size_t)N * m, s.tr.begin());
    std::copy(s.ai.begin(), s.ai.begin() + (size_t)N * m, s.ti.begin());
    for (int k = 1; k < 6; ++k) {
      cgemm(N, m, s.Vr.data(), s.Vi.data(), s.tr.data(), s.ti.data(), s.cr.data(), s.ci.data());
      const double inv = 1.0 / k;
      for (size_t e = 0; e < (size_t)N * m; ++e) {
        s.tr[e] = s.cr[e] * inv;
        s.ti[e] = s.ci[e] * inv;
        s.ar[e] += s.tr[e];
        s.ai[e] += s.ti[e];
      }
    }
    cgemm(N, m, c.B_re, c.B_im, s.ar.data(), s.ai.data(), dr, di);
  }
  // phaseless importance function
  const cd old_ov = st.ovlp[w];
  const cd new_ov = overlap_theta(c, pr, pi, s, false);
  const cd ratio = new_ov / old_ov;
  const cd imp = std::exp(-sdt * shift + fbterm + c.dt * (eshift + cd(c.pc_re, c.pc_im))) * ratio;
  const double th = std::arg(std::exp(-sdt * shift) * ratio);
  double val = std::abs(imp) * cos(th);
  if (val < 1.0e-3 || val > 100.0 || std::isnan(val)) val = 0.0;
  st.ovlp[w] = new_ov;
  return val;
}

void walker_qr(State& st, int w) {
  const CpuCase& c = st.c;
  const int N = c.N;
  double* pr = st.pr.data() + (size_t)w * c.ncw * N;
  double* pi = st.pi.data() + (size_t)w * c.ncw * N;
  cd fac = 1.0;
  for (int b = 0; b < c.nblk; ++b) {
    for (int j = 0; j < c.blk_nc[b]; ++j) {
      double* ar = pr + (size_t)(c.blk_c0[b] + j) * N;
      double* ai = pi + (size_t)(c.blk_c0[b] + j) * N;
      for (int i = 0; i < j; ++i) {
        const double* qr = pr + (size_t)(c.blk_c0[b] + i) * N;
        const double* qi = pi + (size_t)(c.blk_c0[b] + i) * N;
        double sr = 0.0, si = 0.0;  // <q_i, a_j>
        for (int p = 0; p < N; ++p) {
          sr += qr[p] * ar[p] + qi[p] * ai[p];
          si += qr[p] * ai[p] - qi[p] * ar[p];
        }
        for (int p = 0; p < N; ++p) {
          ar[p] -= sr * qr[p] - si * qi[p];
          ai[p] -= sr * qi[p] + si * qr[p];
        }
      }
      double nrm = 0.0;
      for (int p = 0; p < N; ++p) nrm += ar[p] * ar[p] + ai[p] * ai[p];
      nrm = sqrt(nrm);
      const double inv = 1.0 / nrm;
      for (int p = 0; p < N; ++p) {
        ar[p] *= inv;
        ai[p] *= inv;
      }
      fac *= nrm;
    }
  }
  st.ovlp[w] /= (c.nblk == 1 && c.mult == 2) ? fac * fac : fac;
}

cd walker_energy(State& st, int w, Scratch& s) {
  const CpuCase& c = st.c;
  const int N = c.N;
  const double* pr = st.pr.data() + (size_t)w * c.ncw * N;
  const double* pi = st.pi.data() + (size_t)w * c.ncw * N;
  overlap_theta(c, pr, pi, s, true);
  cd e1 = 0.0;
  for (int k = 0; k < c.nce * N; ++k) e1 += cd(s.thr[k], s.thi[k]) * c.h1phi[k];
  cd e = c.ecore + (double)c.mult * e1;
  std::vector<cd> csum(c.Gene, 0.0);
  cd exch = 0.0;
  for (int ch = 0; ch < c.nchan; ++ch) {
    const int n = c.ch_n[ch], off = c.ch_col_off[ch];
    for (int p = 0; p < N; ++p)  // theta transposed: [p][j]
      for (int j = 0; j < n; ++j) {
        s.thTr[(size_t)p * n + j] = s.thr[(size_t)(off + j) * N + p];
        s.thTi[(size_t)p * n + j] = s.thi[(size_t)(off + j) * N + p];
      }
    for (int g = 0; g < c.Gene; ++g) {
      std::fill(s.fr.begin(), s.fr.begin() + (size_t)n * n, 0.0);
      std::fill(s.fi.begin(), s.fi.begin() + (size_t)n * n, 0.0);
      const double* rg = c.rot + (size_t)g * c.nce * N;
      for (int i = 0; i < n; ++i) {
        const double* r = rg + (size_t)(off + i) * N;
        double* fr = s.fr.data() + (size_t)i * n;
        double* fi = s.fi.data() + (size_t)i * n;
        for (int p = 0; p < N; ++p) {
          const double a = r[p];
          const double* tr = s.thTr.data() + (size_t)p * n;
          const double* ti = s.thTi.data() + (size_t)p * n;
          for (int j = 0; j < n; ++j) {
            fr[j] += a * tr[j];
            fi[j] += a * ti[j];
          }
        }
      }
      cd tr = 0.0, x = 0.0;
      for (int i = 0; i < n; ++i) {
        tr += cd(s.fr[(size_t)i * n + i], s.fi[(size_t)i * n + i]);
        for (int j = 0; j < n; ++j)
          x += cd(s.fr[(size_t)i * n + j], s.fi[(size_t)i * n + j]) * cd(s.fr[(size_t)j * n + i], s.fi[(size_t)j * n + i]);
      }
      csum[g] += tr;
      exch += x;
    }
  }
  cd coul = 0.0;
  for (int g = 0; g < c.Gene; ++g) coul += ((double)c.mult * csum[g]) * ((double)c.mult * csum[g]);
  return e + 0.5 * (coul - (double)c.mult * exch);
}

int nthreads_or_default(int nt) {
#ifdef _OPENMP
  return nt > 0 ? nt : omp_get_max_threads();
#else
  (void)nt;
  return 1;
#endif
}

}  // namespace

extern "C" {

void* cpu_create(const CpuCase* c, int W, uint64_t seed, int nthreads) {
  State* st = new State();
  st->c = *c;
  st->W = W;
  st->pr.assign((size_t)W * c->ncw * c->N, 0.0);
  st->pi.assign((size_t)W * c->ncw * c->N, 0.0);
  st->ovlp.assign(W, 1.0);
  st->w.assign(W, 1.0);
  const int nt = nthreads_or_default(nthreads);
  st->scr.resize(nt);
  for (int t = 0; t < nt; ++t) init_scratch(*c, st->scr[t], seed * 1000003ull + (uint64_t)t);
  return st;
}

void cpu_destroy(void* h) { delete (State*)h; }

int cpu_nthreads(void* h) { return (int)((State*)h)->scr.size(); }

// dets: [W][ncw][N] complex interleaved; overlaps [W] complex (NULL: computed); weights [W] (NULL: 1)
int cpu_set_walkers(void* h, const double* dets, const double* ovl, const double* w) {
  State* st = (State*)h;
  const size_t n = (size_t)st->W * st->c.ncw * st->c.N;
  for (size_t e = 0; e < n; ++e) {
    st->pr[e] = dets[2 * e];
    st->pi[e] = dets[2 * e + 1];
  }
  for (int k = 0; k < st->W; ++k) st->w[k] = w ? w[k] : 1.0;
  if (ovl) {
    for (int k = 0; k < st->W; ++k) st->ovlp[k] = cd(ovl[2 * k], ovl[2 * k + 1]);
  } else {
    for (int k = 0; k < st->W; ++k)
      st->ovlp[k] = overlap_theta(st->c, st->pr.data() + (size_t)k * st->c.ncw * st->c.N,
                                  st->pi.data() + (size_t)k * st->c.ncw * st->c.N, st->scr[0], false);
  }
  return 0;
}

int cpu_get_walkers(void* h, double* dets, double* ovl, double* w) {
  State* st = (State*)h;
  const size_t n = (size_t)st->W * st->c.ncw * st->c.N;
  if (dets)
    for (size_t e = 0; e < n; ++e) {
      dets[2 * e] = st->pr[e];
      dets[2 * e + 1] = st->pi[e];
    }
  for (int k = 0; k < st->W; ++k) {
    if (ovl) { ovl[2 * k] = st->ovlp[k].real(); ovl[2 * k + 1] = st->ovlp[k].imag(); }
    if (w) w[k] = st->w[k];
  }
  return 0;
}

// One step of every live walker (weight > 1e-8) with the weight cap; xi [W][G]
// host fields or NULL (each thread's own mt19937_64 + normal_distribution).
// Returns the sum of weights after the step.
double cpu_step(void* h, const double* xi, double eshift, double weight_cap) {
  State* st = (State*)h;
  const int W = st->W, G = st->c.G;
  const int nt = (int)st->scr.size();
  double sumw = 0.0;
#pragma omp parallel for num_threads(nt) schedule(static) reduction(+ : sumw)
  for (int w = 0; w < W; ++w) {
#ifdef _OPENMP
    Scratch& s = st->scr[omp_get_thread_num()];
#else
    Scratch& s = st->scr[0];
#endif
    if (st->w[w] > 1.0e-8) {
      double wt = st->w[w] * walker_step(*st, w, s, xi ? xi + (size_t)w * G : nullptr, eshift);
      if (wt > weight_cap) wt = 0.0;
      st->w[w] = wt;
    }
    sumw += st->w[w];
  }
  return sumw;
}

int cpu_orthonormalize(void* h) {
  State* st = (State*)h;
  const int nt = (int)st->scr.size();
#pragma omp parallel for num_threads(nt) schedule(static)
  for (int w = 0; w < st->W; ++w) walker_qr(*st, w);
  return 0;
}

// local energies of the walkers with weight != 0 (others 0): eloc [W] complex
int cpu_local_energy(void* h, double* eloc) {
  State* st = (State*)h;
  const int nt = (int)st->scr.size();
#pragma omp parallel for num_threads(nt) schedule(static)
  for (int w = 0; w < st->W; ++w) {
#ifdef _OPENMP
    Scratch& s = st->scr[omp_get_thread_num()];
#else
    Scratch& s = st->scr[0];
#endif
    cd e = st->w[w] != 0.0 ? walker_energy(*st, w, s) : cd(0.0);
    if (eloc) { eloc[2 * w] = e.real(); eloc[2 * w + 1] = e.imag(); }
  }
  return 0;
}

// Timed loop: nsteps steps with population control from e_est
// (eshift = e_est - 0.1 ln(sum_w / W) / dt), QR every ortho_every steps, an
// exact energy of every live walker every energy_every steps.  out: seconds
// in the steps, in the QR, in the energies, and the walker-steps done.
int cpu_run_timed(void* h, int nsteps, int ortho_every, int energy_every, double e_est, double weight_cap,
                  double* out) {
  State* st = (State*)h;
  using clk = std::chrono::steady_clock;
  double t_step = 0.0, t_qr = 0.0, t_e = 0.0, ws = 0.0;
  double eshift = e_est;
  for (int k = 1; k <= nsteps; ++k) {
    auto t0 = clk::now();
    const double sw = cpu_step(h, nullptr, eshift, weight_cap);
    auto t1 = clk::now();
    t_step += std::chrono::duration<double>(t1 - t0).count();
    ws += st->W;
    eshift = e_est - 0.1 * log(std::max(sw, 1e-300) / st->W) / st->c.dt;
    if (ortho_every > 0 && k % ortho_every == 0) {
      t0 = clk::now();
      cpu_orthonormalize(h);
      t_qr += std::chrono::duration<double>(clk::now() - t0).count();
    }
    if (energy_every > 0 && k % energy_every == 0) {
      t0 = clk::now();
      cpu_local_energy(h, nullptr);
      t_e += std::chrono::duration<double>(clk::now() - t0).count();
    }
  }
  out[0] = t_step;
  out[1] = t_qr;
  out[2] = t_e;
  out[3] = ws;
  return 0;
}

}  // extern "C"
