// solver.cu -- set-up and driver of the batched Poisson/Helmholtz solve.
//
// Assembly follows solver.f90:158-372 (init_matrix_3d) and 687-842 + 981-1020
// (init_matrix_2d, init_n_2d_matrices): 7- or 5-point operators weighted by the
// cell volume/area, boundary folding with sgn = +1 (N), -1 (centred D),
// 0 (staggered D), and lambda(k)*dl1_2*dl2_2 on the diagonal of wavenumber k.
// The hierarchy is built here once: axes are halved only where every block
// keeps an even extent and offset and where the coupling is strong
// (semicoarsening as PFMG does); coarse operators are rediscretised from the
// summed cell widths; the coarsest level is inverted densely per system.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <cstdlib>

#include "snac_host.h"
#include "snac_prof.h"

namespace snac {

int fft_setup(PoissonSolver &S);

void *PoissonSolver::alloc(size_t bytes) {
  void *p = nullptr;
  if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
  cudaMemset(p, 0, bytes);
  allocs.push_back(p);
  return p;
}
PoissonSolver::~PoissonSolver() {
  if (inner_exec) cudaGraphExecDestroy(inner_exec);
  for (void *p : allocs) cudaFree(p);
  if (W64.h_count) cudaFreeHost(W64.h_count);
  if (W32.h_count) cudaFreeHost(W32.h_count);
  if (h_ocount) cudaFreeHost(h_ocount);
}

namespace {

struct HLevel {
  int n[3] = {1, 1, 1};
  long ncell = 1;
  int coarsened[3] = {0, 0, 0};
  std::vector<double> W[3];
  std::vector<unsigned short> code;
  std::vector<double> cc, cp[3];
  std::vector<double> dinv;
};

inline int fold_type(char cbc, int centered) {
  if (cbc == 'N') return 1;
  if (cbc == 'D') return centered ? 2 : 3;
  return 0;
}
inline double fold_sgn(int t) { return t == 1 ? 1.0 : (t == 2 ? -1.0 : 0.0); }

struct Builder {
  PoissonSolver &S;
  std::vector<HLevel> L;
  int na;
  explicit Builder(PoissonSolver &s) : S(s), na(s.mode3d ? 3 : 2) {}

  long nbr(const HLevel &l, int i, int j, int k, int a, int s) const {
    int c[3] = {i, j, k};
    c[a] += s ? 1 : -1;
    if (c[a] < 0 || c[a] >= l.n[a]) {
      if (!S.periodic[a]) return -1;
      c[a] = c[a] < 0 ? c[a] + l.n[a] : c[a] - l.n[a];
    }
    return c[0] + (long)l.n[0] * (c[1] + (long)l.n[1] * c[2]);
  }

  void alloc_level(HLevel &l) {
    l.ncell = (long)l.n[0] * l.n[1] * l.n[2];
    for (int a = 0; a < 3; a++) { l.W[a].assign(l.n[a], 0.0); l.cp[a].assign(l.ncell, 0.0); }
    l.code.assign(l.ncell, 0x8000);
    l.cc.assign(l.ncell, 0.0);
  }

  // rediscretised operator of a coarse level
  void coarse_operator(HLevel &l, double alpha) {
    for (int k = 0; k < l.n[2]; k++)
      for (int j = 0; j < l.n[1]; j++)
        for (int i = 0; i < l.n[0]; i++) {
          const long c = i + (long)l.n[0] * (j + (long)l.n[1] * k);
          const int idx[3] = {i, j, k};
          for (int a = 0; a < 3; a++) l.cp[a][c] = 0.0;
          l.cc[c] = 0.0;
          if (l.code[c] & 0x8000) continue;
          double weight = 1.0;
          for (int a = 0; a < na; a++) weight *= l.W[a][idx[a]];
          double cm[3] = {0, 0, 0}, cpv[3] = {0, 0, 0}, sum = 0.0;
          for (int a = 0; a < na; a++) {
            if (S.periodic[a] && l.n[a] == 1) continue;
            double wt = 1.0;
            for (int b = 0; b < na; b++)
              if (b != a) wt *= l.W[b][idx[b]];
            const int n = l.n[a], q = idx[a];
            const double Wq = l.W[a][q];
            const double Wm = q > 0 ? l.W[a][q - 1] : (S.periodic[a] ? l.W[a][n - 1] : Wq);
            const double Wp = q < n - 1 ? l.W[a][q + 1] : (S.periodic[a] ? l.W[a][0] : Wq);
            const int tm = (l.code[c] >> (2 * (2 * a))) & 3, tp = (l.code[c] >> (2 * (2 * a + 1))) & 3;
            const double dm = tm ? Wq : 0.5 * (Wm + Wq);
            const double dp = tp ? Wq : 0.5 * (Wq + Wp);
            cm[a] = 1.0 / dm * wt;
            cpv[a] = 1.0 / dp * wt;
            sum += cm[a] + cpv[a];
          }
          double cc = -sum + alpha * weight;
          for (int a = 0; a < na; a++) {
            const int tm = (l.code[c] >> (2 * (2 * a))) & 3, tp = (l.code[c] >> (2 * (2 * a + 1))) & 3;
            if (tm) { cc += fold_sgn(tm) * cm[a]; cm[a] = 0; }
            if (tp) { cc += fold_sgn(tp) * cpv[a]; cpv[a] = 0; }
            l.cp[a][c] = cpv[a];
          }
          l.cc[c] = cc;
        }
  }

  double diag(const HLevel &l, long c, int i, int j, int s) const {
    if (S.mode3d) return l.cc[c];
    return l.cc[c] + S.lambda[s] * l.W[0][i] * l.W[1][j];
  }

  // dense inverse of the coarsest operator of system s (Cholesky of -A, +11^T when singular)
  bool dense(const HLevel &l, int s, bool singular, double *M) const {
    const long n = l.ncell;
    std::vector<double> A((size_t)n * n, 0.0);
    for (int k = 0; k < l.n[2]; k++)
      for (int j = 0; j < l.n[1]; j++)
        for (int i = 0; i < l.n[0]; i++) {
          const long c = i + (long)l.n[0] * (j + (long)l.n[1] * k);
          if (l.code[c] & 0x8000) continue;
          A[c * n + c] -= diag(l, c, i, j, s);
          for (int a = 0; a < na; a++) {
            if (S.periodic[a] && l.n[a] == 1) continue;
            const long p = nbr(l, i, j, k, a, 1), m = nbr(l, i, j, k, a, 0);
            if (p >= 0) A[c * n + p] -= l.cp[a][c];
            if (m >= 0) A[c * n + m] -= l.cp[a][m];
          }
        }
    long nact = 0;
    double dsum = 0.0;
    for (long c = 0; c < n; c++) {
      if (l.code[c] & 0x8000) { A[c * n + c] = 1.0; continue; }
      nact++;
      dsum += A[c * n + c];
    }
    if (singular && nact > 0) {
      const double sh = dsum / nact;
      for (long r = 0; r < n; r++)
        for (long c = 0; c < n; c++)
          if (!(l.code[r] & 0x8000) && !(l.code[c] & 0x8000)) A[r * n + c] += sh;
    }
    for (long j = 0; j < n; j++) {
      double d = A[j * n + j];
      for (long k = 0; k < j; k++) d -= A[j * n + k] * A[j * n + k];
      if (d <= 0.0) return false;
      d = std::sqrt(d);
      A[j * n + j] = d;
      for (long i = j + 1; i < n; i++) {
        double v = A[i * n + j];
        for (long k = 0; k < j; k++) v -= A[i * n + k] * A[j * n + k];
        A[i * n + j] = v / d;
      }
    }
    std::vector<double> e(n);
    for (long c = 0; c < n; c++) {
      std::fill(e.begin(), e.end(), 0.0);
      e[c] = 1.0;
      for (long i = 0; i < n; i++) { double v = e[i]; for (long k = 0; k < i; k++) v -= A[i * n + k] * e[k]; e[i] = v / A[i * n + i]; }
      for (long i = n - 1; i >= 0; i--) { double v = e[i]; for (long k = i + 1; k < n; k++) v -= A[k * n + i] * e[k]; e[i] = v / A[i * n + i]; }
      // stored by columns, M[c n + r] = inverse(r, c): a warp of consecutive rows reads contiguous memory
      for (long r = 0; r < n; r++) M[c * n + r] = ((l.code[r] & 0x8000) || (l.code[c] & 0x8000)) ? 0.0 : -e[r];
    }
    return true;
  }
};

}  // namespace

char field_cbc(const HostBlock &H, int field, int p, int side) {
  if (field == HF_P) return H.desc.cbcpre[p][side];
  if (field < HF_S0) return H.desc.cbcvel[field][p][side];
  return H.desc.cbcscal[field - HF_S0][p][side];
}
double field_bc(const HostBlock &H, int field, int p, int side) {
  if (field == HF_P) return H.desc.bcpre[p][side];
  if (field < HF_S0) return H.desc.bcvel[field][p][side];
  return H.desc.bcscal[field - HF_S0][p][side];
}

// init_bc_rhs (solver.f90:44-157) of a field in 3-D mode over lo..hif, with the field's centring,
// spacings and boundary values; dl is dxc at lo-1 and hi along a centred axis, dxf at lo and hi along a
// staggered one (main.f90:725-727, 771-773).  Planes rhs?(.., .., 0:1) over the solved extents.  The
// velocity components pass the boundary-value planes bcu%x.. (main.f90:580-582: uniform bcvel, or the
// inflow planes on an inflow face), which scale a plane by bcval/bc where bc is nonzero (solver.f90:122-123);
// the scalars do not.
static void init_bc_rhs_field(const HostBlock &H, int field, const int periods[3], int fft_axis,
                              std::vector<double> rhs[3]) {
  int nf[3], cen[3], q3[3];
  const double *d1[3], *d2[3];
  double factor[3][2];
  for (int a = 0; a < 3; a++) {
    nf[a] = field_hi(H, field, a) - H.lo[a] + 1;
    cen[a] = field_centered(field, a);
    q3[a] = cen[a] ? 0 : 1;
    d1[a] = cen[a] ? H.g[a][0].data() : H.g[a][1].data();
    d2[a] = cen[a] ? H.g[a][1].data() : H.g[a][0].data();
    for (int s = 0; s < 2; s++) {
      factor[a][s] = 0.0;
      if (!H.is_bound[a][s]) continue;
      const char cb = field_cbc(H, field, a, s);
      const double bc = field_bc(H, field, a, s);
      const double dl = cen[a] ? H.dl[a][s] : H.g[a][1][s ? H.ng[a] : 1];
      if (cb == 'N') { factor[a][s] = 1.0 * dl * bc; if (s == 1) factor[a][s] = -factor[a][s]; }
      else if (cb == 'D') factor[a][s] = cen[a] ? -2.0 * bc : -1.0 * bc;
    }
  }
  rhs[0].assign((size_t)nf[1] * nf[2] * 2, 0.0);
  rhs[1].assign((size_t)nf[0] * nf[2] * 2, 0.0);
  rhs[2].assign((size_t)nf[0] * nf[1] * 2, 0.0);
  // local 1-based indices; with a transform axis the weight leaves it out (solver.f90:98-106)
  auto W = [&](int i, int j, int k) {
    if (fft_axis == 1) return d2[1][j] * d2[2][k];
    if (fft_axis == 2) return d2[0][i] * d2[2][k];
    if (fft_axis == 3) return d2[0][i] * d2[1][j];
    return d2[0][i] * d2[1][j] * d2[2][k];
  };
  const bool has_bcval = field >= HF_U && field < HF_S0;
  // bcval at local (1-based) in-plane indices p1, p2: the inflow plane on an inflow face (main.f90:605-625),
  // else the uniform bc
  auto scale = [&](double r, int a, int sd, int p1, int p2) {
    const double bc = field_bc(H, field, a, sd);
    if (!has_bcval || bc == 0.0) return r;
    double bv = bc;
    if (H.inflow[a][sd]) {
      const int t1 = a == 0 ? 1 : 0;
      bv = H.vin[a][sd][field - HF_U][p1 + (size_t)(H.ng[t1] + 2) * p2];
    }
    return r * bv / bc;
  };
  for (int idir = 0; idir < 3; idir++) {
    if (periods[idir] != 0) continue;
    const int n = nf[idir];
    for (int sd = 0; sd < (n > 1 ? 2 : 1); sd++) {
      if (!H.is_bound[idir][sd]) continue;
      const int cf = sd ? n : 1;  // boundary cell (local, 1-based)
      const double *a1 = d1[idir], *a2 = d2[idir];
      const double den = a1[cf - (1 - sd) + q3[idir]] * a2[cf];
      if (idir == 0)
        for (int k = 1; k <= nf[2]; k++)
          for (int j = 1; j <= nf[1]; j++)
            rhs[0][(j - 1) + (size_t)nf[1] * ((k - 1) + (size_t)nf[2] * sd)] = scale(factor[0][sd] * W(cf, j, k) / den, 0, sd, j, k);
      else if (idir == 1)
        for (int k = 1; k <= nf[2]; k++)
          for (int i = 1; i <= nf[0]; i++)
            rhs[1][(i - 1) + (size_t)nf[0] * ((k - 1) + (size_t)nf[2] * sd)] = scale(factor[1][sd] * W(i, cf, k) / den, 1, sd, i, k);
      else
        for (int j = 1; j <= nf[1]; j++)
          for (int i = 1; i <= nf[0]; i++)
            rhs[2][(i - 1) + (size_t)nf[0] * ((j - 1) + (size_t)nf[1] * sd)] = scale(factor[2][sd] * W(i, j, cf) / den, 2, sd, i, j);
    }
  }
}

// Build the box problem of a field: the pressure (centred in every direction, alpha = 0), or for
// IMPDIFF a velocity component (staggered along its own direction, one unknown fewer at a wall there,
// main.f90:771-826) or a scalar (centred), with the field's own boundary conditions.
int solver_create(Domain &d, PoissonSolver &S, bool upload, int field) {
  const snac_case &c = d.c;
  S.field = field;
  S.helm = field != HF_P;
  S.precision = d.opt.precision;
  const snac_options &o = d.opt;
  if (o.inner_iters > 0) S.inner_iters = o.inner_iters;
  if (o.inner_tol > 0.0) S.inner_tol = o.inner_tol;
  S.adapt_inner = o.inner_adapt >= 0;  // -1: every inner solve reduces by inner_tol, whatever the outer needs
  if (o.refine_steps > 0) S.refine_steps = o.refine_steps;
  S.use_graph = d.opt.use_graph ? 1 : 0;
  S.tol = c.tol;
  S.maxiter = c.maxiter;
  S.fft_axis = c.fft_axis;
  S.mode3d = c.fft_axis == 0;
  if (S.mode3d) { S.ax[0] = 0; S.ax[1] = 1; S.ax[2] = 2; }
  else {
    const int idir = c.fft_axis - 1;
    S.ax[0] = idir == 0 ? 1 : 0;
    S.ax[1] = idir == 2 ? 1 : 2;
    S.ax[2] = idir;
  }
  int lo_min[3], hi_max[3];
  for (int p = 0; p < 3; p++) {
    lo_min[p] = d.hb[0].lo[p];
    hi_max[p] = field_hi(d.hb[0], field, p);
    for (int b = 1; b < d.nblocks; b++) {
      lo_min[p] = std::min(lo_min[p], d.hb[b].lo[p]);
      hi_max[p] = std::max(hi_max[p], field_hi(d.hb[b], field, p));
    }
    S.lo_min[p] = lo_min[p];
  }
  Builder B(S);
  const int na = B.na;
  B.L.reserve(MG_MAXLEV);  // levels are appended below while references to level 0 are held
  B.L.resize(1);
  HLevel &L0 = B.L[0];
  for (int a = 0; a < 3; a++) {
    const int p = S.ax[a];
    L0.n[a] = a < na ? hi_max[p] - lo_min[p] + 1 : 1;
    S.periodic[a] = a < na ? (d.periods[p] != 0) : 0;
  }
  if (!S.mode3d) {
    const int pf = S.ax[2];
    S.nsys = hi_max[pf] - lo_min[pf] + 1;
    for (int b = 0; b < d.nblocks; b++)
      if (d.hb[b].lo[pf] != lo_min[pf] || field_hi(d.hb[b], field, pf) != hi_max[pf]) {
        set_error("every block must span the whole transform direction");
        return SNAC_ERR_UNSUPPORTED;
      }
    // fft.f90 set-up with the field's boundary pair and centring along the transform axis: kinds, the
    // transform length n - q (fftini drops the wall face of a staggered non-periodic component), normfft,
    // eigenvalues(n)/dl^2 (init_fft_reduction, solver.f90:1124-1138) of which the first nsys are used
    const HostBlock &H0 = d.hb[0];
    const int cen_f = field_centered(field, pf), n_full = H0.ng[pf];
    const char bc[2] = {field_cbc(H0, field, pf, 0), field_cbc(H0, field, pf, 1)};
    const int q = ((bc[0] == 'F' && bc[1] == 'F') || cen_f) ? 0 : 1;
    double norm[2];
    find_fft(bc[0], bc[1], cen_f, &S.kind_fwd, &S.kind_bwd, norm);
    if (S.kind_fwd < 0) { set_error("unsupported boundary pair along the transform direction"); return SNAC_ERR_UNSUPPORTED; }
    S.nfft = n_full - q;
    if (S.nfft != S.nsys) { set_error("transform length and solved extent differ along the transform direction"); return SNAC_ERR_UNSUPPORTED; }
    S.normfft = 1.0 / (norm[0] * (n_full + norm[1] - q));
    std::vector<double> lam(n_full, 0.0);
    if (eigenvalues(n_full, bc[0], bc[1], cen_f, lam.data())) {
      set_error("no eigenvalues for this boundary pair (the reference defines none)");
      return SNAC_ERR_UNSUPPORTED;
    }
    // dl(0, idir): dxc(lo-1) along a centred axis, dxf(lo) along a staggered one (main.f90:725, 771-773)
    const double dl0 = cen_f ? H0.dl[pf][0] : H0.g[pf][1][1];
    S.lambda.assign(lam.begin(), lam.begin() + S.nsys);
    for (auto &v : S.lambda) v = v / (dl0 * dl0);
    if (upload) SNAC_TRY(fft_setup(S));
  } else {
    S.nsys = 1;
    S.lambda.assign(1, 0.0);
  }
  B.alloc_level(L0);
  const double alpha = 0.0;
  int centered[3];
  for (int p = 0; p < 3; p++) centered[p] = field_centered(field, p);
  std::vector<double> cmv_all[3];
  for (int a = 0; a < 3; a++) cmv_all[a].assign(L0.ncell, 0.0);
  std::vector<char> have[3];
  for (int a = 0; a < 3; a++) have[a].assign(L0.n[a], 0);
  for (int b = 0; b < d.nblocks; b++) {
    const HostBlock &H = d.hb[b];
    const double *d1[3], *d2[3];
    int q3[3];
    for (int p = 0; p < 3; p++) {
      d1[p] = centered[p] ? H.g[p][0].data() : H.g[p][1].data();
      d2[p] = centered[p] ? H.g[p][1].data() : H.g[p][0].data();
      q3[p] = centered[p] ? 0 : 1;
    }
    auto LOC = [&](int p, int g) { return g - H.lo[p] + 1; };
    int loc[3], hic[3], bhi[3];
    for (int p = 0; p < 3; p++) bhi[p] = field_hi(H, field, p);
    for (int a = 0; a < 3; a++) {
      const int p = S.ax[a];
      loc[a] = a < na ? H.lo[p] : 0;
      hic[a] = a < na ? bhi[p] : 0;
    }
    for (int g2 = loc[2]; g2 <= hic[2]; g2++)
      for (int g1 = loc[1]; g1 <= hic[1]; g1++)
        for (int g0 = loc[0]; g0 <= hic[0]; g0++) {
          const int gg[3] = {g0, g1, g2};
          int idx[3];
          for (int a = 0; a < 3; a++) idx[a] = a < na ? gg[a] - lo_min[S.ax[a]] : 0;
          const long cidx = idx[0] + (long)L0.n[0] * (idx[1] + (long)L0.n[1] * idx[2]);
          if (!(L0.code[cidx] & 0x8000)) { set_error("overlapping blocks in the solver box"); return SNAC_ERR_ARG; }
          for (int a = 0; a < na; a++) {
            const int p = S.ax[a];
            const double wv = d2[p][LOC(p, gg[a])];
            if (have[a][idx[a]] && L0.W[a][idx[a]] != wv) {
              set_error("inconsistent grid spacing along axis %d at global index %d", p + 1, gg[a]);
              return SNAC_ERR_ARG;
            }
            L0.W[a][idx[a]] = wv;
            have[a][idx[a]] = 1;
          }
          double weight, cmv[3] = {0, 0, 0}, cpv[3] = {0, 0, 0}, cc;
          if (S.mode3d) {
            const double dx2 = d2[0][LOC(0, g0)], dy2 = d2[1][LOC(1, g1)], dz2 = d2[2][LOC(2, g2)];
            weight = dx2 * dy2 * dz2;
            cmv[0] = 1.0 / (d1[0][LOC(0, g0 - 1 + q3[0])]) * dy2 * dz2;
            cpv[0] = 1.0 / (d1[0][LOC(0, g0 + q3[0])]) * dy2 * dz2;
            cmv[1] = 1.0 / (d1[1][LOC(1, g1 - 1 + q3[1])]) * dx2 * dz2;
            cpv[1] = 1.0 / (d1[1][LOC(1, g1 + q3[1])]) * dx2 * dz2;
            cmv[2] = 1.0 / (d1[2][LOC(2, g2 - 1 + q3[2])]) * dx2 * dy2;
            cpv[2] = 1.0 / (d1[2][LOC(2, g2 + q3[2])]) * dx2 * dy2;
            // a periodic axis of one cell couples each cell to itself: its +/- terms cancel
            for (int a = 0; a < 3; a++)
              if (S.periodic[a] && L0.n[a] == 1) cmv[a] = cpv[a] = 0.0;
            cc = 0.0;
            cc = cc - (cmv[0] + cpv[0] + cmv[1] + cpv[1] + cmv[2] + cpv[2]) + alpha * weight;
          } else {
            const int p1 = S.ax[0], p2 = S.ax[1];
            const double w1 = d2[p1][LOC(p1, g0)], w2 = d2[p2][LOC(p2, g1)];
            weight = w1 * w2;
            cmv[0] = 1.0 / (d1[p1][LOC(p1, g0 - 1 + q3[p1])]) * w2;
            cpv[0] = 1.0 / (d1[p1][LOC(p1, g0 + q3[p1])]) * w2;
            cmv[1] = 1.0 / (d1[p2][LOC(p2, g1 - 1 + q3[p2])]) * w1;
            cpv[1] = 1.0 / (d1[p2][LOC(p2, g1 + q3[p2])]) * w1;
            for (int a = 0; a < 2; a++)  // a periodic axis of one cell: the self-couplings cancel
              if (S.periodic[a] && L0.n[a] == 1) cmv[a] = cpv[a] = 0.0;
            cc = -(cmv[0] + cpv[0] + cmv[1] + cpv[1]) + alpha * weight;
          }
          unsigned short code = 0;
          for (int a = 0; a < na; a++) {
            const int p = S.ax[a];
            if (d.periods[p] != 0) continue;
            if (H.is_bound[p][0] && gg[a] == H.lo[p]) {
              const int t = fold_type(field_cbc(H, field, p, 0), centered[p]);
              cc = cc + fold_sgn(t) * cmv[a];
              cmv[a] = 0.0;
              code |= (unsigned short)(t << (2 * (2 * a)));
            }
            if (H.is_bound[p][1] && gg[a] == bhi[p]) {
              const int t = fold_type(field_cbc(H, field, p, 1), centered[p]);
              cc = cc + fold_sgn(t) * cpv[a];
              cpv[a] = 0.0;
              code |= (unsigned short)(t << (2 * (2 * a + 1)));
            }
          }
          L0.code[cidx] = code;
          L0.cc[cidx] = cc;
          for (int a = 0; a < na; a++) { L0.cp[a][cidx] = cpv[a]; cmv_all[a][cidx] = cmv[a]; }
        }
  }
  // coupling consistency: cm(c) == cp(c - e_a) for coupled faces
  for (int k = 0; k < L0.n[2]; k++)
    for (int j = 0; j < L0.n[1]; j++)
      for (int i = 0; i < L0.n[0]; i++) {
        const long cidx = i + (long)L0.n[0] * (j + (long)L0.n[1] * k);
        if (L0.code[cidx] & 0x8000) continue;
        for (int a = 0; a < na; a++) {
          const long m = B.nbr(L0, i, j, k, a, 0);
          const int tm = (L0.code[cidx] >> (2 * (2 * a))) & 3;
          if (m < 0 || (L0.code[m] & 0x8000)) {
            if (!tm) { set_error("unfolded block face on the solver box boundary"); return SNAC_ERR_ARG; }
            continue;
          }
          const int tpn = (L0.code[m] >> (2 * (2 * a + 1))) & 3;
          if (tm && tpn) continue;
          if (tm || tpn || cmv_all[a][cidx] != L0.cp[a][m]) {
            set_error("inconsistent coupling between adjacent cells along axis %d", S.ax[a] + 1);
            return SNAC_ERR_ARG;
          }
        }
      }
  bool has_dir = false;
  long nact = 0;
  for (long q = 0; q < L0.ncell; q++) {
    if (L0.code[q] & 0x8000) continue;
    nact++;
    for (int f = 0; f < 6; f++) {
      const int t = (L0.code[q] >> (2 * f)) & 3;
      if (t == 2 || t == 3) has_dir = true;
    }
  }
  S.nact0 = nact;
  std::vector<int> singular(S.nsys);
  for (int s = 0; s < S.nsys; s++) singular[s] = (!S.helm && !has_dir && alpha == 0.0 && S.lambda[s] == 0.0) ? 1 : 0;
  // hierarchy
  std::vector<std::array<int, 3>> boff(d.nblocks), bext(d.nblocks);
  for (int b = 0; b < d.nblocks; b++)
    for (int a = 0; a < 3; a++) {
      const int p = S.ax[a];
      boff[b][a] = a < na ? d.hb[b].lo[p] - lo_min[p] : 0;
      bext[b][a] = a < na ? field_hi(d.hb[b], field, p) - d.hb[b].lo[p] + 1 : 1;
    }
  while ((int)B.L.size() < MG_MAXLEV) {
    const HLevel &F = B.L.back();
    if (F.ncell <= MG_DENSE_MAX) break;
    // eligible axes: every block keeps an even offset and extent, periodic rings stay even (or 1);
    // among them halve only the strongly coupled ones (smallest spacing within a factor 2), as PFMG does
    double hmin[3] = {1e300, 1e300, 1e300}, hall = 1e300;
    bool elig[3] = {false, false, false};
    for (int a = 0; a < na; a++) {
      if (F.n[a] < 2 || F.n[a] % 2) continue;
      bool ok = true;
      for (int b = 0; b < d.nblocks; b++)
        if (boff[b][a] % 2 || bext[b][a] % 2) ok = false;
      if (S.periodic[a] && (F.n[a] / 2) % 2 && F.n[a] / 2 != 1) ok = false;
      if (!ok) continue;
      elig[a] = true;
      for (int q = 0; q < F.n[a]; q++) hmin[a] = std::min(hmin[a], F.W[a][q]);
      hall = std::min(hall, hmin[a]);
    }
    int co[3] = {0, 0, 0}, any = 0;
    for (int a = 0; a < na; a++)
      if (elig[a] && hmin[a] <= 2.0 * hall) { co[a] = 1; any = 1; }
    if (!any) break;
    HLevel C;
    for (int a = 0; a < 3; a++) { C.n[a] = co[a] ? F.n[a] / 2 : F.n[a]; C.coarsened[a] = co[a]; }
    B.alloc_level(C);
    for (int a = 0; a < 3; a++)
      for (int q = 0; q < C.n[a]; q++) C.W[a][q] = co[a] ? F.W[a][2 * q] + F.W[a][2 * q + 1] : F.W[a][q];
    for (int k = 0; k < C.n[2]; k++)
      for (int j = 0; j < C.n[1]; j++)
        for (int i = 0; i < C.n[0]; i++) {
          const long cidx = i + (long)C.n[0] * (j + (long)C.n[1] * k);
          const int f0[3] = {co[0] ? 2 * i : i, co[1] ? 2 * j : j, co[2] ? 2 * k : k};
          const long fc = f0[0] + (long)F.n[0] * (f0[1] + (long)F.n[1] * f0[2]);
          unsigned short code = F.code[fc];
          if (!(code & 0x8000)) {
            for (int a = 0; a < 3; a++) {
              if (!co[a]) continue;
              int f1[3] = {f0[0], f0[1], f0[2]};
              f1[a] += 1;
              const long fc1 = f1[0] + (long)F.n[0] * (f1[1] + (long)F.n[1] * f1[2]);
              const int tp = (F.code[fc1] >> (2 * (2 * a + 1))) & 3;
              code = (unsigned short)((code & ~(3u << (2 * (2 * a + 1)))) | (tp << (2 * (2 * a + 1))));
            }
          }
          C.code[cidx] = code;
        }
    B.coarse_operator(C, alpha);
    for (int b = 0; b < d.nblocks; b++)
      for (int a = 0; a < 3; a++)
        if (co[a]) { boff[b][a] /= 2; bext[b][a] /= 2; }
    B.L.push_back(std::move(C));
  }
  HLevel &Lc = B.L.back();
  // Helmholtz problems: the dense inverse would depend on the shift; their coarsest level is
  // diagonally dominant and is smoothed instead
  if (Lc.ncell <= MG_DENSE_MAX && !S.helm) {
    Lc.dinv.assign((size_t)Lc.ncell * Lc.ncell * S.nsys, 0.0);
    for (int s = 0; s < S.nsys; s++)
      if (!B.dense(Lc, s, singular[s] != 0, Lc.dinv.data() + (size_t)Lc.ncell * Lc.ncell * s)) {
        set_error("coarsest operator of system %d is not definite", s);
        return SNAC_ERR_ARG;
      }
  }
  S.host_levels = (int)B.L.size();
  S.host_coarse_cells = B.L.back().ncell;
  // launch limits of the level kernels: 32-bit cell index within a system, grid.y over rows / 8,
  // grid.z over the systems (plane mode) or the k planes (3-D mode)
  if (L0.ncell > 0x7fffffffL || (L0.n[1] + 7) / 8 > 65535 || (S.mode3d ? L0.n[2] : S.nsys) > 65535) {
    set_error("solver box of %d x %d x %d cells (%d systems) exceeds the kernel launch limits", L0.n[0], L0.n[1],
              L0.n[2], S.nsys);
    return SNAC_ERR_UNSUPPORTED;
  }
  if (!upload) return SNAC_OK;
  // upload
  MgProblem &P = S.P;
  P.mode3d = S.mode3d;
  for (int a = 0; a < 3; a++) P.periodic[a] = S.periodic[a];
  P.nsys = S.nsys;
  P.nlev = (int)B.L.size();
  P.nu = d.opt.nu > 0 ? d.opt.nu : 2;
  // levels from 2 down: one sweep per side in plane mode (the tiled levels 0 and 1 keep nu; on the
  // channel this halves the one-CTA coarse V-cycle at the same refinement-step count), nu in 3-D mode
  P.lnu = o.mg_lnu > 0 ? o.mg_lnu : 2;
  P.nu_coarse = d.opt.nu_coarse > 0 ? d.opt.nu_coarse : (S.mode3d ? P.nu : 1);
  P.tile_shape = o.mg_tile >= 1 && o.mg_tile <= 6 ? o.mg_tile : 0;
  P.tile_inv = o.mg_inv == 1 ? 1 : 0;
  P.tile_restrict = o.mg_restrict == -1 ? 0 : 1;
  P.waves = o.mg_waves > 0 ? o.mg_waves : 2;
  P.red_batch = o.mg_red_batch == -1 ? 0 : 1;
  auto up = [&](const void *src, size_t bytes) -> void * {
    void *p = S.alloc(bytes ? bytes : 8);
    if (p && bytes) cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice);
    return p;
  };
  auto upf = [&](const std::vector<double> &v) -> float * {
    std::vector<float> f(v.begin(), v.end());
    return (float *)up(f.data(), f.size() * sizeof(float));
  };
  // 3-D mode: factor every level's couplings into 1-D face tables, cp[a](c) = Ca[a][q_a] * W_b * W_c over the
  // unfolded faces (a tensor-product grid with per-axis spacings makes them so); checked face by face, else
  // the FP32 kernels keep reading the per-cell couplings
  std::vector<std::vector<double>> fac[MG_MAXLEV][3];
  P.sep = S.mode3d ? 1 : 0;
  for (int l = 0; l < (int)B.L.size() && P.sep; l++) {
    const HLevel &h = B.L[l];
    for (int a = 0; a < 3; a++) {
      fac[l][a].assign(1, std::vector<double>(h.n[a], 0.0));
      std::vector<double> &F = fac[l][a][0];
      for (int k = 0; k < h.n[2] && P.sep; k++)
        for (int j = 0; j < h.n[1] && P.sep; j++)
          for (int i = 0; i < h.n[0]; i++) {
            const long c = i + (long)h.n[0] * (j + (long)h.n[1] * k);
            if (h.code[c] & 0x8000) continue;
            if ((h.code[c] >> (2 * (2 * a + 1))) & 3) continue;  // folded +a face
            const double cpv = h.cp[a][c];
            if (cpv == 0.0) continue;  // one-cell periodic axis
            const int idx[3] = {i, j, k};
            double wt = 1.0;
            for (int b = 0; b < 3; b++)
              if (b != a) wt *= h.W[b][idx[b]];
            const double v = cpv / wt;
            double &f = F[idx[a]];
            if (f == 0.0) f = v;
            else if (std::fabs(f - v) > 1e-12 * std::fabs(v)) { P.sep = 0; break; }
          }
    }
  }
  for (int l = 0; l < P.nlev; l++) {
    const HLevel &h = B.L[l];
    MgLevelD &D = P.L[l];
    for (int a = 0; a < 3; a++) { D.n[a] = h.n[a]; D.coarsened[a] = h.coarsened[a]; }
    for (int a = 0; a < 3; a++) D.caf[a] = P.sep ? upf(fac[l][a][0]) : nullptr;
    D.ncell = h.ncell;
    D.code = (const unsigned short *)up(h.code.data(), h.code.size() * sizeof(unsigned short));
    D.cc = (const double *)up(h.cc.data(), h.cc.size() * sizeof(double));
    D.ccf = upf(h.cc);
    for (int a = 0; a < 3; a++) {
      D.cp[a] = (const double *)up(h.cp[a].data(), h.cp[a].size() * sizeof(double));
      D.cpf[a] = upf(h.cp[a]);
      D.W[a] = (const double *)up(h.W[a].data(), h.W[a].size() * sizeof(double));
      D.Wf[a] = upf(h.W[a]);
    }
    {  // weight of the per-system diagonal shift: area W0 W1 (plane mode), volume W0 W1 W2 (3-D mode)
      std::vector<double> w01(h.ncell);
      for (int k = 0; k < h.n[2]; k++)
        for (int j = 0; j < h.n[1]; j++)
          for (int i = 0; i < h.n[0]; i++)
            w01[i + (size_t)h.n[0] * (j + (size_t)h.n[1] * k)] =
                S.mode3d ? h.W[0][i] * h.W[1][j] * h.W[2][k] : h.W[0][i] * h.W[1][j];
      D.w01 = (const double *)up(w01.data(), w01.size() * sizeof(double));
      D.w01f = upf(w01);
    }
    const size_t nv = (size_t)h.ncell * S.nsys;
    D.x = (double *)S.alloc(nv * sizeof(double));
    D.b = (double *)S.alloc(nv * sizeof(double));
    D.xf = (float *)S.alloc(nv * sizeof(float));
    D.bf = (float *)S.alloc(nv * sizeof(float));
    if (!S.mode3d && l + 1 < P.nlev) {
      D.xp = (double *)S.alloc(nv * sizeof(double));
      D.xpf = (float *)S.alloc(nv * sizeof(float));
      if (!D.xp || !D.xpf) { set_error("device allocation failed for multigrid level %d", l); return SNAC_ERR_NOMEM; }
    }
    if (!h.dinv.empty()) {
      D.dinv = (const double *)up(h.dinv.data(), h.dinv.size() * sizeof(double));
      D.dinvf = upf(h.dinv);
    }
    if (!D.code || !D.cc || !D.x || !D.xf) { set_error("device allocation failed for multigrid level %d", l); return SNAC_ERR_NOMEM; }
  }
  // fused kernels: tiled plane smoother and a one-CTA coarse tail where its levels fit in shared memory
  {
    // bit mask: 1 tiled smoother FP32, 2 coarse tail FP32, 4 tiled FP64, 8 coarse tail FP64.  Default 11: the
    // tile's redundant halo updates cost more than they save where FP64 arithmetic bounds.
    P.fused = o.mg_fuse == -1 ? 0 : (o.mg_fuse > 0 ? o.mg_fuse & 15 : 11);
    // the finest level the one-CTA coarse tail may start at: the one asked for, or by default the finest that
    // fits (3-D mode, and FP32 plane systems with the tiled smoother: and has at most MG_COARSE3D_CELLS cells)
    const int lmin = std::max(0, o.mg_cta_level);
    for (int prec = 0; prec < 2; prec++) {
      P.cta_level[prec] = P.nlev;
      for (int l = lmin; l < P.nlev; l++) {
        size_t bytes;
        if (S.mode3d) bytes = prec ? coarse3d_smem_bytes<double>(P, l) : coarse3d_smem_bytes<float>(P, l);
        else bytes = prec ? coarse_smem_bytes<double>(P, l) : coarse_smem_bytes<float>(P, l);
        // by default the one-CTA cycle takes no level of more than MG_COARSE3D_CELLS cells where that level has
        // a kernel that spreads over the GPU: always in 3-D mode, and for the FP32 plane systems where the tiled
        // smoother takes the level (channel 256 x 144: from the 2,304-cell level 16.52 ms per step, from the
        // 9,216-cell one 16.66 ms)
        const bool spread = S.mode3d || (prec == 0 && (P.fused & 1) && tile2d_geometry_ok(P, l));
        if (spread && o.mg_cta_level <= 0 && P.L[l].ncell > MG_COARSE3D_CELLS) continue;
        if (bytes <= (S.mode3d ? MG_COARSE3D_SMEM_MAX : MG_COARSE_SMEM_MAX)) { P.cta_level[prec] = l; break; }
      }
    }
  }
  P.shift = (const double *)up(S.lambda.data(), S.lambda.size() * sizeof(double));
  P.shiftf = upf(S.lambda);
  P.singular = (const int *)up(singular.data(), singular.size() * sizeof(int));
  P.any_singular = 0;
  for (int v : singular) P.any_singular |= v;
  P.nact0 = nact;
  {
    std::vector<int> list;
    for (int q = 0; q < S.nsys; q++)
      if (singular[q]) list.push_back(q);
    P.nsing = (int)list.size();
    P.sing_list = list.empty() ? nullptr : (const int *)up(list.data(), list.size() * sizeof(int));
  }
  {
    int dev = 0;
    SNAC_CUDA(cudaGetDevice(&dev));
    SNAC_CUDA(cudaDeviceGetAttribute(&P.nsm, cudaDevAttrMultiProcessorCount, dev));
  }
  if (!S.mode3d) {  // smoothers: 1 / diagonal per system and cell, made once
    double *tabs[MG_MAXLEV];
    float *tabsf[MG_MAXLEV];
    for (int l = 0; l < P.nlev; l++) {
      tabs[l] = (double *)S.alloc((size_t)P.L[l].ncell * S.nsys * sizeof(double));
      tabsf[l] = (float *)S.alloc((size_t)P.L[l].ncell * S.nsys * sizeof(float));
      if (!tabs[l] || !tabsf[l]) { set_error("device allocation failed for the diagonal tables"); return SNAC_ERR_NOMEM; }
    }
    SNAC_TRY(plane_make_invd(P, tabs, tabsf, 0));
    SNAC_CUDA(cudaStreamSynchronize(0));
    for (int l = 0; l < P.nlev; l++) { S.invd_tab[l] = tabs[l]; S.invd_tabf[l] = tabsf[l]; }
    if (S.helm) {  // the shift of each wavenumber is lambda_k + alphai, set per solve
      S.d_lambda = (double *)up(S.lambda.data(), S.lambda.size() * sizeof(double));
      if (!S.d_lambda) { set_error("device allocation failed (eigenvalues)"); return SNAC_ERR_NOMEM; }
    }
  }
  S.ncell0 = L0.ncell;
  const size_t nv0 = (size_t)L0.ncell * S.nsys;
  const int stride = mg_partial_stride(P);
  S.box_b = (double *)S.alloc(nv0 * sizeof(double));
  S.box_x = (double *)S.alloc(nv0 * sizeof(double));
  S.r64 = (double *)S.alloc(nv0 * sizeof(double));
  S.box_e32 = (float *)S.alloc(nv0 * sizeof(float));
  S.active_outer = (int *)S.alloc(S.nsys * sizeof(int));
  S.sc_outer = (SysScal *)S.alloc(S.nsys * sizeof(SysScal));
  for (CgWork *W : {&S.W64, &S.W32}) {
    const size_t es = W == &S.W64 ? sizeof(double) : sizeof(float);
    W->r = S.alloc(nv0 * es);
    W->z = S.alloc(nv0 * es);
    W->p = S.alloc(nv0 * es);
    W->p2 = W == &S.W32 ? S.alloc(nv0 * es) : nullptr;
    W->q = S.alloc(nv0 * es);
    W->stride = stride;
    for (double **pp : {&W->part0, &W->part1, &W->part2, &W->part3, &W->part4})
      *pp = (double *)S.alloc((size_t)stride * S.nsys * sizeof(double));
    W->sc = (SysScal *)S.alloc(S.nsys * sizeof(SysScal));
    W->active = (int *)S.alloc(S.nsys * sizeof(int));
    W->d_count = (int *)S.alloc(2 * sizeof(int));
    SNAC_CUDA(cudaMallocHost(&W->h_count, 2 * sizeof(int)));
    if (!W->r || !W->z || !W->p || !W->q || (W == &S.W32 && !W->p2) || !W->part0 || !W->part1 || !W->part2 || !W->part3 || !W->part4 || !W->sc ||
        !W->active || !W->d_count) {
      set_error("device allocation failed for Krylov vectors");
      return SNAC_ERR_NOMEM;
    }
  }
  if (S.helm) {
    std::vector<std::vector<double>> planes[3];
    for (int a = 0; a < 3; a++) planes[a].resize(d.nblocks);
    for (int b = 0; b < d.nblocks; b++) {
      std::vector<double> r[3];
      init_bc_rhs_field(d.hb[b], field, d.periods, c.fft_axis, r);
      for (int a = 0; a < 3; a++) planes[a][b] = std::move(r[a]);
    }
    SNAC_TRY(helm_upload_tables(d, S, planes));
  }
  return SNAC_OK;
}

// FP64: PCG with FP64 V-cycles.  Mixed: FP64 residual / FP32 PCG with FP32 V-cycles / FP64 update.
// one refinement step of the mixed path: scaled FP32 residual, FP32 PCG with FP32 V-cycles, FP64 update.
// It has no host synchronisation, so with use_graph it is captured once per solver as a CUDA graph and
// replayed (every pointer and launch shape is fixed for the solver's lifetime).
static int refine_step_body(PoissonSolver &S, const CgWork &Wr, cudaStream_t st) {
  MgProblem &P = S.P;
  SNAC_TRY(mg_ir_down(P, Wr, S.W32, S.r64, (float *)S.W32.r, S.box_e32, S.inner_tol, S.adapt_inner ? S.tol : 0.0, st));
  int it1 = 0;
  SNAC_TRY(mg_pcg<float>(P, S.W32, S.box_e32, S.inner_iters, S.inner_tol, true, false, &it1, st));
  SNAC_TRY(mg_ir_up(P, Wr, S.box_e32, S.box_x, st));
  return SNAC_OK;
}

static int refine_step(PoissonSolver &S, const CgWork &Wr, cudaStream_t st) {
  if (!S.use_graph || prof_active() || trace_on()) return refine_step_body(S, Wr, st);
  if (!S.inner_exec) {
    long long c0 = 0, c1 = 0;
    snac_launch_count(&c0);
    SNAC_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
    const int rc = refine_step_body(S, Wr, st);
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(st, &g);
    snac_launch_count(&c1);
    add_launches(c0 - c1);  // captured, not run
    if (rc != SNAC_OK) { if (g) cudaGraphDestroy(g); return rc; }
    if (ce != cudaSuccess) { set_error("stream capture of the refinement step failed: %s", cudaGetErrorString(ce)); return SNAC_ERR_CUDA; }
    const cudaError_t ie = cudaGraphInstantiate(&S.inner_exec, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) { S.inner_exec = nullptr; set_error("graph instantiation failed: %s", cudaGetErrorString(ie)); return SNAC_ERR_CUDA; }
    S.inner_nodes = c1 - c0;
  }
  SNAC_CUDA(cudaGraphLaunch(S.inner_exec, st));
  add_launches(S.inner_nodes);
  return SNAC_OK;
}

static int solve_box(PoissonSolver &S, cudaStream_t st, int *iters_out, double *res_out) {
  MgProblem &P = S.P;
  SNAC_TRY(mg_project_singular(P, S.W64, S.box_b, st));
  trace("solve: projection of singular systems", st);
  std::vector<SysScal> sc(P.nsys);
  double worst = 0.0;
  if (S.precision == 0) {
    CgWork &W = S.W64;
    int iters = 0;
    SNAC_TRY(mg_set_active(P.nsys, W.active, nullptr, st));
    SNAC_TRY(mg_residual<double>(P, W, S.box_x, S.box_b, (double *)W.r, S.tol, 1, 0, 0, st));
    SNAC_TRY(mg_restart_bad_guess(P, W, S.box_x, S.box_b, (double *)W.r, st));
    // singular systems: r = b - A x0 keeps its zero mean only up to rounding; CG cannot remove a
    // null-space part, so it is projected out
    SNAC_TRY(mg_project_singular(P, W, (double *)W.r, st));
    SNAC_CUDA(cudaMemcpyAsync(W.h_count, W.d_count, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
    SNAC_CUDA(cudaStreamSynchronize(st));
    if (W.h_count[1]) SNAC_TRY(mg_zero_rhs_systems(P, W, S.box_x, st));
    trace("pcg64: initial residual", st);
    if (W.h_count[0]) SNAC_TRY(mg_pcg<double>(P, W, S.box_x, S.maxiter, S.tol, false, true, &iters, st));
    SNAC_CUDA(cudaMemcpyAsync(sc.data(), W.sc, P.nsys * sizeof(SysScal), cudaMemcpyDeviceToHost, st));
    SNAC_CUDA(cudaStreamSynchronize(st));
    for (auto &v : sc) worst = std::max(worst, v.rel);
    *iters_out = iters;
    *res_out = worst;
    return (worst > S.tol && iters >= S.maxiter) ? SNAC_ERR_NOT_CONVERGED : SNAC_OK;
  }
  // mixed precision: iterative refinement in FP64 around FP32 Krylov solves (zero initial guess).  The
  // first `spec` refinement steps run without a host round trip (converged systems are skipped on the
  // device by their active flags); the counts of every step are read after step `spec`.
  int outer = 0, needed = -1, polish = 0;
  CgWork Wr = S.W64;  // residual-only use of the FP64 work area
  Wr.active = S.active_outer;
  Wr.sc = S.sc_outer;
  if (!S.d_ocount) {
    S.d_ocount = (int *)S.alloc(2 * PoissonSolver::SPEC_MAX * sizeof(int));
    SNAC_CUDA(cudaMallocHost(&S.h_ocount, 2 * PoissonSolver::SPEC_MAX * sizeof(int)));
    if (!S.d_ocount) { set_error("device allocation failed (refinement counts)"); return SNAC_ERR_NOMEM; }
  }
  const int spec = std::min(S.spec_outer, PoissonSolver::SPEC_MAX - 1);
  SNAC_TRY(mg_set_active(P.nsys, S.active_outer, nullptr, st));
  for (outer = 0; outer < S.maxiter; outer++) {
    CgWork Wo = Wr;
    if (outer <= spec) Wo.d_count = S.d_ocount + 2 * outer;
    // r64 = b - A x64 with norms, convergence and the scale of the FP32 residual
    SNAC_TRY(mg_residual<double>(P, Wo, S.box_x, S.box_b, S.r64, S.tol, outer == 0 ? 1 : 0, 1, S.nact0, st));
    SNAC_TRY(mg_project_singular(P, Wo, S.r64, st));  // as in the FP64 path: the correction equation stays consistent
    if (outer < spec) {
      if (outer == 0) {
        SNAC_TRY(mg_zero_rhs_systems(P, Wo, S.box_x, st));  // a no-op for systems with a right-hand side
        SNAC_TRY(mg_restart_bad_guess(P, Wo, S.box_x, S.box_b, S.r64, st));
      }
      SNAC_TRY(refine_step(S, Wr, st));
      continue;
    }
    int cnt[2];
    if (outer == spec) {
      SNAC_CUDA(cudaMemcpyAsync(S.h_ocount, S.d_ocount, 2 * (spec + 1) * sizeof(int), cudaMemcpyDeviceToHost, st));
      SNAC_CUDA(cudaStreamSynchronize(st));
      for (int o = 0; o <= spec && needed < 0; o++)
        if (S.h_ocount[2 * o] == 0) needed = o;
      cnt[0] = S.h_ocount[2 * spec];
      cnt[1] = S.h_ocount[2 * spec + 1];
    } else {
      SNAC_CUDA(cudaMemcpyAsync(Wo.h_count, Wo.d_count, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
      SNAC_CUDA(cudaStreamSynchronize(st));
      cnt[0] = Wo.h_count[0];
      cnt[1] = Wo.h_count[1];
    }
    if (outer == 0 && cnt[1]) SNAC_TRY(mg_zero_rhs_systems(P, Wo, S.box_x, st));
    if (outer == 0) SNAC_TRY(mg_restart_bad_guess(P, Wo, S.box_x, S.box_b, S.r64, st));
    if (cnt[0] == 0) break;
    if (S.refine_steps > 0 && outer >= S.refine_steps) {
      // Each FP32 refinement step gains about seven digits at best (the FP32 floor); after refine_steps of
      // them only a few systems are still above the tolerance -- typically the singular zero-wavenumber one,
      // the worst conditioned, whose steps gain fewer.  Option: FP64 PCG iterations from the current iterate,
      // on those systems only, finish them (the same stopping test as the plain FP64 path) instead of another
      // FP32 step.  On the channel the FP32 step is the faster (its launches replay as a graph, these do not).
      CgWork Wf = S.W64;
      Wf.r = S.r64;
      Wf.active = S.active_outer;
      Wf.sc = S.sc_outer;
      Wf.d_count = Wo.d_count;
      Wf.h_count = outer <= spec ? S.h_ocount + 2 * outer : Wo.h_count;
      SNAC_TRY(mg_restart_krylov(P, Wf, st));
      int pit = 0;
      SNAC_TRY(mg_pcg<double>(P, Wf, S.box_x, S.maxiter, S.tol, false, true, &pit, st));
      polish = pit;
      outer++;
      break;
    }
    SNAC_TRY(refine_step(S, Wr, st));
  }
  if (needed < 0) needed = outer;
  S.spec_outer = std::min(needed, S.refine_steps > 0 ? S.refine_steps : needed);
  SNAC_CUDA(cudaMemcpyAsync(sc.data(), S.sc_outer, P.nsys * sizeof(SysScal), cudaMemcpyDeviceToHost, st));
  SNAC_CUDA(cudaStreamSynchronize(st));
  for (auto &v : sc) worst = std::max(worst, v.rel);
  *iters_out = needed;
  S.last_polish = polish;
  *res_out = worst;
  return (worst > S.tol && (outer >= S.maxiter || polish >= S.maxiter)) ? SNAC_ERR_NOT_CONVERGED : SNAC_OK;
}

// solve_impdiff_field_3d (solve_helmholtz.f90:109-138): right-hand side alphai V phi + BC planes, the
// shift alphai on the diagonal, the solve warm-started from the previous solution, the field overwritten
// solve_impdiff_field_fft (solve_helmholtz.f90:32-102) with a transform axis: the same right-hand side
// weighted by the in-plane area, the forward transform of the field, per-wavenumber solves with the shift
// lambda_k + alphai, the backward transform and normfft.
int solver_solve_helmholtz(Domain &d, PoissonSolver &S, double alphai) {
  cudaStream_t st = d.st;
  if (!S.helm) { set_error("not a Helmholtz solver"); return SNAC_ERR_STATE; }
  SNAC_TRY(helm_rhs(d, S, alphai, st));
  SNAC_TRY(helm_shift(S, alphai, st));
  if (S.fft_axis) SNAC_TRY(fft_forward_to_box(d, S, st));
  else SNAC_TRY(helm_io(d, S, S.box_b, 1, st));
  int it = 0;
  double res = 0.0;
  const int rc = solve_box(S, st, &it, &res);
  if (rc != SNAC_OK && rc != SNAC_ERR_NOT_CONVERGED) return rc;
  if (S.fft_axis) SNAC_TRY(fft_backward_from_box(d, S, st));
  else SNAC_TRY(helm_io(d, S, S.box_x, 0, st));
  S.last_iters = it;
  S.last_res = res;
  if (rc == SNAC_ERR_NOT_CONVERGED)
    set_error("Helmholtz solve stopped at maxiter=%d with relative residual %.3e > tol %.3e", S.maxiter, res, S.tol);
  return rc;
}

// main.f90:1004-1022: transform (or gather), solve every system warm-started from po, back-transform + normfft
int solver_solve_pressure(Domain &d, PoissonSolver &S) {
  cudaStream_t st = d.st;
  trace("solve: start", st);
  prof_begin(KID_SOLVE, st);
  if (S.fft_axis) SNAC_TRY(fft_forward_to_box(d, S, st));
  else SNAC_TRY(box_gather(d, S, st));
  trace("solve: forward transform / gather", st);
  if (d.guess) SNAC_TRY(guess_before(d, S, st));
  int it = 0;
  double res = 0.0;
  const int rc = solve_box(S, st, &it, &res);
  if (d.guess && (rc == SNAC_OK || rc == SNAC_ERR_NOT_CONVERGED)) SNAC_TRY(guess_after(d, S, st));
  trace("solve: box solve", st);
  if (rc != SNAC_OK && rc != SNAC_ERR_NOT_CONVERGED) return rc;
  if (S.fft_axis) SNAC_TRY(fft_backward_from_box(d, S, st));
  else SNAC_TRY(box_scatter(d, S, st));
  prof_end(KID_SOLVE, st);
  trace("solve: backward transform / scatter", st);
  S.last_iters = it;
  S.last_res = res;
  if (rc == SNAC_ERR_NOT_CONVERGED)
    set_error("pressure solve stopped at maxiter=%d with relative residual %.3e > tol %.3e", S.maxiter, res, S.tol);
  return rc;
}

}  // namespace snac
