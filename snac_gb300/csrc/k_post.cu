// k_post.cu -- post.f90:8-156 on the device: vorticity, strain rate S_ij S_ij, rotation rate W_ij W_ij and
// the Q criterion of one block at the cell centres, with the reference's expressions term by term (divisions
// by the centre spacings, the four-point averages of the cross derivatives).  One thread per cell; inputs
// halo'd (0:n+1), outputs interior.  These run at the output cadence, so they keep the reference's divisions
// instead of reciprocal tables.
#include "snac_host.h"

namespace snac {

namespace {

struct PostArgs {
  int n[3];
  const double *dxc, *dyc, *dzc, *dxf, *dyf, *dzf;  // n + 2 entries from lo - 1
  const double *ux, *uy, *uz;                       // halo'd
};

__device__ __forceinline__ double sq(double a) { return a * a; }

// the cross terms of the strain (sgn = +1) or rotation (sgn = -1) rate at cell (i, j, k), 1-based
__device__ __forceinline__ void rate_terms(const PostArgs &A, int i, int j, int k, double sgn, double &a12,
                                           double &a13, double &a23) {
  const int n0 = A.n[0] + 2, n1 = A.n[1] + 2;
  auto H = [&](const double *a, int ii, int jj, int kk) { return a[ii + (long)n0 * (jj + (long)n1 * kk)]; };
  const double *ux = A.ux, *uy = A.uy, *uz = A.uz, *dxc = A.dxc, *dyc = A.dyc, *dzc = A.dzc;
  a12 = .25 * (sq((H(ux, i, j + 1, k) - H(ux, i, j, k)) / dyc[j] + sgn * ((H(uy, i + 1, j, k) - H(uy, i, j, k)) / dxc[i])) +
               sq((H(ux, i, j, k) - H(ux, i, j - 1, k)) / dyc[j - 1] + sgn * ((H(uy, i + 1, j - 1, k) - H(uy, i, j - 1, k)) / dxc[i])) +
               sq((H(ux, i - 1, j + 1, k) - H(ux, i - 1, j, k)) / dyc[j] + sgn * ((H(uy, i, j, k) - H(uy, i - 1, j, k)) / dxc[i - 1])) +
               sq((H(ux, i - 1, j, k) - H(ux, i - 1, j - 1, k)) / dyc[j - 1] + sgn * ((H(uy, i, j - 1, k) - H(uy, i - 1, j - 1, k)) / dxc[i - 1]))) * .25;
  a13 = .25 * (sq((H(ux, i, j, k + 1) - H(ux, i, j, k)) / dzc[k] + sgn * ((H(uz, i + 1, j, k) - H(uz, i, j, k)) / dxc[i])) +
               sq((H(ux, i, j, k) - H(ux, i, j, k - 1)) / dzc[k - 1] + sgn * ((H(uz, i + 1, j, k - 1) - H(uz, i, j, k - 1)) / dxc[i])) +
               sq((H(ux, i - 1, j, k + 1) - H(ux, i - 1, j, k)) / dzc[k] + sgn * ((H(uz, i, j, k) - H(uz, i - 1, j, k)) / dxc[i - 1])) +
               sq((H(ux, i - 1, j, k) - H(ux, i - 1, j, k - 1)) / dzc[k - 1] + sgn * ((H(uz, i, j, k - 1) - H(uz, i - 1, j, k - 1)) / dxc[i - 1]))) * .25;
  a23 = .25 * (sq((H(uy, i, j, k + 1) - H(uy, i, j, k)) / dzc[k] + sgn * ((H(uz, i, j + 1, k) - H(uz, i, j, k)) / dyc[j])) +
               sq((H(uy, i, j, k) - H(uy, i, j, k - 1)) / dzc[k - 1] + sgn * ((H(uz, i, j + 1, k - 1) - H(uz, i, j, k - 1)) / dyc[j])) +
               sq((H(uy, i, j - 1, k + 1) - H(uy, i, j - 1, k)) / dzc[k] + sgn * ((H(uz, i, j, k) - H(uz, i, j - 1, k)) / dyc[j - 1])) +
               sq((H(uy, i, j - 1, k) - H(uy, i, j - 1, k - 1)) / dzc[k - 1] + sgn * ((H(uz, i, j, k - 1) - H(uz, i, j - 1, k - 1)) / dyc[j - 1]))) * .25;
}

__device__ __forceinline__ double strain_at(const PostArgs &A, int i, int j, int k) {
  const int n0 = A.n[0] + 2, n1 = A.n[1] + 2;
  auto H = [&](const double *a, int ii, int jj, int kk) { return a[ii + (long)n0 * (jj + (long)n1 * kk)]; };
  double a12, a13, a23;
  rate_terms(A, i, j, k, 1.0, a12, a13, a23);
  const double s11 = sq((H(A.ux, i, j, k) - H(A.ux, i - 1, j, k)) / A.dxf[i]);
  const double s22 = sq((H(A.uy, i, j, k) - H(A.uy, i, j - 1, k)) / A.dyf[j]);
  const double s33 = sq((H(A.uz, i, j, k) - H(A.uz, i, j, k - 1)) / A.dzf[k]);
  return s11 + s22 + s33 + 2 * (a12 + a13 + a23);
}

__device__ __forceinline__ double rotation_at(const PostArgs &A, int i, int j, int k) {
  double a12, a13, a23;
  rate_terms(A, i, j, k, -1.0, a12, a13, a23);
  return 2.0 * (a12 + a13 + a23);
}

// what: 0 vorticity (o0, o1, o2), 1 strain rate (o0), 2 rotation rate (o0), 3 Q criterion from the velocities (o0)
__global__ void __launch_bounds__(256) k_post(PostArgs A, int what, double *o0, double *o1, double *o2) {
  const int i = blockIdx.x * 32 + threadIdx.x + 1, j = blockIdx.y * 8 + threadIdx.y + 1, k = blockIdx.z + 1;
  if (i > A.n[0] || j > A.n[1]) return;
  const long q = (i - 1) + (long)A.n[0] * ((j - 1) + (long)A.n[1] * (k - 1));
  if (what == 1) { o0[q] = strain_at(A, i, j, k); return; }
  if (what == 2) { o0[q] = rotation_at(A, i, j, k); return; }
  if (what == 3) { o0[q] = .5 * (rotation_at(A, i, j, k) - strain_at(A, i, j, k)); return; }
  const int n0 = A.n[0] + 2, n1 = A.n[1] + 2;
  auto H = [&](const double *a, int ii, int jj, int kk) { return a[ii + (long)n0 * (jj + (long)n1 * kk)]; };
  const double *ux = A.ux, *uy = A.uy, *uz = A.uz, *dxc = A.dxc, *dyc = A.dyc, *dzc = A.dzc;
  o0[q] = 0.25 * ((H(uz, i, j + 1, k) - H(uz, i, j, k)) / dyc[j] - (H(uy, i, j, k + 1) - H(uy, i, j, k)) / dzc[k] +
                  (H(uz, i, j + 1, k - 1) - H(uz, i, j, k - 1)) / dyc[j] - (H(uy, i, j, k) - H(uy, i, j, k - 1)) / dzc[k - 1] +
                  (H(uz, i, j, k) - H(uz, i, j - 1, k)) / dyc[j - 1] - (H(uy, i, j - 1, k + 1) - H(uy, i, j - 1, k)) / dzc[k] +
                  (H(uz, i, j, k - 1) - H(uz, i, j - 1, k - 1)) / dyc[j - 1] - (H(uy, i, j - 1, k) - H(uy, i, j - 1, k - 1)) / dzc[k - 1]);
  o1[q] = 0.25 * ((H(ux, i, j, k + 1) - H(ux, i, j, k)) / dzc[k] - (H(uz, i + 1, j, k) - H(uz, i, j, k)) / dxc[i] +
                  (H(ux, i, j, k) - H(ux, i, j, k - 1)) / dzc[k - 1] - (H(uz, i + 1, j, k - 1) - H(uz, i, j, k - 1)) / dxc[i] +
                  (H(ux, i - 1, j, k + 1) - H(ux, i - 1, j, k)) / dzc[k] - (H(uz, i, j, k) - H(uz, i - 1, j, k)) / dxc[i - 1] +
                  (H(ux, i - 1, j, k) - H(ux, i - 1, j, k - 1)) / dzc[k - 1] - (H(uz, i, j, k - 1) - H(uz, i - 1, j, k - 1)) / dxc[i - 1]);
  o2[q] = 0.25 * ((H(uy, i + 1, j, k) - H(uy, i, j, k)) / dxc[i] - (H(ux, i, j + 1, k) - H(ux, i, j, k)) / dyc[j] +
                  (H(uy, i + 1, j - 1, k) - H(uy, i, j - 1, k)) / dxc[i] - (H(ux, i, j, k) - H(ux, i, j - 1, k)) / dyc[j - 1] +
                  (H(uy, i, j, k) - H(uy, i - 1, j, k)) / dxc[i - 1] - (H(ux, i - 1, j + 1, k) - H(ux, i - 1, j, k)) / dyc[j] +
                  (H(uy, i, j - 1, k) - H(uy, i - 1, j - 1, k)) / dxc[i - 1] - (H(ux, i - 1, j, k) - H(ux, i - 1, j - 1, k)) / dyc[j - 1]);
}

__global__ void k_q_from_rates(long m, const double *ens, const double *str, double *qcr) {
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < m) qcr[q] = .5 * (ens[q] - str[q]);
}

// the caller's host arrays on the device (registered mirrors or copies around the call)
int run_post(const int n[3], const double *dxc, const double *dyc, const double *dzc, const double *dxf,
             const double *dyf, const double *dzf, const double *ux, const double *uy, const double *uz, int what,
             double *o0, double *o1, double *o2) {
  for (int a = 0; a < 3; a++)
    if (n[a] < 1) { set_error("post-processing: n must be positive"); return SNAC_ERR_ARG; }
  if (n[2] > 65535 || (n[1] + 7) / 8 > 65535) { set_error("post-processing: block too large for one launch"); return SNAC_ERR_UNSUPPORTED; }
  const size_t halo = (size_t)(n[0] + 2) * (n[1] + 2) * (n[2] + 2) * sizeof(double);
  const size_t inner = (size_t)n[0] * n[1] * n[2] * sizeof(double);
  ArgArray X, Y, Z, Mx[6], O0, O1, O2;
  const double *m[6] = {dxc, dyc, dzc, dxf ? dxf : dxc, dyf ? dyf : dyc, dzf ? dzf : dzc};
  SNAC_TRY(X.bind(ux, halo, true, false));
  SNAC_TRY(Y.bind(uy, halo, true, false));
  SNAC_TRY(Z.bind(uz, halo, true, false));
  for (int q = 0; q < 6; q++) SNAC_TRY(Mx[q].bind(m[q], (size_t)(n[q % 3] + 2) * sizeof(double), true, false));
  SNAC_TRY(O0.bind(o0, inner, false, true));
  if (what == 0) {
    SNAC_TRY(O1.bind(o1, inner, false, true));
    SNAC_TRY(O2.bind(o2, inner, false, true));
  }
  PostArgs A;
  for (int a = 0; a < 3; a++) A.n[a] = n[a];
  A.dxc = (const double *)Mx[0].dev; A.dyc = (const double *)Mx[1].dev; A.dzc = (const double *)Mx[2].dev;
  A.dxf = (const double *)Mx[3].dev; A.dyf = (const double *)Mx[4].dev; A.dzf = (const double *)Mx[5].dev;
  A.ux = (const double *)X.dev; A.uy = (const double *)Y.dev; A.uz = (const double *)Z.dev;
  const dim3 g((unsigned)((n[0] + 31) / 32), (unsigned)((n[1] + 7) / 8), (unsigned)n[2]);
  k_post<<<g, dim3(32, 8), 0, 0>>>(A, what, (double *)O0.dev, what == 0 ? (double *)O1.dev : nullptr,
                                   what == 0 ? (double *)O2.dev : nullptr), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  SNAC_CUDA(cudaDeviceSynchronize());
  SNAC_TRY(O0.finish());
  if (what == 0) {
    SNAC_TRY(O1.finish());
    SNAC_TRY(O2.finish());
  }
  return SNAC_OK;
}

}  // namespace

}  // namespace snac

using namespace snac;

int snac_cmpt_vorticity(const int n[3], const double *dxc, const double *dyc, const double *dzc, const double *ux,
                        const double *uy, const double *uz, double *vox, double *voy, double *voz) {
  if (!n || !dxc || !dyc || !dzc || !ux || !uy || !uz || !vox || !voy || !voz) { set_error("snac_cmpt_vorticity: null argument"); return SNAC_ERR_ARG; }
  return run_post(n, dxc, dyc, dzc, nullptr, nullptr, nullptr, ux, uy, uz, 0, vox, voy, voz);
}

int snac_cmpt_strain_rate(const int n[3], const double *dxc, const double *dyc, const double *dzc, const double *dxf,
                          const double *dyf, const double *dzf, const double *ux, const double *uy, const double *uz,
                          double *str) {
  if (!n || !dxc || !dyc || !dzc || !dxf || !dyf || !dzf || !ux || !uy || !uz || !str) { set_error("snac_cmpt_strain_rate: null argument"); return SNAC_ERR_ARG; }
  return run_post(n, dxc, dyc, dzc, dxf, dyf, dzf, ux, uy, uz, 1, str, nullptr, nullptr);
}

int snac_cmpt_rotation_rate(const int n[3], const double *dxc, const double *dyc, const double *dzc, const double *ux,
                            const double *uy, const double *uz, double *ens) {
  if (!n || !dxc || !dyc || !dzc || !ux || !uy || !uz || !ens) { set_error("snac_cmpt_rotation_rate: null argument"); return SNAC_ERR_ARG; }
  return run_post(n, dxc, dyc, dzc, nullptr, nullptr, nullptr, ux, uy, uz, 2, ens, nullptr, nullptr);
}

int snac_cmpt_q_criterion(const int n[3], const double *ens, const double *str, double *qcr) {
  if (!n || !ens || !str || !qcr) { set_error("snac_cmpt_q_criterion: null argument"); return SNAC_ERR_ARG; }
  for (int a = 0; a < 3; a++)
    if (n[a] < 1) { set_error("snac_cmpt_q_criterion: n must be positive"); return SNAC_ERR_ARG; }
  const long m = (long)n[0] * n[1] * n[2];
  ArgArray E, S, Q;
  SNAC_TRY(E.bind(ens, m * sizeof(double), true, false));
  SNAC_TRY(S.bind(str, m * sizeof(double), true, false));
  SNAC_TRY(Q.bind(qcr, m * sizeof(double), false, true));
  k_q_from_rates<<<(unsigned)((m + 255) / 256), 256>>>(m, (const double *)E.dev, (const double *)S.dev, (double *)Q.dev),
      ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  SNAC_CUDA(cudaDeviceSynchronize());
  return Q.finish();
}

int snac_q_criterion(const int n[3], const double *dxc, const double *dyc, const double *dzc, const double *dxf,
                     const double *dyf, const double *dzf, const double *ux, const double *uy, const double *uz,
                     double *qcr) {
  if (!n || !dxc || !dyc || !dzc || !dxf || !dyf || !dzf || !ux || !uy || !uz || !qcr) { set_error("snac_q_criterion: null argument"); return SNAC_ERR_ARG; }
  return run_post(n, dxc, dyc, dzc, dxf, dyf, dzf, ux, uy, uz, 3, qcr, nullptr, nullptr);
}
