// api_ref.cu -- error state, host-mirror registry and the reference-signature
// entry points of the C ABI (one block per call, the caller's host arrays).
#include <cstdarg>
#include <cmath>
#include <cstring>
#include <mutex>
#include <unordered_map>

#include "snac_bound.h"
#include "snac_host.h"

namespace snac {

static thread_local std::string g_err;

void set_error(const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
}

bool trace_on() {
  static int on = -1;
  if (on < 0) {
    const char *e = getenv("SNAC_DEBUG");
    on = (e && e[0] && e[0] != '0') ? 1 : 0;
  }
  return on != 0;
}

void trace(const char *what, cudaStream_t st) {
  if (!trace_on()) return;
  cudaError_t e = cudaStreamSynchronize(st);
  fprintf(stderr, "[snac] %s: %s\n", what, cudaGetErrorString(e));
  fflush(stderr);
}

int cuda_fail(cudaError_t e, const char *what, const char *file, int line) {
  set_error("CUDA error %s (%d) in %s at %s:%d", cudaGetErrorString(e), (int)e, what, file, line);
  return SNAC_ERR_CUDA;
}

// ---------------------------------------------------------------- mirrors
struct Mirror {
  void *dev;
  size_t bytes;
};
static std::mutex g_mtx;
static std::unordered_map<const void *, Mirror> g_mirrors;

const void *mirror_of(const void *host, size_t need) {
  std::lock_guard<std::mutex> lk(g_mtx);
  auto it = g_mirrors.find(host);
  if (it == g_mirrors.end() || it->second.bytes < need) return nullptr;
  return it->second.dev;
}

// Device view of one argument array of a reference-signature call.
int ArgArray::bind(const void *h, size_t nbytes, bool in, bool out) {
  host = h;
  bytes = nbytes;
  copy_out = out;
  const void *m = mirror_of(h, nbytes);
  if (m) {
    dev = const_cast<void *>(m);
    owned = false;
    return SNAC_OK;
  }
  SNAC_CUDA(cudaMalloc(&dev, nbytes));
  owned = true;
  if (in) SNAC_CUDA(cudaMemcpy(dev, h, nbytes, cudaMemcpyHostToDevice));
  return SNAC_OK;
}
int ArgArray::finish() {
  if (owned && copy_out) SNAC_CUDA(cudaMemcpy(const_cast<void *>(host), dev, bytes, cudaMemcpyDeviceToHost));
  return SNAC_OK;
}
ArgArray::~ArgArray() {
  if (owned && dev) cudaFree(dev);
}

// AxisArr tables of one axis from the reference's dc/df arrays (n+2 entries)
std::vector<double> axis_tables(const double *dc, const double *df, int n) {
  const int m = n + 2;
  std::vector<double> t((size_t)AX_NARR * m, 0.0);
  for (int q = 0; q < m; q++) {
    const double c = dc[q], f = df[q];
    t[AX_DC * m + q] = c;
    t[AX_DF * m + q] = f;
    t[AX_RC * m + q] = 1.0 / c;
    t[AX_RF * m + q] = 1.0 / f;
    t[AX_A * m + q] = 0.25 / c;
    t[AX_E0 * m + q] = 0.25 * f / c;
    t[AX_E1 * m + q] = q + 1 < m ? 0.25 * df[q + 1] / c : 0.0;
    t[AX_SP * m + q] = q + 1 < m ? 1.0 / (c * df[q + 1]) : 0.0;
    t[AX_SM * m + q] = 1.0 / (c * f);
    t[AX_CP * m + q] = 1.0 / (f * c);
    t[AX_CM * m + q] = q > 0 ? 1.0 / (f * dc[q - 1]) : 0.0;
  }
  return t;
}

// A single block described by reference arguments, with its device table and tiles.
int OneBlock::setup(const int lo_[3], const int hi_[3], const double *dxc, const double *dxf, const double *dyc,
                    const double *dyf, const double *dzc, const double *dzf, bool halo_tiles) {
  memset(&hb, 0, sizeof(hb));
  for (int a = 0; a < 3; a++) {
    hb.lo[a] = lo_[a];
    hb.n[a] = hi_[a] - lo_[a] + 1;
    if (hb.n[a] < 1) { set_error("hi < lo along axis %d", a + 1); return SNAC_ERR_ARG; }
  }
  const double *dc[3] = {dxc, dyc, dzc}, *df[3] = {dxf, dyf, dzf};
  std::vector<double> all;
  size_t off[3];
  for (int a = 0; a < 3; a++) {
    off[a] = all.size();
    if (dc[a] && df[a]) {
      auto t = axis_tables(dc[a], df[a], hb.n[a]);
      all.insert(all.end(), t.begin(), t.end());
    } else {
      std::vector<double> one(hb.n[a] + 2, 1.0);
      auto t = axis_tables(one.data(), one.data(), hb.n[a]);
      all.insert(all.end(), t.begin(), t.end());
    }
  }
  SNAC_CUDA(cudaMalloc(&dax, all.size() * sizeof(double)));
  SNAC_CUDA(cudaMemcpy(dax, all.data(), all.size() * sizeof(double), cudaMemcpyHostToDevice));
  for (int a = 0; a < 3; a++) hb.ax[a] = dax + off[a];
  hb.bchk = bounds_flag();
  std::vector<std::array<int, 3>> sz{{hb.n[0] + (halo_tiles ? 2 : 0), hb.n[1] + (halo_tiles ? 2 : 0),
                                      hb.n[2] + (halo_tiles ? 2 : 0)}};
  auto tl = make_tiles(sz, TX, TY, TZ);
  ntiles = (int)tl.size();
  SNAC_CUDA(cudaMalloc(&dtiles, tl.size() * sizeof(Tile)));
  SNAC_CUDA(cudaMemcpy(dtiles, tl.data(), tl.size() * sizeof(Tile), cudaMemcpyHostToDevice));
  return SNAC_OK;
}
int OneBlock::upload() {
  if (!dblk) SNAC_CUDA(cudaMalloc(&dblk, sizeof(DBlock)));
  SNAC_CUDA(cudaMemcpy(dblk, &hb, sizeof(DBlock), cudaMemcpyHostToDevice));
  return SNAC_OK;
}
int OneBlock::scratch(size_t bytes, double **p) {
  void *q;
  SNAC_CUDA(cudaMalloc(&q, bytes));
  SNAC_CUDA(cudaMemset(q, 0, bytes));
  temps.push_back(q);
  *p = (double *)q;
  return SNAC_OK;
}
OneBlock::~OneBlock() {
  if (dax) cudaFree(dax);
  if (dtiles) cudaFree(dtiles);
  if (dblk) cudaFree(dblk);
  for (void *q : temps) cudaFree(q);
}
size_t OneBlock::halo_bytes() const { return (size_t)(hb.n[0] + 2) * (hb.n[1] + 2) * (hb.n[2] + 2) * sizeof(double); }
size_t OneBlock::interior_bytes() const { return (size_t)hb.n[0] * hb.n[1] * hb.n[2] * sizeof(double); }

namespace {
// bound.f90:8-106 for one block on the caller's arrays: self-neighbour halo exchange along each direction,
// then set_bc face by face.  ent[a] holds one BcEntry per field along axis a (both sides in one entry).
int bound_block(OneBlock &ob, const int *flds, int nf, const int nb[3][2], int myrank,
                       const std::vector<BcEntry> (&ent)[3]) {
  int *dfl = nullptr;
  {
    double *q = nullptr;
    SNAC_TRY(ob.scratch(sizeof(int) * 8, &q));
    dfl = (int *)q;
    SNAC_CUDA(cudaMemcpy(dfl, flds, nf * sizeof(int), cudaMemcpyHostToDevice));
  }
  for (int a = 0; a < 3; a++) {
    FaceLink fl[2];
    int nl = 0;
    for (int sd = 0; sd < 2; sd++)
      if (nb[a][sd] == myrank) fl[nl++] = FaceLink{0, 0, sd, 0};
    const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
    const int maxplane = (ob.hb.n[t1] + 2) * (ob.hb.n[t2] + 2);
    if (nl) {
      double *q = nullptr;
      SNAC_TRY(ob.scratch(sizeof(fl), &q));
      SNAC_CUDA(cudaMemcpy(q, fl, nl * sizeof(FaceLink), cudaMemcpyHostToDevice));
      SNAC_TRY(launch_exchange(ob.dblk, (const FaceLink *)q, nl, dfl, nf, a, maxplane, 0));
    }
  }
  for (int a = 0; a < 3; a++) {
    if (ent[a].empty()) continue;
    const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
    double *q = nullptr;
    SNAC_TRY(ob.scratch(ent[a].size() * sizeof(BcEntry), &q));
    SNAC_CUDA(cudaMemcpy(q, ent[a].data(), ent[a].size() * sizeof(BcEntry), cudaMemcpyHostToDevice));
    SNAC_TRY(launch_setbc(ob.dblk, (const BcEntry *)q, (int)ent[a].size(), a, (ob.hb.n[t1] + 2) * (ob.hb.n[t2] + 2), 0));
  }
  SNAC_CUDA(cudaDeviceSynchronize());
  return bounds_check(0);
}

bool bound_args_ok(const int lo[3], const int hi[3], const int is_bound[3][2], const int nb[3][2]) {
  if (!lo || !hi || !is_bound || !nb) { set_error("null argument"); return false; }
  return true;
}

}  // namespace

}  // namespace snac

using namespace snac;

extern "C" {

const char *snac_last_error(void) { return g_err.c_str(); }

int snac_device_count(int *n) {
  int c = 0;
  cudaError_t e = cudaGetDeviceCount(&c);
  if (e != cudaSuccess) { *n = 0; return cuda_fail(e, "cudaGetDeviceCount", __FILE__, __LINE__); }
  *n = c;
  return SNAC_OK;
}

int snac_register(void *host, size_t bytes) {
  if (!host || !bytes) { set_error("snac_register: null pointer or zero size"); return SNAC_ERR_ARG; }
  void *dev = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mtx);
    if (g_mirrors.count(host)) { set_error("snac_register: pointer already registered"); return SNAC_ERR_ARG; }
  }
  SNAC_CUDA(cudaMalloc(&dev, bytes));
  SNAC_CUDA(cudaMemcpy(dev, host, bytes, cudaMemcpyHostToDevice));
  std::lock_guard<std::mutex> lk(g_mtx);
  g_mirrors[host] = Mirror{dev, bytes};
  return SNAC_OK;
}

int snac_unregister(void *host) {
  Mirror m;
  {
    std::lock_guard<std::mutex> lk(g_mtx);
    auto it = g_mirrors.find(host);
    if (it == g_mirrors.end()) { set_error("snac_unregister: pointer not registered"); return SNAC_ERR_ARG; }
    m = it->second;
    g_mirrors.erase(it);
  }
  SNAC_CUDA(cudaFree(m.dev));
  return SNAC_OK;
}

int snac_update_device(void *host) {
  Mirror m;
  {
    std::lock_guard<std::mutex> lk(g_mtx);
    auto it = g_mirrors.find(host);
    if (it == g_mirrors.end()) { set_error("snac_update_device: pointer not registered"); return SNAC_ERR_ARG; }
    m = it->second;
  }
  SNAC_CUDA(cudaMemcpy(m.dev, host, m.bytes, cudaMemcpyHostToDevice));
  return SNAC_OK;
}

int snac_update_host(void *host) {
  Mirror m;
  {
    std::lock_guard<std::mutex> lk(g_mtx);
    auto it = g_mirrors.find(host);
    if (it == g_mirrors.end()) { set_error("snac_update_host: pointer not registered"); return SNAC_ERR_ARG; }
    m = it->second;
  }
  SNAC_CUDA(cudaDeviceSynchronize());
  SNAC_CUDA(cudaMemcpy(host, m.dev, m.bytes, cudaMemcpyDeviceToHost));
  return SNAC_OK;
}

int snac_rk_mom(const double rkpar[2], const int lo[3], const int hi[3], const double *dxc, const double *dxf,
                const double *dyc, const double *dyf, const double *dzc, const double *dzf, double dt,
                const double bforce[3], const double gacc[3], double beta, const double *s1, double visc, double *u,
                double *v, double *w, const double *p, double *dudtrko, double *dvdtrko, double *dwdtrko, int impdiff,
                int boussinesq) {
  OneBlock ob;
  SNAC_TRY(ob.setup(lo, hi, dxc, dxf, dyc, dyf, dzc, dzf, false));
  const size_t hb = ob.halo_bytes(), ib = ob.interior_bytes();
  ArgArray U, V, W, Pa, RU, RV, RW, S;
  SNAC_TRY(U.bind(u, hb, true, true));
  SNAC_TRY(V.bind(v, hb, true, true));
  SNAC_TRY(W.bind(w, hb, true, true));
  SNAC_TRY(Pa.bind(p, hb, true, false));
  SNAC_TRY(RU.bind(dudtrko, ib, true, true));
  SNAC_TRY(RV.bind(dvdtrko, ib, true, true));
  SNAC_TRY(RW.bind(dwdtrko, ib, true, true));
  if (boussinesq) {
    if (!s1) { set_error("snac_rk_mom: boussinesq needs the scalar field"); return SNAC_ERR_ARG; }
    SNAC_TRY(S.bind(s1, hb, true, false));
    ob.hb.s[0] = (double *)S.dev;
  }
  ob.hb.u = (double *)U.dev; ob.hb.v = (double *)V.dev; ob.hb.w = (double *)W.dev; ob.hb.p = (double *)Pa.dev;
  ob.hb.ru = (double *)RU.dev; ob.hb.rv = (double *)RV.dev; ob.hb.rw = (double *)RW.dev;
  SNAC_TRY(ob.scratch(ib, &ob.hb.nu));
  SNAC_TRY(ob.scratch(ib, &ob.hb.nv));
  SNAC_TRY(ob.scratch(ib, &ob.hb.nw));
  SNAC_TRY(ob.upload());
  RkMomParams prm;
  prm.f1 = rkpar[0] * dt;
  prm.f2 = rkpar[1] * dt;
  prm.f12 = prm.f1 + prm.f2;
  for (int a = 0; a < 3; a++) {
    prm.bforce[a] = bforce ? bforce[a] : 0.0;
    prm.gb[a] = boussinesq ? prm.f12 * gacc[a] * beta * 0.5 : 0.0;
  }
  prm.visc = visc;
  prm.impdiff = impdiff;
  prm.halo_out = 0;  // the caller owns u, v, w: interior scratch, written back
  prm.boussinesq = boussinesq;
  SNAC_TRY(launch_rk_mom(ob.dblk, ob.dtiles, ob.ntiles, prm, 0));
  SNAC_TRY(launch_rk_mom_writeback(ob.dblk, ob.dtiles, ob.ntiles, 0));
  SNAC_CUDA(cudaDeviceSynchronize());
  SNAC_TRY(bounds_check(0));
  SNAC_TRY(U.finish()); SNAC_TRY(V.finish()); SNAC_TRY(W.finish());
  SNAC_TRY(RU.finish()); SNAC_TRY(RV.finish()); SNAC_TRY(RW.finish());
  return SNAC_OK;
}

int snac_rk_scal(const double rkpar[2], const int lo[3], const int hi[3], const double *dxc, const double *dxf,
                 const double *dyc, const double *dyf, const double *dzc, const double *dzf, double dt, double alpha,
                 double vol_all, const double *u, const double *v, const double *w, int is_forced, double scalf,
                 double ssource, double *dsdtrko, double *s, double *f, int impdiff) {
  OneBlock ob;
  SNAC_TRY(ob.setup(lo, hi, dxc, dxf, dyc, dyf, dzc, dzf, false));
  const size_t hb = ob.halo_bytes(), ib = ob.interior_bytes();
  ArgArray U, V, W, S, RS;
  SNAC_TRY(U.bind(u, hb, true, false));
  SNAC_TRY(V.bind(v, hb, true, false));
  SNAC_TRY(W.bind(w, hb, true, false));
  SNAC_TRY(S.bind(s, hb, true, true));
  SNAC_TRY(RS.bind(dsdtrko, ib, true, true));
  ob.hb.u = (double *)U.dev; ob.hb.v = (double *)V.dev; ob.hb.w = (double *)W.dev;
  ob.hb.s[0] = (double *)S.dev;
  ob.hb.rs[0] = (double *)RS.dev;
  SNAC_TRY(ob.scratch(ib, &ob.hb.ns));
  SNAC_TRY(ob.upload());
  RkScalParams prm;
  prm.f1 = rkpar[0] * dt;
  prm.f2 = rkpar[1] * dt;
  prm.f12 = prm.f1 + prm.f2;
  prm.alpha = alpha;
  prm.ssource = ssource;
  prm.impdiff = impdiff;
  prm.sidx = 0;
  // bulk_mean_s (scal.f90:156-179) is fused into the update kernel as per-tile partial sums
  double *part = nullptr, *res = nullptr, r[2] = {0.0, 0.0};
  if (is_forced && f) {
    SNAC_TRY(ob.scratch((size_t)ob.ntiles * 2 * sizeof(double), &part));
    SNAC_TRY(ob.scratch(2 * sizeof(double), &res));
  }
  SNAC_TRY(launch_rk_scal(ob.dblk, ob.dtiles, ob.ntiles, prm, part, 0));
  SNAC_TRY(launch_rk_scal_writeback(ob.dblk, ob.dtiles, ob.ntiles, 0, 0));
  if (part) {
    SNAC_TRY(launch_reduce_final(part, ob.ntiles, res, 0));
    SNAC_CUDA(cudaMemcpy(r, res, 2 * sizeof(double), cudaMemcpyDeviceToHost));
  }
  SNAC_CUDA(cudaDeviceSynchronize());
  SNAC_TRY(bounds_check(0));
  SNAC_TRY(S.finish());
  SNAC_TRY(RS.finish());
  if (f) *f = (is_forced ? scalf - r[0] / vol_all : 0.0);
  return SNAC_OK;
}

int snac_fillps(const int lo[3], const int hi[3], const double *dxf, const double *dyf, const double *dzf, double dt,
                const double *u, const double *v, const double *w, double *p, int fft_axis) {
  OneBlock ob;
  SNAC_TRY(ob.setup(lo, hi, dxf, dxf, dyf, dyf, dzf, dzf, false));
  const size_t hb = ob.halo_bytes();
  ArgArray U, V, W, Pp;
  SNAC_TRY(U.bind(u, hb, true, false));
  SNAC_TRY(V.bind(v, hb, true, false));
  SNAC_TRY(W.bind(w, hb, true, false));
  SNAC_TRY(Pp.bind(p, hb, true, true));
  ob.hb.u = (double *)U.dev; ob.hb.v = (double *)V.dev; ob.hb.w = (double *)W.dev; ob.hb.pp = (double *)Pp.dev;
  SNAC_TRY(ob.upload());
  SNAC_TRY(launch_fillps(ob.dblk, ob.dtiles, ob.ntiles, dt, fft_axis, 0));
  SNAC_CUDA(cudaDeviceSynchronize());
  SNAC_TRY(bounds_check(0));
  SNAC_TRY(Pp.finish());
  return SNAC_OK;
}

int snac_correc(const int lo[3], const int hi[3], const double *dxc, const double *dyc, const double *dzc, double dt,
                const double *p, double *u, double *v, double *w) {
  OneBlock ob;
  SNAC_TRY(ob.setup(lo, hi, dxc, dxc, dyc, dyc, dzc, dzc, true));
  const size_t hb = ob.halo_bytes();
  ArgArray U, V, W, Pp;
  SNAC_TRY(U.bind(u, hb, true, true));
  SNAC_TRY(V.bind(v, hb, true, true));
  SNAC_TRY(W.bind(w, hb, true, true));
  SNAC_TRY(Pp.bind(p, hb, true, false));
  ob.hb.u = (double *)U.dev; ob.hb.v = (double *)V.dev; ob.hb.w = (double *)W.dev; ob.hb.pp = (double *)Pp.dev;
  SNAC_TRY(ob.upload());
  SNAC_TRY(launch_correc(ob.dblk, ob.dtiles, ob.ntiles, dt, 0));
  SNAC_CUDA(cudaDeviceSynchronize());
  SNAC_TRY(bounds_check(0));
  SNAC_TRY(U.finish()); SNAC_TRY(V.finish()); SNAC_TRY(W.finish());
  return SNAC_OK;
}

int snac_updt_pressure(const int lo[3], const int hi[3], const double *dxc, const double *dxf, const double *dyc,
                       const double *dyf, const double *dzc, const double *dzf, double alpha, const double *pp,
                       double *p, int impdiff) {
  OneBlock ob;
  SNAC_TRY(ob.setup(lo, hi, dxc, dxf, dyc, dyf, dzc, dzf, false));
  const size_t hb = ob.halo_bytes();
  ArgArray PP, Pa;
  SNAC_TRY(PP.bind(pp, hb, true, false));
  SNAC_TRY(Pa.bind(p, hb, true, true));
  ob.hb.pp = (double *)PP.dev;
  ob.hb.p = (double *)Pa.dev;
  SNAC_TRY(ob.upload());
  SNAC_TRY(launch_updt_pressure(ob.dblk, ob.dtiles, ob.ntiles, alpha, impdiff, 0));
  SNAC_CUDA(cudaDeviceSynchronize());
  SNAC_TRY(bounds_check(0));
  SNAC_TRY(Pa.finish());
  return SNAC_OK;
}

int snac_updt_rhs(const int lo[3], const int hi[3], const int is_bound[3][2], const double *rhsx, const double *rhsy,
                  const double *rhsz, double *p) {
  OneBlock ob;
  SNAC_TRY(ob.setup(lo, hi, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, false));
  const int nx = ob.hb.n[0], ny = ob.hb.n[1], nz = ob.hb.n[2];
  ArgArray Pa, RX, RY, RZ;
  SNAC_TRY(Pa.bind(p, ob.halo_bytes(), true, true));
  SNAC_TRY(RX.bind(rhsx, (size_t)ny * nz * 2 * sizeof(double), true, false));
  SNAC_TRY(RY.bind(rhsy, (size_t)nx * nz * 2 * sizeof(double), true, false));
  SNAC_TRY(RZ.bind(rhsz, (size_t)nx * ny * 2 * sizeof(double), true, false));
  int isb[6];
  for (int a = 0; a < 3; a++) for (int s = 0; s < 2; s++) isb[2 * a + s] = is_bound[a][s];
  SNAC_TRY(launch_updt_rhs(nx, ny, nz, isb, (const double *)RX.dev, (const double *)RY.dev, (const double *)RZ.dev,
                           (double *)Pa.dev, 0));
  SNAC_CUDA(cudaDeviceSynchronize());
  SNAC_TRY(bounds_check(0));
  SNAC_TRY(Pa.finish());
  return SNAC_OK;
}

static int reduce_one(OneBlock &ob, int which, double vol, double out[2]) {
  double *part = nullptr, *res = nullptr;
  SNAC_TRY(ob.scratch((size_t)ob.ntiles * 2 * sizeof(double), &part));
  SNAC_TRY(ob.scratch(2 * sizeof(double), &res));
  if (which == 0) SNAC_TRY(launch_chkdt_partial(ob.dblk, ob.dtiles, ob.ntiles, part, 0));
  else SNAC_TRY(launch_chkdiv_partial(ob.dblk, ob.dtiles, ob.ntiles, vol, part, 0));
  SNAC_TRY(launch_reduce_final(part, ob.ntiles, res, 0));
  SNAC_CUDA(cudaMemcpy(out, res, 2 * sizeof(double), cudaMemcpyDeviceToHost));
  return SNAC_OK;
}

int snac_chkdt(const int lo[3], const int hi[3], const double *dxc, const double *dxf, const double *dyc,
               const double *dyf, const double *dzc, const double *dzf, double visc, const double *u, const double *v,
               const double *w, int impdiff, double *dtmax) {
  OneBlock ob;
  SNAC_TRY(ob.setup(lo, hi, dxc, dxf, dyc, dyf, dzc, dzf, false));
  const size_t hb = ob.halo_bytes();
  ArgArray U, V, W;
  SNAC_TRY(U.bind(u, hb, true, false));
  SNAC_TRY(V.bind(v, hb, true, false));
  SNAC_TRY(W.bind(w, hb, true, false));
  ob.hb.u = (double *)U.dev; ob.hb.v = (double *)V.dev; ob.hb.w = (double *)W.dev;
  SNAC_TRY(ob.upload());
  double r[2];
  SNAC_TRY(reduce_one(ob, 0, 1.0, r));
  double dti = r[1];
  if (std::isinf(dti)) { set_error("snac_chkdt: non-finite velocity"); return SNAC_ERR_NAN; }
  if (dti == 0.0) dti = 1.0;
  double dtm = std::sqrt(3.0) / dti;
  if (!impdiff) {
    double dlmin = dxf[0];
    for (int q = 0; q < ob.hb.n[0] + 2; q++) dlmin = std::min(dlmin, dxf[q]);
    for (int q = 0; q < ob.hb.n[1] + 2; q++) dlmin = std::min(dlmin, dyf[q]);
    for (int q = 0; q < ob.hb.n[2] + 2; q++) dlmin = std::min(dlmin, dzf[q]);
    dtm = std::min(dtm, 1.65 / 12.0 / visc * (dlmin * dlmin));
  }
  *dtmax = dtm;
  return SNAC_OK;
}

int snac_chkdiv(const int lo[3], const int hi[3], const double *dxf, const double *dyf, const double *dzf,
                const double *u, const double *v, const double *w, double vol, double *divtot, double *divmax) {
  OneBlock ob;
  SNAC_TRY(ob.setup(lo, hi, dxf, dxf, dyf, dyf, dzf, dzf, false));
  const size_t hb = ob.halo_bytes();
  ArgArray U, V, W;
  SNAC_TRY(U.bind(u, hb, true, false));
  SNAC_TRY(V.bind(v, hb, true, false));
  SNAC_TRY(W.bind(w, hb, true, false));
  ob.hb.u = (double *)U.dev; ob.hb.v = (double *)V.dev; ob.hb.w = (double *)W.dev;
  SNAC_TRY(ob.upload());
  double r[2];
  SNAC_TRY(reduce_one(ob, 1, vol, r));
  *divtot = r[0];
  *divmax = r[1];
  return SNAC_OK;
}

int snac_set_bc(char ctype, int ibound, const int lo[3], const int hi[3], int idir, int centered, double rvalue,
                double dr, double *p) {
  if (idir < 1 || idir > 3 || ibound < 0 || ibound > 1) { set_error("snac_set_bc: bad idir/ibound"); return SNAC_ERR_ARG; }
  OneBlock ob;
  SNAC_TRY(ob.setup(lo, hi, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, false));
  ArgArray Pa;
  SNAC_TRY(Pa.bind(p, ob.halo_bytes(), true, true));
  ob.hb.p = (double *)Pa.dev;
  SNAC_TRY(ob.upload());
  BcEntry e;
  memset(&e, 0, sizeof(e));
  e.b = 0;
  e.f = 3;
  bc_mode(ctype, ibound, centered, rvalue, dr, &e.mode[ibound], &e.factor[ibound], &e.sgn[ibound]);
  BcEntry *de = nullptr;
  SNAC_CUDA(cudaMalloc(&de, sizeof(BcEntry)));
  cudaMemcpy(de, &e, sizeof(e), cudaMemcpyHostToDevice);
  const int a = idir - 1;
  const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
  int rc = launch_setbc(ob.dblk, de, 1, a, (ob.hb.n[t1] + 2) * (ob.hb.n[t2] + 2), 0);
  cudaDeviceSynchronize();
  cudaFree(de);
  SNAC_TRY(rc);
  SNAC_TRY(Pa.finish());
  return SNAC_OK;
}

int snac_bounduvw(const char cbc[3][3][2], const int lo[3], const int hi[3], const double bc[3][3][2], int is_correc,
                  const int is_bound[3][2], const int nb[3][2], int myrank, const double *dxc, const double *dxf,
                  const double *dyc, const double *dyf, const double *dzc, const double *dzf, double *u, double *v,
                  double *w) {
  if (!bound_args_ok(lo, hi, is_bound, nb) || !cbc || !bc || !dxc || !dxf || !dyc || !dyf || !dzc || !dzf || !u ||
      !v || !w) {
    set_error("snac_bounduvw: null argument");
    return SNAC_ERR_ARG;
  }
  OneBlock ob;
  SNAC_TRY(ob.setup(lo, hi, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, false));
  ArgArray Ua, Va, Wa;
  SNAC_TRY(Ua.bind(u, ob.halo_bytes(), true, true));
  SNAC_TRY(Va.bind(v, ob.halo_bytes(), true, true));
  SNAC_TRY(Wa.bind(w, ob.halo_bytes(), true, true));
  ob.hb.u = (double *)Ua.dev; ob.hb.v = (double *)Va.dev; ob.hb.w = (double *)Wa.dev;
  SNAC_TRY(ob.upload());
  const double *dc[3] = {dxc, dyc, dzc}, *df[3] = {dxf, dyf, dzf};
  std::vector<BcEntry> ent[3];
  for (int a = 0; a < 3; a++)
    for (int c = 0; c < 3; c++) {
      BcEntry e;
      memset(&e, 0, sizeof(e));
      e.b = 0;
      e.f = c;
      const int centered = c != a;
      bool any = false;
      for (int sd = 0; sd < 2; sd++) {
        if (!is_bound[a][sd] || (!centered && is_correc)) continue;
        const int q = sd ? ob.hb.n[a] : 0;  // dl(lo-1) or dl(hi)
        bc_mode(cbc[c][a][sd], sd, centered, bc[c][a][sd], centered ? dc[a][q] : df[a][q], &e.mode[sd],
                &e.factor[sd], &e.sgn[sd]);
        any = true;
      }
      if (any) ent[a].push_back(e);
    }
  const int flds[3] = {0, 1, 2};
  SNAC_TRY(bound_block(ob, flds, 3, nb, myrank, ent));
  SNAC_TRY(Ua.finish());
  SNAC_TRY(Va.finish());
  SNAC_TRY(Wa.finish());
  return SNAC_OK;
}

int snac_boundp(const char cbc[3][2], const int lo[3], const int hi[3], const double bc[3][2], const int is_bound[3][2],
                const int nb[3][2], int myrank, const double *dxc, const double *dyc, const double *dzc, double *p) {
  if (!bound_args_ok(lo, hi, is_bound, nb) || !cbc || !bc || !dxc || !dyc || !dzc || !p) {
    set_error("snac_boundp: null argument");
    return SNAC_ERR_ARG;
  }
  OneBlock ob;
  SNAC_TRY(ob.setup(lo, hi, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, false));
  ArgArray Pa;
  SNAC_TRY(Pa.bind(p, ob.halo_bytes(), true, true));
  ob.hb.p = (double *)Pa.dev;
  SNAC_TRY(ob.upload());
  const double *dc[3] = {dxc, dyc, dzc};
  std::vector<BcEntry> ent[3];
  for (int a = 0; a < 3; a++) {
    BcEntry e;
    memset(&e, 0, sizeof(e));
    e.b = 0;
    e.f = 3;
    bool any = false;
    for (int sd = 0; sd < 2; sd++) {
      if (!is_bound[a][sd]) continue;
      const int q = sd ? ob.hb.n[a] : 0;
      bc_mode(cbc[a][sd], sd, 1, bc[a][sd], dc[a][q], &e.mode[sd], &e.factor[sd], &e.sgn[sd]);
      any = true;
    }
    if (any) ent[a].push_back(e);
  }
  const int flds[1] = {3};
  SNAC_TRY(bound_block(ob, flds, 1, nb, myrank, ent));
  SNAC_TRY(Pa.finish());
  return SNAC_OK;
}

}  // extern "C"
