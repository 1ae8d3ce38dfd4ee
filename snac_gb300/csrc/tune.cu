// tune.cu -- snac_autotune: the solver settings for the case at hand, chosen by timing RK3 steps.
//
// The candidates differ in the solve (plain FP64, or mixed with 5, 6 or 7 FP32 Krylov iterations per
// refinement step, finished in FP64 or refined in FP32 to convergence), the smoothing sweeps per side on the
// coarse levels and, for the transform-axis solve, the smoother tile shape, the CTA waves per launch and the
// first level of the one-CTA coarse V-cycle; all solve to the same tolerance.  Each candidate rebuilds the
// solvers and runs from the same snapshot of the state; the state is restored afterwards, including the
// solvers' warm starts, so the run continues as if only the settings had changed.
#include <string>
#include <vector>

#include "snac_host.h"

namespace snac {
namespace {

struct SnapArray {
  double *live, *copy;
  size_t bytes;
};
struct Snapshot {
  std::vector<SnapArray> arrays;
  std::vector<std::pair<size_t, double *>> boxes;     // per solver slot (0 pressure, 1.. Helmholtz): size, copy
  double dt = 0.0, time = 0.0;
  int istep = 0;
  ~Snapshot() {
    for (auto &a : arrays) cudaFree(a.copy);
    for (auto &b : boxes) cudaFree(b.second);
  }
};

int snap_array(Snapshot &s, double *live, size_t bytes, cudaStream_t st) {
  if (!live) return SNAC_OK;
  double *c = nullptr;
  if (cudaMalloc(&c, bytes) != cudaSuccess) { set_error("snac_autotune: device allocation failed (snapshot)"); return SNAC_ERR_NOMEM; }
  s.arrays.push_back({live, c, bytes});
  SNAC_CUDA(cudaMemcpyAsync(c, live, bytes, cudaMemcpyDeviceToDevice, st));
  return SNAC_OK;
}

std::vector<PoissonSolver *> solvers(Domain &d) {
  std::vector<PoissonSolver *> v{d.ps.get()};
  for (auto &h : d.hs) v.push_back(h.get());
  return v;
}

size_t box_bytes(const PoissonSolver &S) { return (size_t)S.P.L[0].ncell * S.P.nsys * sizeof(double); }

int take(Domain &d, Snapshot &s) {
  cudaStream_t st = d.st;
  for (int b = 0; b < d.nblocks; b++) {
    const DBlock &B = d.db[b];
    const size_t nh = (size_t)(B.n[0] + 2) * (B.n[1] + 2) * (B.n[2] + 2) * sizeof(double);
    const size_t ni = (size_t)B.n[0] * B.n[1] * B.n[2] * sizeof(double);
    for (double *p : {B.u, B.v, B.w, B.p, B.pp}) SNAC_TRY(snap_array(s, p, nh, st));
    for (double *p : {B.ru, B.rv, B.rw}) SNAC_TRY(snap_array(s, p, ni, st));
    for (int q = 0; q < d.c.nscal; q++) {
      SNAC_TRY(snap_array(s, B.s[q], nh, st));
      SNAC_TRY(snap_array(s, B.rs[q], ni, st));
    }
  }
  for (PoissonSolver *S : solvers(d)) {
    double *c = nullptr;
    size_t n = 0;
    if (S && S->box_x) {
      n = box_bytes(*S);
      if (cudaMalloc(&c, n) != cudaSuccess) { set_error("snac_autotune: device allocation failed (snapshot)"); return SNAC_ERR_NOMEM; }
      SNAC_CUDA(cudaMemcpyAsync(c, S->box_x, n, cudaMemcpyDeviceToDevice, st));
    }
    s.boxes.push_back({n, c});
  }
  s.dt = d.dt;
  s.time = d.time;
  s.istep = d.istep;
  SNAC_CUDA(cudaStreamSynchronize(st));
  return SNAC_OK;
}

// rebuild the pressure solver and the Helmholtz solvers with the current settings
int rebuild(Domain &d) {
  SNAC_CUDA(cudaStreamSynchronize(d.st));
  d.ps.reset(new PoissonSolver());
  SNAC_TRY(solver_create(d, *d.ps));
  for (int f = HF_U; d.c.impdiff && f < HF_S0 + d.c.nscal; f++) {
    d.hs[f].reset(new PoissonSolver());
    SNAC_TRY(solver_create(d, *d.hs[f], true, f));
  }
  return SNAC_OK;
}

int restore(Domain &d, const Snapshot &s, bool boxes) {
  cudaStream_t st = d.st;
  for (const SnapArray &a : s.arrays) SNAC_CUDA(cudaMemcpyAsync(a.live, a.copy, a.bytes, cudaMemcpyDeviceToDevice, st));
  if (boxes) {
    const auto sv = solvers(d);
    for (size_t i = 0; i < sv.size() && i < s.boxes.size(); i++)
      if (sv[i] && sv[i]->box_x && s.boxes[i].second && box_bytes(*sv[i]) == s.boxes[i].first)
        SNAC_CUDA(cudaMemcpyAsync(sv[i]->box_x, s.boxes[i].second, s.boxes[i].first, cudaMemcpyDeviceToDevice, st));
  }
  d.dt = s.dt;
  d.time = s.time;
  d.istep = s.istep;
  SNAC_CUDA(cudaStreamSynchronize(st));
  return SNAC_OK;
}

int g_fail_candidate = -1;  // snac_tune_inject_failure

}  // namespace
}  // namespace snac

using namespace snac;

int snac_tune_inject_failure(int candidate) {
  g_fail_candidate = candidate;
  return SNAC_OK;
}

int snac_autotune(int steps, snac_tune_result *out) {
  Domain *d = domain();
  if (!d) { set_error("snac_autotune: no domain (call snac_init first)"); return SNAC_ERR_STATE; }
  if (steps < 1) { set_error("snac_autotune: steps must be >= 1"); return SNAC_ERR_ARG; }
  const snac_options opt0 = d->opt;
  const bool plane = d->ps && !d->ps->mode3d;
  // the timed steps solve the same restored state again and again: recording them as training pairs of the
  // learned guess would fill its ring with near-copies, so recording pauses while tuning
  const int gmode0 = guess_get_mode(*d);
  if (gmode0 == 1) guess_set_mode(*d, 0);
  Snapshot snap;
  // on every way out: the chosen (or, after an error, the original) settings, solvers built for them and the
  // state of the snapshot, so that the run goes on as if only the settings had changed
  auto finish = [&](const snac_options &o, int rc) -> int {
    d->opt = o;
    const std::string msg = rc != SNAC_OK ? std::string(snac_last_error()) : std::string();
    int rc2 = rebuild(*d);
    if (rc2 == SNAC_OK && !snap.arrays.empty()) rc2 = restore(*d, snap, true);
    guess_set_mode(*d, gmode0);
    if (rc != SNAC_OK) {
      set_error("%s", msg.c_str());
      return rc;
    }
    return rc2;
  };
  {
    const int rc = take(*d, snap);
    if (rc != SNAC_OK) { guess_set_mode(*d, gmode0); return rc; }
  }
  // the settings in use: one warm-up step and `steps` timed steps from the snapshot
  auto time_current = [&](double *ms) -> int {
    SNAC_TRY(restore(*d, snap, true));
    const int rc1 = snac_step(1);
    if (rc1 != SNAC_OK) return rc1;
    const int rc = snac_step(steps);
    *ms = d->device_ms / steps;
    return rc;
  };
  double ms_before = 0.0;
  {
    const int rc = time_current(&ms_before);
    if (rc != SNAC_OK) return finish(opt0, rc);
  }
  // Candidates are searched one group at a time, each group varying its settings around the best so far:
  // the solve (plain FP64, or mixed with 5, 6 or 7 FP32 iterations per refinement step) x the coarse-level
  // sweeps; then, for the plane systems, the smoother tile shape and the waves of CTAs per batched launch;
  // then the level where the one-CTA coarse V-cycle starts; then, for the mixed solve, FP64 finishing after
  // two refinement steps against FP32 refinement to convergence.
  snac_options best_opt = opt0;
  double best = 1e300;
  int ntimed = 0, found = 0;
  auto try_group = [&](const std::vector<snac_options> &group) -> int {
    for (const snac_options &o : group) {
      d->opt = o;
      int rc = rebuild(*d);
      if (rc == SNAC_OK && ntimed == g_fail_candidate) {
        g_fail_candidate = -1;
        set_error("snac_autotune: failure injected at candidate %d", ntimed);
        rc = SNAC_ERR_STATE;
      }
      double ms = 0.0;
      if (rc == SNAC_OK) rc = time_current(&ms);
      ntimed++;
      if (rc == SNAC_ERR_NOT_CONVERGED) continue;  // this candidate does not reach the tolerance
      if (rc != SNAC_OK) return rc;
      if (ms < best) { best = ms; best_opt = o; found = 1; }
    }
    return SNAC_OK;
  };
  std::vector<snac_options> g;
  for (int nuc : plane ? std::vector<int>{1, 2} : std::vector<int>{0}) {
    for (int inner : {5, 6, 7}) {
      snac_options o = opt0;
      o.precision = 1; o.inner_iters = inner; o.nu_coarse = nuc;
      g.push_back(o);
    }
    snac_options o = opt0;
    o.precision = 0; o.inner_iters = 0; o.nu_coarse = nuc;
    g.push_back(o);
  }
  int rc = try_group(g);
  if (rc == SNAC_OK && found && plane) {
    g.clear();
    for (int t = 1; t <= 6; t++) { snac_options o = best_opt; o.mg_tile = t; g.push_back(o); }
    rc = try_group(g);
  }
  if (rc == SNAC_OK && found && plane) {
    g.clear();
    for (int w : {1, 2, 4}) { snac_options o = best_opt; o.mg_waves = w; g.push_back(o); }
    rc = try_group(g);
  }
  if (rc == SNAC_OK && found && d->ps) {
    // the one-CTA coarse V-cycle from the default level, one level coarser or one level finer
    d->opt = best_opt;
    rc = rebuild(*d);
    if (rc == SNAC_OK) {
      const int prec = best_opt.precision ? 0 : 1;
      const int l0 = d->ps->P.cta_level[prec];
      g.clear();
      if (l0 + 1 < d->ps->P.nlev) {
        snac_options o = best_opt; o.mg_cta_level = l0 + 1; g.push_back(o);
        o.mg_cta_level = l0; g.push_back(o);
        if (l0 > 1) { o.mg_cta_level = l0 - 1; g.push_back(o); }  // (0 would mean the default again)
      }
      rc = try_group(g);
    }
  }
  if (rc == SNAC_OK && found && best_opt.precision == 1) {
    g.clear();
    for (int r : {-1, 2}) { snac_options o = best_opt; o.refine_steps = r; g.push_back(o); }
    rc = try_group(g);
  }
  if (rc != SNAC_OK) return finish(opt0, rc);
  // nothing converged: keep the settings that were in use
  SNAC_TRY(finish(found ? best_opt : opt0, SNAC_OK));
  if (out) {
    out->precision = d->opt.precision;
    out->inner_iters = d->ps ? d->ps->inner_iters : 0;
    out->nu_coarse = d->ps ? d->ps->P.nu_coarse : 0;
    out->ms_per_step = found ? best : ms_before;
    out->ms_before = ms_before;
    out->ncand = ntimed;
    out->mg_tile = d->ps && plane ? tile2d_shape_index(d->ps->P, 0) : 0;
    out->mg_waves = d->ps ? d->ps->P.waves : 0;
    out->mg_cta_level = d->ps ? d->ps->P.cta_level[d->opt.precision ? 0 : 1] : 0;
    out->refine_steps = d->ps ? d->ps->refine_steps : 0;
  }
  return SNAC_OK;
}
