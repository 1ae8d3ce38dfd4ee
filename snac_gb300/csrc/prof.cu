// prof.cu -- CUDA-event timing of one selected kernel class on the launching stream.
#include <atomic>
#include <vector>

#include "snac_prof.h"

namespace snac {

namespace {
struct Prof {
  int kid = 0;
  std::vector<cudaEvent_t> ev;  // pairs
  int n = 0;                    // recorded pairs
  bool open = false;
};
Prof g_prof;
constexpr int PROF_MAX = 8192;
}  // namespace

static std::atomic<long long> g_launches{0};
int g_pdl = 1;
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void add_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
bool prof_active() { return g_prof.kid != 0; }

void prof_begin(int kid, cudaStream_t st) {
  if (g_prof.kid != kid || g_prof.n >= PROF_MAX) return;
  if ((int)g_prof.ev.size() < 2 * (g_prof.n + 1)) {
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    g_prof.ev.push_back(a);
    g_prof.ev.push_back(b);
  }
  cudaEventRecord(g_prof.ev[2 * g_prof.n], st);
  g_prof.open = true;
}

void prof_end(int kid, cudaStream_t st) {
  if (g_prof.kid != kid || !g_prof.open) return;
  cudaEventRecord(g_prof.ev[2 * g_prof.n + 1], st);
  g_prof.n++;
  g_prof.open = false;
}

}  // namespace snac

extern "C" int snac_profile_kernel(int kid) {
  snac::g_prof.kid = kid;
  snac::g_prof.n = 0;
  snac::g_prof.open = false;
  return SNAC_OK;
}

extern "C" int snac_profile_read(int *launches, double *total_ms) {
  SNAC_CUDA(cudaDeviceSynchronize());
  double tot = 0.0;
  for (int q = 0; q < snac::g_prof.n; q++) {
    float ms = 0.f;
    SNAC_CUDA(cudaEventElapsedTime(&ms, snac::g_prof.ev[2 * q], snac::g_prof.ev[2 * q + 1]));
    tot += ms;
  }
  *launches = snac::g_prof.n;
  *total_ms = tot;
  return SNAC_OK;
}

extern "C" int snac_launch_count(long long *n) {
  if (!n) return SNAC_ERR_ARG;
  *n = snac::g_launches.load(std::memory_order_relaxed);
  return SNAC_OK;
}
