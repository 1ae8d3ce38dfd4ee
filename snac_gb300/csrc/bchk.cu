// bchk.cu -- the host side of the bounds-check build (compiled with -DSNAC_BOUNDS_CHECK into
// libsnac_gb300_checked.so; bench and tests use the normal build).  The device checks (snac_internal.h: bchk,
// AX) record the first failing access of any kernel into one library-owned device word; the entry points that
// run kernels read it back (bounds_check) and turn it into SNAC_ERR_BOUNDS with the kernel and the cell.
#include <cstring>

#include "snac_host.h"

namespace snac {

#ifdef SNAC_BOUNDS_CHECK
static unsigned long long *g_flag = nullptr;  // one word per process, on the device current at first use

unsigned long long *bounds_flag() {
  if (!g_flag) {
    if (cudaMalloc(&g_flag, sizeof(unsigned long long)) != cudaSuccess) { g_flag = nullptr; return nullptr; }
    cudaMemset(g_flag, 0, sizeof(unsigned long long));
  }
  return g_flag;
}

int bounds_check(cudaStream_t st) {
  if (!g_flag) return SNAC_OK;
  unsigned long long v = 0;
  SNAC_CUDA(cudaMemcpyAsync(&v, g_flag, sizeof(v), cudaMemcpyDeviceToHost, st));
  SNAC_CUDA(cudaStreamSynchronize(st));
  if (!v) return SNAC_OK;
  SNAC_CUDA(cudaMemsetAsync(g_flag, 0, sizeof(v), st));
  static const char *names[BK_NKIND] = {"?", "tiled stencil", "1-D table", "halo exchange (destination)",
                                        "halo exchange (source)", "boundary condition", "inflow", "probe"};
  const int kid = (int)((v >> 48) & 0x7FFF);
  const int i = (int)((v >> 32) & 0xFFFF) - 32768, j = (int)((v >> 16) & 0xFFFF) - 32768, k = (int)(v & 0xFFFF) - 32768;
  set_error("bounds check: %s kernel addressed (%d, %d, %d) outside its block", kid > 0 && kid < BK_NKIND ? names[kid] : "?",
            i, j, k);
  return SNAC_ERR_BOUNDS;
}

// a check that fails on purpose: cell (n0 + 5, 0, 0) of a 4^3 block is tested, never addressed
__global__ void k_bchk_probe(DBlock B) { (void)bchk(B, BK_PROBE, B.n[0] + 5, 0, 0, 0, 0); }
#else
unsigned long long *bounds_flag() { return nullptr; }
int bounds_check(cudaStream_t) { return SNAC_OK; }
#endif

}  // namespace snac

using namespace snac;

int snac_bounds_checked(void) {
#ifdef SNAC_BOUNDS_CHECK
  return 1;
#else
  return 0;
#endif
}

int snac_bounds_selftest(void) {
#ifdef SNAC_BOUNDS_CHECK
  DBlock B;
  memset(&B, 0, sizeof(B));
  B.n[0] = B.n[1] = B.n[2] = 4;
  B.bchk = bounds_flag();
  if (!B.bchk) { set_error("device allocation failed (bounds flag)"); return SNAC_ERR_NOMEM; }
  k_bchk_probe<<<1, 1>>>(B), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  SNAC_CUDA(cudaDeviceSynchronize());
  return bounds_check(0);
#else
  set_error("snac_bounds_selftest: this library was built without SNAC_BOUNDS_CHECK");
  return SNAC_ERR_UNSUPPORTED;
#endif
}
