// snac_prof.h -- kernel classes that snac_profile_kernel can time with CUDA events.
#pragma once
#include "snac_internal.h"

namespace snac {

enum KernelClass {
  KID_NONE = 0,
  KID_RK_MOM = 1,        // k_rk_mom
  KID_RBGS = 2,          // k_rbgs (every level, both precisions)
  KID_RESTRICT = 3,      // k_resid_restrict
  KID_FFT_FWD = 4,       // k_fft_fwd_box
  KID_FFT_BWD = 5,       // k_fft_bwd_box
  KID_CG_APPLY = 6,      // k_cg_apply
  KID_FILLPS = 7,        // k_fillps
  KID_CORREC = 8,        // k_correc
  KID_COARSE = 9,        // k_vcycle_coarse
  KID_SOLVE = 10,        // one whole pressure solve (transforms + Krylov + V-cycles)
};

void prof_begin(int kid, cudaStream_t st);
void prof_end(int kid, cudaStream_t st);
bool prof_active();                // a kernel class is being timed (graph replay is then not used)
void add_launches(long long n);    // launches of a replayed CUDA graph (negative: undo captured ones)
bool trace_on();                   // SNAC_DEBUG tracing synchronises after every phase (no capture then)

}  // namespace snac
