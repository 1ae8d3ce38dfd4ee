// snac_bound.h -- tables driving the halo-exchange / boundary-condition kernels.
#pragma once
#include "snac_internal.h"

namespace snac {

// one friend link of one block along one axis: ghost plane of `dst` on `side`
// receives the facing interior plane of `src` (updthalo, bound.f90:587-650)
struct FaceLink {
  int dst, src, side, pad;
};

enum BcMode { BC_NONE = 0, BC_CENTRED = 1, BC_STAG_D = 2, BC_STAG_N = 3 };

// set_bc parameters (bound.f90:108-248) for both faces of one axis of one field of one block
struct BcEntry {
  int b, f;          // block, field (0..2 u,v,w, 3 p, 4 pp, 5+s scalar s)
  int mode[2];
  double factor[2], sgn[2];
};

// one inflow face of one block (bound.f90:438-477): the planes u_in, v_in, w_in over (lo-1:hi+1) of the
// two tangential axes (the lower one fastest)
struct InflowFace {
  int b, pad;
  const double *pl[3];
};

void bc_mode(char ctype, int ibound, int centered, double rvalue, double dr, int *mode, double *factor, double *sgn);
int launch_exchange(const DBlock *dB, const FaceLink *dF, int nlinks, const int *dflds, int nflds, int a,
                    int maxplane, cudaStream_t st);
int launch_setbc(const DBlock *dB, const BcEntry *dE, int nent, int a, int maxplane, cudaStream_t st);
int launch_inflow(const DBlock *dB, const InflowFace *dI, int nface, int a, int side, int maxplane, int is_correc,
                  cudaStream_t st);

}  // namespace snac
