// k_tma.cu -- fillps (fillps.f90:27-53) with its 3-D tiles staged through shared memory by TMA.
//
// Persistent CTAs walk a list of 32 x 8 x 4 output tiles over all blocks.  For each tile one thread issues
// three tiled bulk-tensor copies (cp.async.bulk.tensor.3d) of u, v and w, each a 34 x 9 x 5 box of the
// halo'd field (the tile plus the cells before it) described by a tensor map per block and field, into
// one of two shared-memory stages; the copies complete on that stage's mbarrier (transaction bytes), so the
// next tile streams in while the current one is computed.  The divergence of fillps then reads only shared
// memory: the backward differences u(i)-u(i-1), v(j)-v(j-1), w(k)-w(k-1) of a thread's four cells along z.
// Same arithmetic as k_fillps, term by term, so the two agree bit for bit.
//
// Constraints of the tiled copies (checked on the host; else the plain kernel runs): the box's innermost
// coordinate starts at a multiple of 32 cells (16-byte aligned for FP64), the row pitch (n0 + 2) * 8 bytes is
// a multiple of 16 (n0 even), at most TMA_MAX_BLOCKS blocks.  Every mbarrier wait is bounded: past the limit the
// kernel records an error (SNAC_ERR_TIMEOUT on the host), waits (bounded) for its copies in flight and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <vector>

#include "snac_host.h"
#include "snac_prof.h"

namespace snac {

struct TmaMaps {
  CUtensorMap m[TMA_MAX_BLOCKS][3];  // per block: u, v, w
};

namespace {

constexpr int FX = 32, FY = 8, FZ = 4;              // output tile (interior cells); FX x FY threads
// staged box: the tile and the cell before it along each axis (fillps takes backward differences); x is one
// cell wider still, so that the box row is a whole number of 16-byte units
constexpr int BX = FX + 2, BY = FY + 1, BZ = FZ + 1;
constexpr int BOX_BYTES = BX * BY * BZ * 8;          // 12,240 bytes of one field's box
constexpr int BOX_PITCH = 12288;                     // box slot in shared memory (128-byte aligned)
constexpr int STAGE_BYTES = 3 * BOX_PITCH;           // u, v, w
constexpr int TMA_SMEM = 2 * STAGE_BYTES + 16;      // two stages and their mbarriers
constexpr long TMA_POLLS = 1L << 24;

__device__ __forceinline__ uint32_t sm32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity, long limit) {
  uint32_t done = 0;
  for (long it = 0; it < limit && !done; it++) {
    asm volatile(
        "{\n .reg .pred pw;\n mbarrier.try_wait.parity.shared::cta.b64 pw, [%1], %2;\n selp.u32 %0, 1, 0, pw;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
  }
  return done != 0;
}

// one thread: the three boxes of tile t into `stage`, completing on `bar`
__device__ __forceinline__ void issue_tile(const TmaMaps &maps, int4 t, unsigned char *stage, uint32_t bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(3 * BOX_BYTES) : "memory");
  // halo'd coordinates of the box start: interior (i0 - 1, j0 - 1, k0 - 1) is halo'd (i0, j0, k0)
  for (int f = 0; f < 3; f++) {
    const uint64_t map = reinterpret_cast<uint64_t>(&maps.m[t.x][f]);
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(sm32(stage + f * BOX_PITCH)), "l"(map), "r"(t.y), "r"(t.z), "r"(t.w), "r"(bar)
        : "memory");
  }
}

}  // namespace

__global__ void __launch_bounds__(FX * FY) k_fillps_tma(const __grid_constant__ TmaMaps maps,
                                                        const DBlock *__restrict__ Bs, const int4 *__restrict__ tiles,
                                                        int ntiles, double rdt, int fft_axis, int *__restrict__ err) {
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + 2 * STAGE_BYTES);  // two mbarriers after the stages
  const int tid = threadIdx.x, tx = tid % FX, ty = tid / FX;
  // the tiled copies need 128-byte aligned destinations: a misaligned window is reported, nothing is copied
  if (sm32(smem) & 127u) {
    if (tid == 0) atomicExch(err, 2);
    return;
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sm32(&bars[0])), "r"(1));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sm32(&bars[1])), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  uint32_t phase[2] = {0u, 0u};
  int pending[2] = {0, 0};  // copies issued into a stage and not yet waited for
  int stage = 0;
  int t = blockIdx.x;
  if (t < ntiles && tid == 0) issue_tile(maps, tiles[t], smem, sm32(&bars[0]));
  if (t < ntiles) pending[0] = 1;
  bool failed = false;
  for (; t < ntiles; t += gridDim.x) {
    const int tn = t + gridDim.x;
    if (tn < ntiles) {  // the other stage was released by the barrier that ended the previous tile
      if (tid == 0) issue_tile(maps, tiles[tn], smem + (stage ^ 1) * STAGE_BYTES, sm32(&bars[stage ^ 1]));
      pending[stage ^ 1] = 1;
    }
    const bool ok = bar_wait(sm32(&bars[stage]), phase[stage], TMA_POLLS);
    if (!__syncthreads_and(ok ? 1 : 0)) {
      if (tid == 0) atomicExch(err, 1);
      failed = true;
      break;
    }
    pending[stage] = 0;
    phase[stage] ^= 1u;
    const int4 tl = tiles[t];
    const DBlock &B = Bs[tl.x];
    const int nx = B.n[0], ny = B.n[1], nz = B.n[2];
    const double *su = reinterpret_cast<const double *>(smem + stage * STAGE_BYTES);
    const double *sv = su + BOX_PITCH / 8, *sw = sv + BOX_PITCH / 8;
    const int i = tl.y + tx, j = tl.z + ty;
    if (i < nx && j < ny) {
      const double dxf = AX(B, 0, AX_DF, i), dyf = AX(B, 1, AX_DF, j);
      const double xrf = AX(B, 0, AX_RF, i), yrf = AX(B, 1, AX_RF, j);
      for (int z = 0; z < FZ; z++) {
        const int k = tl.w + z;
        if (k >= nz) break;
        const int q = ((z + 1) * BY + (ty + 1)) * BX + (tx + 1);
        const double dwv = sw[q] - sw[q - BX * BY], dvv = sv[q] - sv[q - BX], duv = su[q] - su[q - 1];
        const double dzf = AX(B, 2, AX_DF, k);
        double r;
        switch (fft_axis) {
          case 3: r = fma(dwv * AX(B, 2, AX_RF, k), dxf * dyf, fma(dvv, dxf, duv * dyf)); break;
          case 2: r = fma(dwv, dxf, fma(dvv * yrf, dxf * dzf, duv * dzf)); break;
          case 1: r = fma(dwv, dyf, fma(dvv, dzf, duv * xrf * (dyf * dzf))); break;
          default: r = fma(dwv, dxf * dyf, fma(dvv, dxf * dzf, duv * (dyf * dzf)));
        }
        B.pp[hidx(i, j, k, nx, ny)] = r * rdt;
      }
    }
    __syncthreads();  // the stage is read: it may be refilled
    stage ^= 1;
  }
  if (failed) {  // let the copies in flight land (bounded) before the CTA's shared memory goes away
    for (int s = 0; s < 2; s++)
      if (pending[s]) bar_wait(sm32(&bars[s]), phase[s], TMA_POLLS);
  }
}

// the driver's cuTensorMapEncodeTiled (null when the driver does not provide it)
void *tma_encode_fn() {
  static void *fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return p;
  }();
  return fn;
}

namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(tma_encode_fn());
}

}  // namespace

// Tensor maps of u, v, w of every block and the tile list; d.tma stays null where the tiled copies do not
// apply (the plain kernels run then)
int tma_setup(Domain &d) {
  if (d.tma || d.opt.tma == -1) return SNAC_OK;
  if (d.nblocks > TMA_MAX_BLOCKS) return SNAC_OK;
  for (int b = 0; b < d.nblocks; b++)
    if (d.db[b].n[0] & 1) return SNAC_OK;  // row pitch not a multiple of 16 bytes
  PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
  if (!enc) return SNAC_OK;
  // maps of u, v, w as they are now, and of nu, nv, nw, which become u, v, w after the next momentum stage
  auto maps = new TmaMaps(), alt = new TmaMaps();
  std::vector<int4> tl;
  for (int b = 0; b < d.nblocks; b++) {
    const DBlock &B = d.db[b];
    const cuuint64_t gdim[3] = {(cuuint64_t)B.n[0] + 2, (cuuint64_t)B.n[1] + 2, (cuuint64_t)B.n[2] + 2};
    const cuuint64_t gstr[2] = {gdim[0] * 8, gdim[0] * gdim[1] * 8};
    const cuuint32_t box[3] = {BX, BY, BZ}, estr[3] = {1, 1, 1};
    double *f[2][3] = {{B.u, B.v, B.w}, {B.nu, B.nv, B.nw}};
    for (int s = 0; s < 2; s++)
      for (int q = 0; q < 3; q++) {
        const CUresult r = enc(&(s ? alt : maps)->m[b][q], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, f[s][q], gdim, gstr,
                               box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) {
          delete maps;
          delete alt;
          set_error("cuTensorMapEncodeTiled failed (%d) for block %d field %d", (int)r, b, q);
          return SNAC_ERR_CUDA;
        }
      }
    for (int k = 0; k < B.n[2]; k += FZ)
      for (int j = 0; j < B.n[1]; j += FY)
        for (int i = 0; i < B.n[0]; i += FX) tl.push_back(make_int4(b, i, j, k));
  }
  int4 *dt = (int4 *)d.alloc(tl.size() * sizeof(int4));
  int *derr = (int *)d.alloc(sizeof(int));
  if (!dt || !derr) { delete maps; delete alt; set_error("device allocation failed (TMA tiles)"); return SNAC_ERR_NOMEM; }
  SNAC_CUDA(cudaMemcpy(dt, tl.data(), tl.size() * sizeof(int4), cudaMemcpyHostToDevice));
  int dev = 0, nsm = 0;
  SNAC_CUDA(cudaGetDevice(&dev));
  SNAC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  SNAC_CUDA(cudaFuncSetAttribute((const void *)k_fillps_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, TMA_SMEM));
  d.tma = maps;
  d.tma_alt = alt;
  d.tma_tiles = dt;
  d.tma_ntiles = (int)tl.size();
  d.tma_err = derr;
  d.tma_ctas = std::min(d.tma_ntiles, 3 * nsm);  // 74 KB of stages each: three CTAs per multiprocessor
  return SNAC_OK;
}

void tma_destroy(Domain &d) {
  delete d.tma;
  delete d.tma_alt;
  d.tma = nullptr;
  d.tma_alt = nullptr;
}

// fillps on every block through the TMA-staged kernel; false in *done when it does not apply
int launch_fillps_tma(Domain &d, double dt, int *done) {
  *done = 0;
  if (!d.tma || d.tma_ntiles == 0) return SNAC_OK;
  prof_begin(KID_FILLPS, d.st);
  k_fillps_tma<<<d.tma_ctas, FX * FY, TMA_SMEM, d.st>>>(*d.tma, d.d_db, d.tma_tiles, d.tma_ntiles, 1.0 / dt,
                                                               d.c.fft_axis, d.tma_err), ::snac::count_launch();
  prof_end(KID_FILLPS, d.st);
  SNAC_CUDA(cudaGetLastError());
  *done = 1;
  return SNAC_OK;
}

// the error flag of the TMA kernels (a bounded mbarrier wait that ran out); cleared when read
int tma_check(Domain &d) {
  if (!d.tma_err) return SNAC_OK;
  int e = 0;
  SNAC_CUDA(cudaMemcpyAsync(&e, d.tma_err, sizeof(int), cudaMemcpyDeviceToHost, d.st));
  SNAC_CUDA(cudaStreamSynchronize(d.st));
  if (e) {
    SNAC_CUDA(cudaMemsetAsync(d.tma_err, 0, sizeof(int), d.st));
    if (e == 2) { set_error("TMA-staged kernel: shared-memory window not 128-byte aligned"); return SNAC_ERR_CUDA; }
    set_error("a TMA tile copy did not complete in time");
    return SNAC_ERR_TIMEOUT;
  }
  return SNAC_OK;
}

}  // namespace snac
