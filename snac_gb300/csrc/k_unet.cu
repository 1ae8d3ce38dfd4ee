// k_unet.cu -- the three-level U-Net of the learned initial guess of the 3-D pressure solve.
//
// Network (about 180k parameters, BF16 operands on the tensor cores, FP32 accumulation and masters):
//   E0  conv 3x3x3  16 -> 16, ReLU        (input: channel 0 = residual / RMS, channel 1 = live-cell mask)
//   pool 2x2x2 (mean, zero outside the grid)
//   E1  conv        16 -> 32, ReLU        (half resolution)
//   pool
//   B   conv        32 -> 64, ReLU        (quarter resolution)
//   D1  conv [up(B) 64 | E1 32] -> 32, ReLU   (half resolution; nearest-neighbour upsampling of B)
//   D0  conv [up(D1) 32 | E0 16] -> 16, ReLU  (full resolution)
//   head 1x1x1 16 -> 1 (FP32)
// Every 3x3x3 convolution is one kernel, k_u3_conv, an implicit GEMM on tcgen05 (kind::f16, BF16 operands,
// FP32 accumulation in TMEM): M = 128 cells of one x-row segment (126 of them outputs), N = 3 x the output
// channels (the three x taps of every output channel side by side), K = 16 channels per group; one MMA per
// (dz, dy) row and channel group, so a segment is 9 x groups MMAs.  Activations are BF16 in 16-channel groups,
// each cell's group one 32-byte record, records of consecutive x adjacent.  Lane 0 of a fifth warp stages each
// (segment, group) with one 5-D TMA box (128 records x 3 x 3 rows, 32-byte swizzle, zero fill outside the grid)
// into one of up to four stages, keeps the layer's weights resident in shared memory when they fit (else they
// stream with each stage as a bulk copy), and issues the MMAs.  Two TMEM accumulators alternate per segment:
// the four epilogue warps read one back (tcgen05.ld) while the next segment's MMAs run, add the x-shifted tap
// blocks (rows m, m + 1, m + 2 by warp shuffle, across warps through shared memory), and store bias + ReLU as
// BF16 or the raw sums as FP32.  A skip connection is a second source tensor of the same convolution; an
// upsampled input is materialised first (nearest neighbour).  Every mbarrier wait is bounded; past the bound
// the kernel records an error, waits (bounded) for its copies and MMAs in flight, frees its TMEM and returns.
// Training: the input gradient of a convolution is the same kernel run on the output gradient with the
// transposed, tap-flipped weights; the weight gradients are FP32 reductions over cells on the CUDA cores
// (per-chunk partials summed in a fixed order), Adam updates the FP32 masters.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>

#include "snac_host.h"
#include "snac_mgdev.h"

namespace snac {
namespace u3 {

constexpr int M = 128;                 // cells per segment (the MMA's M)
constexpr int TAPS = 27;
constexpr int NL = 5;                  // convolution layers E0, E1, B, D1, D0
constexpr int CIN[NL] = {16, 16, 32, 96, 48};
constexpr int COUT[NL] = {16, 32, 64, 32, 16};
constexpr long MBAR_POLLS = 1L << 24;
constexpr int DW_TILE = 64;            // cells per tile of the weight-gradient kernel
constexpr long DW_CHUNK = 4096;        // cells per partial of the weight and bias gradients

constexpr int woff(int l) {  // offset of layer l in the parameter vector
  int o = 0;
  for (int j = 0; j < l; j++) o += CIN[j] * COUT[j] * TAPS + COUT[j];
  return o;
}
constexpr int HEAD = woff(NL);         // head: 16 weights then 1 bias
constexpr int NPAR = HEAD + 17;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
// shared-memory matrix descriptor (tcgen05), K-major with the 32-byte swizzle (layout type 6 at bit 61): start
// >> 4, leading-dimension offset unused (16 bytes), stride between 8-row groups >> 4, version 1 at bit 46
__device__ __forceinline__ uint64_t smem_desc_sw32(uint32_t addr, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | (1ull << 16) | ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46) |
         (6ull << 61);
}
// kind::f16 instruction descriptor: FP32 accumulator, BF16 A and B, both K-major, N >> 3, M >> 4
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}
// element offset of (row r, k) in a rows x 16 K-major block of 8x8 core matrices (LBO 128 B, SBO 256 B)
// element offset of (row r, k) in a rows x 16 K-major operand with the 32-byte swizzle: rows 32 bytes apart,
// the two 16-byte halves of rows 4-7 of every 8-row group swapped (address bit 4 ^= bit 7; the block starts on
// a 256-byte boundary)
__host__ __device__ __forceinline__ int sw32_el(int r, int k) { return r * 16 + ((((k >> 3) ^ (r >> 2)) & 1) << 3) + (k & 7); }
// activations: per 16-channel group g, per cell a 32-byte pair of records (channels 0-7 | 8-15); the index of
// the 16-byte record gh = 2 g + h of cell `cell` in a tensor of `tot` cells (all volumes)
__host__ __device__ __forceinline__ long rec16(int gh, long cell, long tot) { return ((long)(gh >> 1) * tot + cell) * 2 + (gh & 1); }

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, long limit) {
  uint32_t done = 0;
  for (long it = 0; it < limit && !done; it++) {
    asm volatile(
        "{\n .reg .pred pw;\n mbarrier.try_wait.parity.shared::cta.b64 pw, [%1], %2;\n selp.u32 %0, 1, 0, pw;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity));
  }
  return done != 0;
}
// one input tensor of a convolution: grouped BF16 records, `groups` 16-channel groups, on grid n (per
// volume), at half the convolution's resolution when up = 1
struct Src {
  const __nv_bfloat16 *p;
  int groups;
  int n[3];
  int up;
};
struct ConvArgs {
  Src s[2];
  int kb;                   // channel groups of the input (sum over the sources)
  int n[3], nb;             // output grid per volume, volumes
  const __nv_bfloat16 *w;   // packed weights [group][tap][N x 16 core layout]
  const float *bias;        // forward: N biases
  __nv_bfloat16 *yb;        // forward output (grouped BF16, bias + ReLU)
  float *yf;                // backward output: planar FP32 [yf_off + n][cell]
  int yf_off;
  int *err;
  long poll_limit;
};

// record (16 bytes = 8 channels) of group g, half h at the fine cell (x, y, z) of volume b, for the source
// that holds group g (the fine coordinates are inside the output grid)
__device__ __forceinline__ const __nv_bfloat16 *src_rec(const ConvArgs &a, int g, int h, int b, int x, int y, int z) {
  const Src &s = g < a.s[0].groups ? a.s[0] : a.s[1];
  const int gs = g < a.s[0].groups ? g : g - a.s[0].groups;
  if (s.up) { x >>= 1; y >>= 1; z >>= 1; }
  const long vol = (long)s.n[0] * s.n[1] * s.n[2];
  const long rec = rec16(2 * gs + h, (long)b * vol + x + (long)s.n[0] * (y + (long)s.n[1] * z), vol * a.nb);
  return s.p + rec * 8;
}

// A operand of a stage: one TMA box of 32-byte cell records (16 channels), 128 cells (the segment's and the one
// before) x 3 x 3 rows, rows ROW bytes apart, written with the 32-byte swizzle; a tap's x offset dx in {0, 1, 2}
// starts its operand dx records later, so of the 128 MMA rows the first MV = 126 are outputs (the last two would
// need records past the box: they read the padding after it and are discarded)
constexpr int MV = M - 2;                              // output cells per segment
constexpr int ROW = M * 32;                            // 4096 bytes
constexpr int ABOX = 9 * ROW;                          // bytes one box writes (36,864)
constexpr int ASTG = ABOX + 1024;                      // with the padding, a multiple of 1024
constexpr int MAXST = 4;                               // stages at most
constexpr int SMEM_LIMIT = 227 * 1024;

struct TmaConv {
  CUtensorMap map[2];       // the sources: 5-D maps of 8-byte units {4 per cell record, x, y, z, group x volume}
  int g0, kb;               // groups of source 0, total groups
  int n[3], nb;             // output grid per volume, volumes (each source has the same grid)
  const __nv_bfloat16 *w;   // packed weights [group][tap][N x 16 core layout]
  const float *bias;        // forward: N biases
  __nv_bfloat16 *yb;        // forward output (grouped BF16, bias + ReLU)
  float *yf;                // input-gradient output: planar FP32 [yf_off + n][cell]
  int yf_off;
  int resw, nst;            // weights resident for the whole launch; pipeline stages
  int *err;
  long poll_limit;
};

// two accumulators of 3 N columns (the x taps dx = 0, 1, 2 of every output channel)
template <int N>
constexpr uint32_t tmem_cols() { return 6 * N <= 128 ? 128u : 6 * N <= 256 ? 256u : 512u; }
__host__ __device__ constexpr int stage_stride(int N, int resw) {
  return resw ? ASTG : ((ASTG + TAPS * N * 32 + 1023) / 1024) * 1024;
}
// the epilogue's exchange area (two segment parities x 4 warps x 3 N floats) after the stages and resident
// weights, the mbarriers after it
__host__ __device__ constexpr int xch_off(int N, int resw, int nst, int kb) {
  return nst * stage_stride(N, resw) + (resw ? kb * TAPS * N * 32 : 0);
}
__host__ __device__ constexpr int bars_off(int N, int resw, int nst, int kb) { return xch_off(N, resw, nst, kb) + 96 * N; }
__host__ constexpr int conv_smem(int N, int resw, int nst, int kb) { return bars_off(N, resw, nst, kb) + 128; }

__device__ __forceinline__ void bar_init(uint64_t *b, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count));
}
__device__ __forceinline__ void bar_expect(uint64_t *b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bar_arrive(uint64_t *b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
// box of cells x.., rows y.., z.. of group x volume w (innermost coordinate 0: the whole 32-byte record)
__device__ __forceinline__ void tma_box(uint32_t dst, const CUtensorMap *map, int x, int y, int z, int w, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], [%7];"
      ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(x), "r"(y), "r"(z), "r"(w), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void bulk_copy(uint32_t dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(dst), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}

// y = conv(x) over nb volumes.  Warps 0-3 read the accumulators back (TMEM lanes 32 w .. 32 w + 31) and store
// them; lane 0 of warp 4 issues the TMA copies of the stages and the MMAs.  FWD writes bias + ReLU as grouped
// BF16, otherwise the raw sums as FP32 planes.
template <int N, bool FWD>
__global__ void __launch_bounds__(160, 1) k_u3_conv(const __grid_constant__ TmaConv a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  constexpr int SB = TAPS * N * 32;
  constexpr uint32_t TC = tmem_cols<N>();
  constexpr uint32_t ACC1 = TC / 2;  // column of the second accumulator
  const int STG = stage_stride(N, a.resw), NST = a.nst;
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + bars_off(N, a.resw, NST, a.kb));
  uint64_t *full = bars, *empty = bars + MAXST, *accf = bars + 2 * MAXST, *acce = bars + 2 * MAXST + 2,
           *wbar = bars + 2 * MAXST + 4;
  uint32_t *tbase = reinterpret_cast<uint32_t *>(bars + 2 * MAXST + 5);
  unsigned char *wres = smem + NST * STG;
  float *xch = reinterpret_cast<float *>(smem + xch_off(N, a.resw, NST, a.kb));
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  // the swizzled copies and operands need a 1024-byte aligned window: a misaligned one is reported, nothing runs
  if (smem_u32(smem) & 1023u) {
    if (t == 0) atomicExch(a.err, 2);
    return;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tbase)), "r"(TC));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (t == 0) {
    for (int q = 0; q < MAXST; q++) { bar_init(&full[q], 1); bar_init(&empty[q], 1); }
    for (int q = 0; q < 2; q++) { bar_init(&accf[q], 1); bar_init(&acce[q], 4); }
    bar_init(wbar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tm = *tbase;
  const int n0 = a.n[0], n1 = a.n[1], n2 = a.n[2];
  const long vol = (long)n0 * n1 * n2, tot = vol * a.nb;
  const int nsx = (n0 + MV - 1) / MV;
  const long total = (long)nsx * n1 * n2 * a.nb;
  const long nloc = (long)blockIdx.x < total ? (total - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  const long T = nloc * a.kb;
  auto seg_of = [&](long k, int &x0, int &y, int &z, int &b) {
    long seg = blockIdx.x + k * gridDim.x;
    x0 = (int)(seg % nsx) * MV; seg /= nsx;
    y = (int)(seg % n1); seg /= n1;
    z = (int)(seg % n2); b = (int)(seg / n2);
  };
  bool ok = true;
  if (warp == 4) {
    if (lane == 0) {
      // producer and MMA issuer.  Per buffer: copies issued / waited, commits issued / waited (for the drain)
      int fiss[MAXST] = {0, 0, 0, 0}, fwt[MAXST] = {0, 0, 0, 0}, eiss[MAXST] = {0, 0, 0, 0}, ewt[MAXST] = {0, 0, 0, 0};
      int wiss = 0;
      if (a.resw && T > 0) {
        bar_expect(wbar, (uint32_t)(a.kb * SB));
        bulk_copy(smem_u32(wres), a.w, (uint32_t)(a.kb * SB), wbar);
        wiss = 1;
      }
      long issued = 0, s = 0;
      auto produce = [&](long u) -> bool {
        const int buf = (int)(u % NST);
        if (eiss[buf] > ewt[buf]) {  // the buffer's previous stage: its MMAs must be done
          if (!mbar_wait(smem_u32(&empty[buf]), (uint32_t)(ewt[buf] & 1), a.poll_limit)) return false;
          ewt[buf]++;
        }
        const int g = (int)(u % a.kb);
        int x0, y, z, b;
        seg_of(u / a.kb, x0, y, z, b);
        unsigned char *A = smem + buf * STG;
        bar_expect(&full[buf], (uint32_t)(ABOX + (a.resw ? 0 : SB)));
        const int src = g < a.g0 ? 0 : 1, gs = g < a.g0 ? g : g - a.g0;
        tma_box(smem_u32(A), &a.map[src], x0 - 1, y - 1, z - 1, gs * a.nb + b, &full[buf]);
        if (!a.resw) bulk_copy(smem_u32(A + ASTG), reinterpret_cast<const unsigned char *>(a.w) + (long)g * SB, SB, &full[buf]);
        fiss[buf]++;
        return true;
      };
      // stages 0 .. NST-2 in flight before the first MMA; then each iteration queues stage s's MMAs before it
      // refills the buffer of stage s-1 (whose MMAs run ahead of them), so the tensor pipe never drains
      while (ok && issued < T && issued < NST - 1) ok = produce(issued++);
      for (s = 0; s < T && ok; s++) {
        const int buf = (int)(s % NST);
        if (!mbar_wait(smem_u32(&full[buf]), (uint32_t)(fwt[buf] & 1), a.poll_limit)) { ok = false; break; }
        fwt[buf]++;
        if (wiss == 1) {
          if (!mbar_wait(smem_u32(wbar), 0u, a.poll_limit)) { ok = false; break; }
          wiss = 2;
        }
        const long k = s / a.kb;
        const int g = (int)(s % a.kb);
        if (g == 0 && k >= 2 && !mbar_wait(smem_u32(&acce[k & 1]), (uint32_t)(((k >> 1) - 1) & 1), a.poll_limit)) {
          ok = false;  // the epilogue of segment k - 2 still holds this accumulator
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        // one MMA per (dz, dy) row r: the row's 128 records (A) times the 3 N rows of its three x taps (B); the
        // x shift of the taps is applied when the accumulator is read back
        constexpr uint32_t idesc = idesc_bf16(M, 3 * N);
        const uint32_t A32 = smem_u32(smem + buf * STG);
        const uint32_t W32 = a.resw ? smem_u32(wres) + g * SB : A32 + ASTG;
        const uint32_t dt = tm + ((k & 1) ? ACC1 : 0u);
#pragma unroll 1
        for (int r = 0; r < 9; r++) {  // r = (dz + 1) * 3 + (dy + 1)
          const uint64_t ad = smem_desc_sw32(A32 + r * ROW, 256);
          const uint64_t bd = smem_desc_sw32(W32 + r * 3 * N * 32, 256);
          const uint32_t acc = (g > 0 || r > 0) ? 1u : 0u;
          asm volatile(
              "{\n .reg .pred pa;\n setp.ne.b32 pa, %4, 0;\n"
              " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, pa;\n}\n" ::"r"(dt),
              "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(&empty[buf])));
        eiss[buf]++;
        if (g == a.kb - 1)
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smem_u32(&accf[k & 1])));
        while (ok && issued < T && issued < s + NST) ok = produce(issued++);
      }
      if (!ok) {
        atomicExch(a.err, 1);
        // drain: every copy issued has landed and every MMA issued has finished before the memory goes away
        for (int q = 0; q < MAXST; q++) {
          while (fwt[q] < fiss[q] && mbar_wait(smem_u32(&full[q]), (uint32_t)(fwt[q] & 1), MBAR_POLLS)) fwt[q]++;
          while (ewt[q] < eiss[q] && mbar_wait(smem_u32(&empty[q]), (uint32_t)(ewt[q] & 1), MBAR_POLLS)) ewt[q]++;
        }
        if (wiss == 1) mbar_wait(smem_u32(wbar), 0u, MBAR_POLLS);
      }
    }
  } else {
    // epilogue warps: one segment at a time, in order, from the accumulator its MMAs filled
    for (long k = 0; k < nloc; k++) {
      const bool got = mbar_wait(smem_u32(&accf[k & 1]), (uint32_t)((k >> 1) & 1), a.poll_limit);
      // the four epilogue warps decide together (their exchange below has a barrier of its own)
      uint32_t any_bad;
      asm volatile(
          "{\n .reg .pred pin, pout;\n setp.ne.u32 pin, %1, 0;\n bar.red.or.pred pout, 1, 128, pin;\n"
          " selp.u32 %0, 1, 0, pout;\n}\n"
          : "=r"(any_bad)
          : "r"(got ? 0u : 1u)
          : "memory");
      if (any_bad) { ok = false; break; }
      asm volatile("tcgen05.fence::after_thread_sync;");
      int x0, y, z, b;
      seg_of(k, x0, y, z, b);
      // accumulator row m = record x0 - 1 + m; columns dx N + c = its product with tap dx of channel c.  Output
      // cell x0 + m sums rows m, m + 1, m + 2 of the dx = 0, 1, 2 blocks: the next lanes' values come by shuffle,
      // those of the next warp's lanes 0 and 1 through shared memory (one exchange per segment)
      const int m = warp * 32 + lane, x = x0 + m;
      const long cell = (long)b * vol + x + (long)n0 * (y + (long)n1 * z);
      const uint32_t col = (k & 1) ? ACC1 : 0u;
      const uint32_t trow = tm + ((uint32_t)(warp * 32) << 16) + col;
      float *xw = xch + ((k & 1) * 4 + warp) * 3 * N;  // this warp's exchange slots: lane 0 dx 1, lane 0 dx 2, lane 1 dx 2
      auto ld16 = [&](uint32_t c, float *v) {
        uint32_t rr[16];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
            : "=r"(rr[0]), "=r"(rr[1]), "=r"(rr[2]), "=r"(rr[3]), "=r"(rr[4]), "=r"(rr[5]), "=r"(rr[6]), "=r"(rr[7]),
              "=r"(rr[8]), "=r"(rr[9]), "=r"(rr[10]), "=r"(rr[11]), "=r"(rr[12]), "=r"(rr[13]), "=r"(rr[14]),
              "=r"(rr[15])
            : "r"(trow + c));
        asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
        for (int e = 0; e < 16; e++) v[e] = __uint_as_float(rr[e]);
      };
#pragma unroll 1
      for (int c16 = 0; c16 < N / 16; c16++) {
        float v1[16], v2[16];
        ld16(N + c16 * 16, v1);
        ld16(2 * N + c16 * 16, v2);
        if (lane == 0)
          for (int e = 0; e < 16; e++) { xw[c16 * 16 + e] = v1[e]; xw[N + c16 * 16 + e] = v2[e]; }
        if (lane == 1)
          for (int e = 0; e < 16; e++) xw[2 * N + c16 * 16 + e] = v2[e];
      }
      asm volatile("bar.sync 1, 128;" ::: "memory");  // the four epilogue warps have published their slots
      const float *xn = xw + 3 * N;                   // the next warp's slots (read by lanes 30 and 31 of warps 0-2)
#pragma unroll 1
      for (int c16 = 0; c16 < N / 16; c16++) {
        float v0[16], v1[16], v2[16];
        ld16(c16 * 16, v0);
        ld16(N + c16 * 16, v1);
        ld16(2 * N + c16 * 16, v2);
        float o[16];
#pragma unroll
        for (int e = 0; e < 16; e++) {
          float s1 = __shfl_down_sync(0xffffffffu, v1[e], 1), s2 = __shfl_down_sync(0xffffffffu, v2[e], 2);
          if (warp < 3 && lane == 31) { s1 = xn[c16 * 16 + e]; s2 = xn[2 * N + c16 * 16 + e]; }
          if (warp < 3 && lane == 30) s2 = xn[N + c16 * 16 + e];
          o[e] = v0[e] + s1 + s2;
        }
        if (m < MV && x < n0) {
          if constexpr (FWD) {
#pragma unroll
            for (int h = 0; h < 2; h++) {
              __align__(16) __nv_bfloat16 ob[8];
#pragma unroll
              for (int e = 0; e < 8; e++) ob[e] = __float2bfloat16(fmaxf(o[h * 8 + e] + a.bias[c16 * 16 + h * 8 + e], 0.f));
              *reinterpret_cast<uint4 *>(a.yb + rec16(2 * c16 + h, cell, tot) * 8) = *reinterpret_cast<const uint4 *>(ob);
            }
          } else {
#pragma unroll
            for (int e = 0; e < 16; e++) a.yf[(long)(a.yf_off + c16 * 16 + e) * tot + cell] = o[e];
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncwarp();
      if (lane == 0) bar_arrive(&acce[k & 1]);  // this warp is done with the accumulator
    }
    if (!ok && lane == 0) atomicExch(a.err, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tm), "r"(TC));
}

// nearest-neighbour upsampling of a grouped BF16 tensor (coarse grid c -> fine grid f), record by record
__global__ void k_u3_upsample(const __nv_bfloat16 *__restrict__ in, int G, int f0, int f1, int f2, int c0, int c1,
                              int c2, int nb, __nv_bfloat16 *__restrict__ out) {
  const long vc = (long)c0 * c1 * c2, vf = (long)f0 * f1 * f2;
  const long total = vf * nb * 2 * G;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const long cell = e % (vf * nb);
    const int gh = (int)(e / (vf * nb));
    const int b = (int)(cell / vf);
    long r = cell % vf;
    const int x = (int)(r % f0); r /= f0;
    const int y = (int)(r % f1), z = (int)(r / f1);
    const long src = rec16(gh, b * vc + (x >> 1) + (long)c0 * ((y >> 1) + (long)c1 * (z >> 1)), vc * nb);
    *reinterpret_cast<uint4 *>(out + rec16(gh, cell, vf * nb) * 8) = *reinterpret_cast<const uint4 *>(in + src * 8);
  }
}

// weights of layer (cin -> cout), FP32 [co][ci][tap], to the packed BF16 blocks of a convolution with N output
// channels: forward (co = n, ci = 16 g + k), or transposed for the input gradient (input channel co = 16 g + k,
// output channel ci = n_off + n, tap mirrored).  Per input group g and (dz, dy) row r one B operand of 3 N rows
// (the three x taps of every output channel) x 16 channels, 32-byte swizzled
__global__ void k_u3_pack(const float *__restrict__ w, int cin, int cout, int trans, int n_off, int N, int kb,
                          __nv_bfloat16 *__restrict__ out) {
  const long total = (long)kb * TAPS * N * 16;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const int k = (int)(e % 16), n = (int)((e / 16) % N), q = (int)((e / (16 * N)) % TAPS), g = (int)(e / (16L * N * TAPS));
    float v;
    if (!trans) v = w[((long)n * cin + g * 16 + k) * TAPS + q];
    else v = w[((long)(g * 16 + k) * cin + n_off + n) * TAPS + (TAPS - 1 - q)];
    // block (g, row r = q / 3) of 3 N rows: row dx N + n holds tap (r, dx = q % 3) of output channel n
    const int r = q / 3, dx = q % 3;
    out[((long)g * 9 + r) * 3 * N * 16 + sw32_el(dx * N + n, k)] = __float2bfloat16(v);
  }
  (void)cout;
}

// mean of the 2x2x2 children (zero outside the fine grid), per record of 8 channels
__global__ void k_u3_pool(const __nv_bfloat16 *__restrict__ in, int G, int f0, int f1, int f2, int c0, int c1, int c2,
                          int nb, __nv_bfloat16 *__restrict__ out) {
  const long vc = (long)c0 * c1 * c2, vf = (long)f0 * f1 * f2;
  const long total = vc * nb * 2 * G;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const long cell = e % (vc * nb);
    const int gh = (int)(e / (vc * nb));
    const int b = (int)(cell / vc);
    long r = cell % vc;
    const int X = (int)(r % c0); r /= c0;
    const int Y = (int)(r % c1), Z = (int)(r / c1);
    float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int dz = 0; dz < 2; dz++)
      for (int dy = 0; dy < 2; dy++)
        for (int dx = 0; dx < 2; dx++) {
          const int x = 2 * X + dx, y = 2 * Y + dy, z = 2 * Z + dz;
          if (x >= f0 || y >= f1 || z >= f2) continue;
          const uint4 v = *reinterpret_cast<const uint4 *>(in + rec16(gh, b * vf + x + (long)f0 * (y + (long)f1 * z), vf * nb) * 8);
          const __nv_bfloat16 *p = reinterpret_cast<const __nv_bfloat16 *>(&v);
#pragma unroll
          for (int c = 0; c < 8; c++) s[c] += __bfloat162float(p[c]);
        }
    __align__(16) __nv_bfloat16 o[8];
#pragma unroll
    for (int c = 0; c < 8; c++) o[c] = __float2bfloat16(s[c] * 0.125f);
    *reinterpret_cast<uint4 *>(out + rec16(gh, cell, vc * nb) * 8) = *reinterpret_cast<const uint4 *>(o);
  }
}

// network input of nb volumes from FP32 planes: channel 0 = r (0 where live = 0), channel 1 = live, rest 0
__global__ void k_u3_input(const float *__restrict__ r, const unsigned char *__restrict__ live, long tot,
                           __nv_bfloat16 *__restrict__ x) {
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < tot; c += (long)gridDim.x * blockDim.x) {
    __align__(16) __nv_bfloat16 o[8];
    const bool l = live[c] != 0;
    o[0] = __float2bfloat16(l ? r[c] : 0.f);
    o[1] = __float2bfloat16(l ? 1.f : 0.f);
#pragma unroll
    for (int e = 2; e < 8; e++) o[e] = __float2bfloat16(0.f);
    *reinterpret_cast<uint4 *>(x + rec16(0, c, tot) * 8) = *reinterpret_cast<const uint4 *>(o);
    *reinterpret_cast<uint4 *>(x + rec16(1, c, tot) * 8) = make_uint4(0u, 0u, 0u, 0u);
  }
}

// head: c = hb + sum_j hw[j] a[j] over the 16 channels of the last layer
__global__ void k_u3_head(const __nv_bfloat16 *__restrict__ a4, long tot, const float *__restrict__ hw,
                          float *__restrict__ c) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < tot; i += (long)gridDim.x * blockDim.x) {
    float acc = hw[16];
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const uint4 v = *reinterpret_cast<const uint4 *>(a4 + rec16(h, i, tot) * 8);
      const __nv_bfloat16 *p = reinterpret_cast<const __nv_bfloat16 *>(&v);
#pragma unroll
      for (int e = 0; e < 8; e++) acc = fmaf(hw[h * 8 + e], __bfloat162float(p[e]), acc);
    }
    c[i] = acc;
  }
}

__device__ __forceinline__ float warp_sum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// loss of nb volumes: L = (1/nb) sum_b sum_live (c - t)^2 / tn_b, and dL/dc (zero at dead cells); one CTA per
// volume and chunk, partial losses per CTA
__global__ void __launch_bounds__(256) k_u3_loss(const float *__restrict__ c, const float *__restrict__ tg,
                                                 const unsigned char *__restrict__ live, const float *__restrict__ tn,
                                                 long vol, int nb, float *__restrict__ dc, float *__restrict__ lpart) {
  const int b = blockIdx.y;
  const float n2 = tn[b];
  const float sc = n2 > 0.f ? 2.f / ((float)nb * n2) : 0.f;
  float acc = 0.f;
  for (long i = blockIdx.x * 256L + threadIdx.x; i < vol; i += (long)gridDim.x * 256) {
    const long j = (long)b * vol + i;
    const float e = live[j] ? c[j] - tg[j] : 0.f;
    dc[j] = sc * e;
    acc += e * e;
  }
  __shared__ float sw[8];
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float s = 0.f;
    for (int w = 0; w < 8; w++) s += sw[w];
    lpart[b * gridDim.x + blockIdx.x] = n2 > 0.f ? s / (n2 * (float)nb) : 0.f;
  }
}

// head backward: dZ4[j] = hw[j] dc (a4[j] > 0) (FP32 planes and grouped BF16); partials of the head's gradient
__global__ void __launch_bounds__(256) k_u3_head_back(const float *__restrict__ dc, const __nv_bfloat16 *__restrict__ a4,
                                                      long tot, const float *__restrict__ hw, float *__restrict__ dz,
                                                      __nv_bfloat16 *__restrict__ dzb, float *__restrict__ part) {
  float acc[17];
#pragma unroll
  for (int j = 0; j < 17; j++) acc[j] = 0.f;
  for (long i = blockIdx.x * 256L + threadIdx.x; i < tot; i += (long)gridDim.x * 256) {
    const float d = dc[i];
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const uint4 v = *reinterpret_cast<const uint4 *>(a4 + rec16(h, i, tot) * 8);
      const __nv_bfloat16 *p = reinterpret_cast<const __nv_bfloat16 *>(&v);
      __align__(16) __nv_bfloat16 o[8];
#pragma unroll
      for (int e = 0; e < 8; e++) {
        const float av = __bfloat162float(p[e]);
        const float g = av > 0.f ? hw[h * 8 + e] * d : 0.f;
        dz[(long)(h * 8 + e) * tot + i] = g;
        o[e] = __float2bfloat16(g);
        acc[h * 8 + e] += d * av;
      }
      *reinterpret_cast<uint4 *>(dzb + rec16(h, i, tot) * 8) = *reinterpret_cast<const uint4 *>(o);
    }
    acc[16] += d;
  }
  __shared__ float sw[8][17];
#pragma unroll
  for (int j = 0; j < 17; j++) {
    const float v = warp_sum(acc[j]);
    if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5][j] = v;
  }
  __syncthreads();
  if (threadIdx.x < 17) {
    float s = 0.f;
    for (int w = 0; w < 8; w++) s += sw[w][threadIdx.x];
    part[blockIdx.x * 17 + threadIdx.x] = s;
  }
}

// out[j] = sum over the nparts rows of part[row * n + j], in row order (fixed-order reduction)
__global__ void k_u3_sum_rows(const float *__restrict__ part, int nparts, int n, float *__restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  float s = 0.f;
  for (int r = 0; r < nparts; r++) s += part[(long)r * n + j];
  out[j] = s;
}

// gradient at a coarse level from the upsampled input's gradient (FP32 planes on the fine grid, channels
// c_off.. c_off + 16 G): sum over the children inside the fine grid, times the ReLU mask of the coarse
// activation; FP32 planes and grouped BF16
__global__ void k_u3_sumchild(const float *__restrict__ gf, int c_off, int G, int f0, int f1, int f2, int c0, int c1,
                              int c2, int nb, const __nv_bfloat16 *__restrict__ act, float *__restrict__ dz,
                              __nv_bfloat16 *__restrict__ dzb) {
  const long vc = (long)c0 * c1 * c2, vf = (long)f0 * f1 * f2, totc = vc * nb, totf = vf * nb;
  const long total = totc * 2 * G;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const long cell = e % totc;
    const int gh = (int)(e / totc);
    const int b = (int)(cell / vc);
    long r = cell % vc;
    const int X = (int)(r % c0); r /= c0;
    const int Y = (int)(r % c1), Z = (int)(r / c1);
    const uint4 av = *reinterpret_cast<const uint4 *>(act + rec16(gh, cell, totc) * 8);
    const __nv_bfloat16 *ap = reinterpret_cast<const __nv_bfloat16 *>(&av);
    __align__(16) __nv_bfloat16 o[8];
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const int ch = gh * 8 + c;
      float s = 0.f;
      for (int kz = 0; kz < 2; kz++)
        for (int ky = 0; ky < 2; ky++)
          for (int kx = 0; kx < 2; kx++) {
            const int x = 2 * X + kx, y = 2 * Y + ky, z = 2 * Z + kz;
            if (x < f0 && y < f1 && z < f2) s += gf[(long)(c_off + ch) * totf + b * vf + x + (long)f0 * (y + (long)f1 * z)];
          }
      const float g = __bfloat162float(ap[c]) > 0.f ? s : 0.f;
      dz[(long)ch * totc + cell] = g;
      o[c] = __float2bfloat16(g);
    }
    *reinterpret_cast<uint4 *>(dzb + rec16(gh, cell, totc) * 8) = *reinterpret_cast<const uint4 *>(o);
  }
}

// gradient of an encoder activation: skip part (FP32 planes, channels s_off..) plus the pooled path's gradient
// (coarse FP32 planes) / 8, times the ReLU mask; FP32 planes and (when dzb) grouped BF16
__global__ void k_u3_skipadd(const float *__restrict__ gs, int s_off, const float *__restrict__ gc, int G, int f0,
                             int f1, int f2, int c0, int c1, int c2, int nb, const __nv_bfloat16 *__restrict__ act,
                             float *__restrict__ dz, __nv_bfloat16 *__restrict__ dzb) {
  const long vc = (long)c0 * c1 * c2, vf = (long)f0 * f1 * f2, totc = vc * nb, totf = vf * nb;
  const long total = totf * 2 * G;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const long cell = e % totf;
    const int gh = (int)(e / totf);
    const int b = (int)(cell / vf);
    long r = cell % vf;
    const int x = (int)(r % f0); r /= f0;
    const int y = (int)(r % f1), z = (int)(r / f1);
    const long par = (long)b * vc + (x >> 1) + (long)c0 * ((y >> 1) + (long)c1 * (z >> 1));
    const uint4 av = *reinterpret_cast<const uint4 *>(act + rec16(gh, cell, totf) * 8);
    const __nv_bfloat16 *ap = reinterpret_cast<const __nv_bfloat16 *>(&av);
    __align__(16) __nv_bfloat16 o[8];
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const int ch = gh * 8 + c;
      const float s = gs[(long)(s_off + ch) * totf + cell] + 0.125f * gc[(long)ch * totc + par];
      const float g = __bfloat162float(ap[c]) > 0.f ? s : 0.f;
      dz[(long)ch * totf + cell] = g;
      o[c] = __float2bfloat16(g);
    }
    if (dzb) *reinterpret_cast<uint4 *>(dzb + rec16(gh, cell, totf) * 8) = *reinterpret_cast<const uint4 *>(o);
  }
}

// weight-gradient partials of one convolution: part[chunk][tap][group][co][ci] = sum over the chunk's cells of
// dZ[co](cell) X[16 group + ci](cell + offset(tap)), X the convolution's input (sources as in the forward)
template <int N>
__global__ void __launch_bounds__(256) k_u3_dw(const __grid_constant__ ConvArgs a, const float *__restrict__ dzp, long chunk,
                                               float *__restrict__ part) {
  __shared__ float sd[N][DW_TILE + 1];
  __shared__ float sx[16][DW_TILE + 1];
  const int q = blockIdx.y, g = blockIdx.z, t = threadIdx.x;
  const int n0 = a.n[0], n1 = a.n[1], n2 = a.n[2];
  const long vol = (long)n0 * n1 * n2, tot = vol * a.nb;
  const int dz = q / 9 - 1, dy = (q / 3) % 3 - 1, dx = q % 3 - 1;
  const long c0 = blockIdx.x * chunk, c1 = min(tot, c0 + chunk);
  constexpr int PP = N * 16 / 256;  // (co, ci) pairs per thread
  float acc[PP];
#pragma unroll
  for (int j = 0; j < PP; j++) acc[j] = 0.f;
  for (long base = c0; base < c1; base += DW_TILE) {
    for (int e = t; e < N * DW_TILE; e += 256) {
      const int co = e / DW_TILE, i = e % DW_TILE;
      sd[co][i] = base + i < c1 ? dzp[(long)co * tot + base + i] : 0.f;
    }
    if (t < 2 * DW_TILE) {
      const int i = t % DW_TILE, h = t / DW_TILE;
      const long cell = base + i;
      float v[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      if (cell < c1) {
        const int b = (int)(cell / vol);
        long r = cell % vol;
        const int x = (int)(r % n0) + dx; r /= n0;
        const int y = (int)(r % n1) + dy, z = (int)(r / n1) + dz;
        if (x >= 0 && x < n0 && y >= 0 && y < n1 && z >= 0 && z < n2) {
          const uint4 u = *reinterpret_cast<const uint4 *>(src_rec(a, g, h, b, x, y, z));
          const __nv_bfloat16 *p = reinterpret_cast<const __nv_bfloat16 *>(&u);
#pragma unroll
          for (int c = 0; c < 8; c++) v[c] = __bfloat162float(p[c]);
        }
      }
#pragma unroll
      for (int c = 0; c < 8; c++) sx[h * 8 + c][i] = v[c];
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < PP; j++) {
      const int p = t + 256 * j, co = p >> 4, ci = p & 15;
      float s = acc[j];
#pragma unroll 16
      for (int i = 0; i < DW_TILE; i++) s = fmaf(sd[co][i], sx[ci][i], s);
      acc[j] = s;
    }
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < PP; j++) part[(((long)blockIdx.x * TAPS + q) * a.kb + g) * N * 16 + t + 256 * j] = acc[j];
}

// weight gradients from the partials, in the master layout [co][ci][tap] (chunks summed in order)
__global__ void k_u3_dw_red(const float *__restrict__ part, int nchunk, int kb, int N, int cin, float *__restrict__ gw) {
  const long total = (long)N * cin * TAPS;
  const long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (e >= total) return;
  const int q = (int)(e % TAPS), ci = (int)((e / TAPS) % cin), co = (int)(e / ((long)TAPS * cin));
  const int g = ci / 16, k = ci % 16;
  float s = 0.f;
  for (int c = 0; c < nchunk; c++) s += part[(((long)c * TAPS + q) * kb + g) * N * 16 + co * 16 + k];
  gw[e] = s;
}

// bias-gradient partials: part[chunk][co] = sum of dZ[co] over the chunk
__global__ void __launch_bounds__(256) k_u3_db(const float *__restrict__ dzp, int N, long tot, long chunk,
                                               float *__restrict__ part) {
  const int co = blockIdx.y;
  const long c0 = blockIdx.x * chunk, c1 = min(tot, c0 + chunk);
  float s = 0.f;
  for (long i = c0 + threadIdx.x; i < c1; i += 256) s += dzp[(long)co * tot + i];
  __shared__ float sw[8];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float r = 0.f;
    for (int w = 0; w < 8; w++) r += sw[w];
    part[(long)blockIdx.x * N + co] = r;
  }
}

__global__ void k_u3_adam(float *__restrict__ w, float *__restrict__ m, float *__restrict__ v,
                          const float *__restrict__ g, int n, float lr, float b1, float b2, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  m[i] = b1 * m[i] + (1.f - b1) * gi;
  v[i] = b2 * v[i] + (1.f - b2) * gi * gi;
  w[i] -= lr * (m[i] / c1) / (sqrtf(v[i] / c2) + 1e-8f);
}

}  // namespace u3

// ---------------------------------------------------------------- host side: the network
using namespace u3;

static long g_u3_poll_limit = u3::MBAR_POLLS;

struct UNet3 {
  float *par = nullptr, *m = nullptr, *v = nullptr, *g = nullptr;
  __nv_bfloat16 *wf = nullptr;      // forward packed weights, layer by layer
  __nv_bfloat16 *wt = nullptr;      // transposed packed weights of E1, B, D1 (two chunks), D0
  long wf_off[NL] = {}, wt_off[NL + 1] = {};
  int adam_t = 0;
  int *err = nullptr;
  // activations for a batch of nb volumes of grid n (capacity in cells per level)
  int n[3][3] = {}, nb = 0;
  long cap[3] = {};
  __nv_bfloat16 *in = nullptr, *a0 = nullptr, *p0 = nullptr, *a1 = nullptr, *p1 = nullptr, *a2 = nullptr,
                *a3 = nullptr, *a4 = nullptr;
  __nv_bfloat16 *u2 = nullptr, *u3 = nullptr;  // B's output upsampled to level 1, D1's to level 0
  float *c = nullptr;
  // training buffers
  float *dc = nullptr, *dz4 = nullptr, *gd0 = nullptr, *dz3 = nullptr, *gd1 = nullptr, *dz2 = nullptr, *gb = nullptr,
        *dz1 = nullptr, *ge1 = nullptr, *dz0 = nullptr, *part = nullptr, *lpart = nullptr;
  __nv_bfloat16 *dz4b = nullptr, *dz3b = nullptr, *dz2b = nullptr, *dz1b = nullptr;
  long part_cap = 0;
  int lparts = 0;
  std::vector<void *> mem;
  void *alloc(size_t bytes) {
    void *p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
    cudaMemset(p, 0, bytes);
    mem.push_back(p);
    return p;
  }
  void release(void *&p) {
    if (!p) return;
    for (auto &q : mem)
      if (q == p) { cudaFree(q); q = nullptr; }
    p = nullptr;
  }
  ~UNet3() { for (void *p : mem) if (p) cudaFree(p); }

  int init(unsigned seed) {
    par = (float *)alloc(NPAR * 4); m = (float *)alloc(NPAR * 4); v = (float *)alloc(NPAR * 4); g = (float *)alloc(NPAR * 4);
    long nf = 0, nt = 0;
    for (int l = 0; l < NL; l++) { wf_off[l] = nf; nf += (long)CIN[l] * COUT[l] * TAPS; }
    for (int l = 1; l < NL; l++) { wt_off[l] = nt; nt += (long)CIN[l] * COUT[l] * TAPS; }
    wf = (__nv_bfloat16 *)alloc(nf * 2);
    wt = (__nv_bfloat16 *)alloc(nt * 2);
    err = (int *)alloc(sizeof(int));
    if (!par || !m || !v || !g || !wf || !wt || !err) { set_error("device allocation failed (U-Net)"); return SNAC_ERR_NOMEM; }
    // He initialisation (fan-in 27 cin), zero biases; the head starts small
    std::mt19937 rng(seed);
    std::normal_distribution<float> nd(0.f, 1.f);
    std::vector<float> h(NPAR, 0.f);
    for (int l = 0; l < NL; l++) {
      const float sc = std::sqrt(2.f / (27.f * (l == 0 ? 2 : CIN[l])));
      for (long i = 0; i < (long)CIN[l] * COUT[l] * TAPS; i++) h[woff(l) + i] = sc * nd(rng);
    }
    for (int j = 0; j < 16; j++) h[HEAD + j] = 0.05f * nd(rng);
    SNAC_CUDA(cudaMemcpy(par, h.data(), NPAR * 4, cudaMemcpyHostToDevice));
    adam_t = 0;
    return SNAC_OK;
  }
  int set_params(const float *hpar) {
    SNAC_CUDA(cudaMemcpy(par, hpar, NPAR * 4, cudaMemcpyHostToDevice));
    SNAC_CUDA(cudaMemset(m, 0, NPAR * 4));
    SNAC_CUDA(cudaMemset(v, 0, NPAR * 4));
    adam_t = 0;
    return SNAC_OK;
  }
  // BF16 packed copies of the current masters (forward, and the transposed ones when training)
  int pack(bool transposed, cudaStream_t st) {
    for (int l = 0; l < NL; l++)
      k_u3_pack<<<64, 256, 0, st>>>(par + woff(l), CIN[l], COUT[l], 0, 0, COUT[l], CIN[l] / 16, wf + wf_off[l]),
          ::snac::count_launch();
    if (transposed)
      for (int l = 1; l < NL; l++) {
        const int nch = CIN[l] > 64 ? 2 : 1, N = CIN[l] / nch;
        for (int ch = 0; ch < nch; ch++)
          k_u3_pack<<<64, 256, 0, st>>>(par + woff(l), CIN[l], COUT[l], 1, ch * N, N, COUT[l] / 16,
                                        wt + wt_off[l] + (long)ch * N * COUT[l] * TAPS), ::snac::count_launch();
      }
    SNAC_CUDA(cudaGetLastError());
    return SNAC_OK;
  }
  static long cells(const int *d) { return (long)d[0] * d[1] * d[2]; }
  long tcap[3] = {};  // capacity of the training buffers (cells per level)
  // buffers for nb volumes of grid n0 (levels: n0, ceil(n0/2), ceil(n0/4)); the training buffers only when
  // training, each set grown to the largest request so far
  int ensure(const int *n0, int nbv, bool training) {
    if (nbv < 1 || nbv > 64) { set_error("U-Net: 1 to 64 volumes per batch"); return SNAC_ERR_ARG; }
    int nn[3][3];
    for (int a = 0; a < 3; a++) { nn[0][a] = n0[a]; nn[1][a] = (n0[a] + 1) / 2; nn[2][a] = (nn[1][a] + 1) / 2; }
    long need[3];
    for (int l = 0; l < 3; l++) need[l] = cells(nn[l]) * nbv;
    if (need[0] > cap[0] || need[1] > cap[1] || need[2] > cap[2]) {
      void **act[] = {(void **)&in, (void **)&a0, (void **)&p0, (void **)&a1, (void **)&p1, (void **)&a2, (void **)&a3,
                      (void **)&a4, (void **)&c, (void **)&u2, (void **)&u3};
      for (void **p : act) release(*p);
      const long c0 = std::max(need[0], cap[0]), c1 = std::max(need[1], cap[1]), c2 = std::max(need[2], cap[2]);
      in = (__nv_bfloat16 *)alloc(c0 * 32); a0 = (__nv_bfloat16 *)alloc(c0 * 32); a4 = (__nv_bfloat16 *)alloc(c0 * 32);
      p0 = (__nv_bfloat16 *)alloc(c1 * 32); a1 = (__nv_bfloat16 *)alloc(c1 * 64); a3 = (__nv_bfloat16 *)alloc(c1 * 64);
      p1 = (__nv_bfloat16 *)alloc(c2 * 64); a2 = (__nv_bfloat16 *)alloc(c2 * 128);
      c = (float *)alloc(c0 * 4);
      u2 = (__nv_bfloat16 *)alloc(c1 * 128); u3 = (__nv_bfloat16 *)alloc(c0 * 64);
      if (!in || !a0 || !a4 || !p0 || !a1 || !a3 || !p1 || !a2 || !c || !u2 || !u3) { set_error("device allocation failed (U-Net activations)"); return SNAC_ERR_NOMEM; }
      cap[0] = c0; cap[1] = c1; cap[2] = c2;
    }
    if (training && (need[0] > tcap[0] || need[1] > tcap[1] || need[2] > tcap[2])) {
      void **tb[] = {(void **)&dc, (void **)&dz4, (void **)&gd0, (void **)&dz3, (void **)&gd1, (void **)&dz2,
                     (void **)&gb, (void **)&dz1, (void **)&ge1, (void **)&dz0, (void **)&dz4b, (void **)&dz3b,
                     (void **)&dz2b, (void **)&dz1b, (void **)&part, (void **)&lpart};
      for (void **p : tb) release(*p);
      const long c0 = std::max(need[0], tcap[0]), c1 = std::max(need[1], tcap[1]), c2 = std::max(need[2], tcap[2]);
      dc = (float *)alloc(c0 * 4); dz4 = (float *)alloc(c0 * 64); gd0 = (float *)alloc(c0 * 192);
      dz3 = (float *)alloc(c1 * 128); gd1 = (float *)alloc(c1 * 384); dz2 = (float *)alloc(c2 * 256);
      gb = (float *)alloc(c2 * 128); dz1 = (float *)alloc(c1 * 128); ge1 = (float *)alloc(c1 * 64);
      dz0 = (float *)alloc(c0 * 64);
      dz4b = (__nv_bfloat16 *)alloc(c0 * 32); dz3b = (__nv_bfloat16 *)alloc(c1 * 64);
      dz2b = (__nv_bfloat16 *)alloc(c2 * 128); dz1b = (__nv_bfloat16 *)alloc(c1 * 64);
      const long nchunk = (c0 + DW_CHUNK - 1) / DW_CHUNK;
      part_cap = std::max<long>(nchunk * TAPS * 6 * 64 * 16, 1024L * 17);
      part = (float *)alloc(part_cap * 4);
      lparts = 64;
      lpart = (float *)alloc((size_t)lparts * 64 * 4);
      if (!dc || !dz4 || !gd0 || !dz3 || !gd1 || !dz2 || !gb || !dz1 || !ge1 || !dz0 || !dz4b || !dz3b || !dz2b ||
          !dz1b || !part || !lpart) { set_error("device allocation failed (U-Net training)"); return SNAC_ERR_NOMEM; }
      tcap[0] = c0; tcap[1] = c1; tcap[2] = c2;
    }
    std::copy(&nn[0][0], &nn[0][0] + 9, &n[0][0]);
    nb = nbv;
    return SNAC_OK;
  }

  // the 5-D tensor map of a grouped BF16 tensor of G groups on level lev, in 8-byte units (four per 32-byte cell
  // record of 16 channels): {record, x, y, z, group x volume}, boxes of 1 record x 128 cells x 3 x 3 x 1 (a
  // segment's rows with the cell before; outside the grid: zeros), written with the 32-byte swizzle
  int encode(CUtensorMap *m, const __nv_bfloat16 *p, int G, int lev) const {
    auto enc = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(tma_encode_fn());
    if (!enc) { set_error("U-Net: cuTensorMapEncodeTiled is not available"); return SNAC_ERR_UNSUPPORTED; }
    const cuuint64_t vol = (cuuint64_t)n[lev][0] * n[lev][1] * n[lev][2];
    const cuuint64_t gdim[5] = {4, (cuuint64_t)n[lev][0], (cuuint64_t)n[lev][1], (cuuint64_t)n[lev][2],
                                (cuuint64_t)(G * nb)};
    const cuuint64_t gstr[4] = {32, 32 * (cuuint64_t)n[lev][0], 32 * (cuuint64_t)n[lev][0] * n[lev][1], 32 * vol};
    const cuuint32_t box[5] = {4, M, 3, 3, 1}, estr[5] = {1, 1, 1, 1, 1};
    const CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_UINT64, 5, const_cast<__nv_bfloat16 *>(p), gdim, gstr, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_32B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) { set_error("U-Net: cuTensorMapEncodeTiled failed (%d)", (int)r); return SNAC_ERR_CUDA; }
    return SNAC_OK;
  }
  // convolution on level lev of the sources (p0: g0 groups, p1: g1 groups, both on level lev)
  template <int N, bool FWD>
  int conv(const __nv_bfloat16 *p0, int g0, const __nv_bfloat16 *p1, int g1, int lev, const __nv_bfloat16 *w,
           const float *bias, __nv_bfloat16 *yb, float *yf, int yf_off, cudaStream_t st) {
    TmaConv a;
    memset(&a, 0, sizeof(a));
    SNAC_TRY(encode(&a.map[0], p0, g0, lev));
    if (p1) SNAC_TRY(encode(&a.map[1], p1, g1, lev));
    a.g0 = g0;
    a.kb = g0 + (p1 ? g1 : 0);
    for (int q = 0; q < 3; q++) a.n[q] = n[lev][q];
    a.nb = nb;
    a.w = w; a.bias = bias; a.yb = yb; a.yf = yf; a.yf_off = yf_off; a.err = err;
    a.poll_limit = g_u3_poll_limit;
    a.resw = conv_smem(N, 1, 2, a.kb) <= SMEM_LIMIT ? 1 : 0;
    a.nst = MAXST;
    while (a.nst > 2 && conv_smem(N, a.resw, a.nst, a.kb) > SMEM_LIMIT) a.nst--;
    const int smem = conv_smem(N, a.resw, a.nst, a.kb);
    if (smem > SMEM_LIMIT) { set_error("U-Net: convolution stages exceed shared memory"); return SNAC_ERR_UNSUPPORTED; }
    static bool attr = false;  // per template instance; the attribute is per function
    if (!attr) {
      SNAC_CUDA(cudaFuncSetAttribute(k_u3_conv<N, FWD>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_LIMIT));
      attr = true;
    }
    int dev = 0, nsm = 0;
    SNAC_CUDA(cudaGetDevice(&dev));
    SNAC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const long total = (long)((a.n[0] + MV - 1) / MV) * a.n[1] * a.n[2] * nb;
    const int grid = (int)std::max<long>(1, std::min<long>(total, nsm));
    k_u3_conv<N, FWD><<<grid, 160, smem, st>>>(a), ::snac::count_launch();
    SNAC_CUDA(cudaGetLastError());
    return SNAC_OK;
  }
  int upsample(const __nv_bfloat16 *x, int G, int lc, __nv_bfloat16 *y, cudaStream_t st) {
    const long total = cells(n[lc - 1]) * nb * 2 * G;
    const int grid = (int)std::min<long>((total + 255) / 256, 8192);
    k_u3_upsample<<<grid, 256, 0, st>>>(x, G, n[lc - 1][0], n[lc - 1][1], n[lc - 1][2], n[lc][0], n[lc][1], n[lc][2], nb,
                                        y), ::snac::count_launch();
    return SNAC_OK;
  }
  Src src(const __nv_bfloat16 *p, int groups, int lev, int up) const {
    Src s;
    s.p = p; s.groups = groups; s.up = up;
    for (int q = 0; q < 3; q++) s.n[q] = n[lev][q];
    return s;
  }
  static Src none() { Src s = {}; return s; }
  int pool(const __nv_bfloat16 *x, int G, int lf, __nv_bfloat16 *y, cudaStream_t st) {
    const long total = cells(n[lf + 1]) * nb * 2 * G;
    const int grid = (int)std::min<long>((total + 255) / 256, 4096);
    k_u3_pool<<<grid, 256, 0, st>>>(x, G, n[lf][0], n[lf][1], n[lf][2], n[lf + 1][0], n[lf + 1][1], n[lf + 1][2], nb, y),
        ::snac::count_launch();
    return SNAC_OK;
  }
  // forward from the BF16 input in `in` to the FP32 head output `c`
  int forward(cudaStream_t st) {
    SNAC_TRY((conv<16, true>(in, 1, nullptr, 0, 0, wf + wf_off[0], par + woff(0) + 16 * 16 * TAPS, a0, nullptr, 0, st)));
    SNAC_TRY(pool(a0, 1, 0, p0, st));
    SNAC_TRY((conv<32, true>(p0, 1, nullptr, 0, 1, wf + wf_off[1], par + woff(1) + 16 * 32 * TAPS, a1, nullptr, 0, st)));
    SNAC_TRY(pool(a1, 2, 1, p1, st));
    SNAC_TRY((conv<64, true>(p1, 2, nullptr, 0, 2, wf + wf_off[2], par + woff(2) + 32 * 64 * TAPS, a2, nullptr, 0, st)));
    SNAC_TRY(upsample(a2, 4, 2, u2, st));
    SNAC_TRY((conv<32, true>(u2, 4, a1, 2, 1, wf + wf_off[3], par + woff(3) + 96 * 32 * TAPS, a3, nullptr, 0, st)));
    SNAC_TRY(upsample(a3, 2, 1, u3, st));
    SNAC_TRY((conv<16, true>(u3, 2, a0, 1, 0, wf + wf_off[4], par + woff(4) + 48 * 16 * TAPS, a4, nullptr, 0, st)));
    const long tot = cells(n[0]) * nb;
    k_u3_head<<<(int)std::min<long>((tot + 255) / 256, 8192), 256, 0, st>>>(a4, tot, par + HEAD, c), ::snac::count_launch();
    SNAC_CUDA(cudaGetLastError());
    return SNAC_OK;
  }
  template <int N>
  int wgrad(int l, const Src &s0, const Src &s1, int lev, const float *dzp, cudaStream_t st) {
    ConvArgs a = {};
    a.s[0] = s0; a.s[1] = s1;
    a.kb = s0.groups + s1.groups;
    for (int q = 0; q < 3; q++) a.n[q] = n[lev][q];
    a.nb = nb;
    const long tot = cells(n[lev]) * nb;
    const int nchunk = (int)((tot + DW_CHUNK - 1) / DW_CHUNK);
    if ((long)nchunk * TAPS * a.kb * N * 16 > part_cap) { set_error("U-Net: gradient partials exceed their buffer"); return SNAC_ERR_STATE; }
    k_u3_dw<N><<<dim3(nchunk, TAPS, a.kb), 256, 0, st>>>(a, dzp, DW_CHUNK, part), ::snac::count_launch();
    const long nw = (long)N * CIN[l] * TAPS;
    k_u3_dw_red<<<(int)((nw + 255) / 256), 256, 0, st>>>(part, nchunk, a.kb, N, CIN[l], g + woff(l)), ::snac::count_launch();
    k_u3_db<<<dim3(nchunk, N), 256, 0, st>>>(dzp, N, tot, DW_CHUNK, part), ::snac::count_launch();
    k_u3_sum_rows<<<1, 64, 0, st>>>(part, nchunk, N, g + woff(l) + (long)N * CIN[l] * TAPS), ::snac::count_launch();
    SNAC_CUDA(cudaGetLastError());
    return SNAC_OK;
  }
  // loss of the batch against the targets tg (FP32, dead cells ignored) with per-volume |t|^2 tn, then the
  // gradients of every parameter into g; the partial losses are left in lpart (lparts per volume)
  int loss_backward(const float *tg, const unsigned char *live, const float *tn, cudaStream_t st) {
    const long v0 = cells(n[0]), t0 = v0 * nb, v1 = cells(n[1]), v2 = cells(n[2]);
    (void)v1; (void)v2;
    k_u3_loss<<<dim3(lparts, nb), 256, 0, st>>>(c, tg, live, tn, v0, nb, dc, lpart), ::snac::count_launch();
    const int hb = (int)std::min<long>((t0 + 255) / 256, 1024);
    k_u3_head_back<<<hb, 256, 0, st>>>(dc, a4, t0, par + HEAD, dz4, dz4b, part), ::snac::count_launch();
    k_u3_sum_rows<<<1, 64, 0, st>>>(part, hb, 17, g + HEAD), ::snac::count_launch();
    // D0: input [up(a3) 2 groups | a0 1 group] at level 0
    SNAC_TRY(wgrad<16>(4, src(a3, 2, 1, 1), src(a0, 1, 0, 0), 0, dz4, st));
    SNAC_TRY((conv<48, false>(dz4b, 1, nullptr, 0, 0, wt + wt_off[4], nullptr, nullptr, gd0, 0, st)));
    auto grid_of = [](long total) { return (int)std::min<long>((total + 255) / 256, 8192); };
    k_u3_sumchild<<<grid_of(cells(n[1]) * nb * 4), 256, 0, st>>>(gd0, 0, 2, n[0][0], n[0][1], n[0][2], n[1][0], n[1][1],
                                                                n[1][2], nb, a3, dz3, dz3b), ::snac::count_launch();
    // D1: input [up(a2) 4 groups | a1 2 groups] at level 1
    SNAC_TRY(wgrad<32>(3, src(a2, 4, 2, 1), src(a1, 2, 1, 0), 1, dz3, st));
    for (int ch = 0; ch < 2; ch++)
      SNAC_TRY((conv<48, false>(dz3b, 2, nullptr, 0, 1, wt + wt_off[3] + (long)ch * 48 * 32 * TAPS, nullptr, nullptr,
                                gd1, ch * 48, st)));
    k_u3_sumchild<<<grid_of(cells(n[2]) * nb * 8), 256, 0, st>>>(gd1, 0, 4, n[1][0], n[1][1], n[1][2], n[2][0], n[2][1],
                                                                n[2][2], nb, a2, dz2, dz2b), ::snac::count_launch();
    // B: input p1 (2 groups) at level 2
    SNAC_TRY(wgrad<64>(2, src(p1, 2, 2, 0), none(), 2, dz2, st));
    SNAC_TRY((conv<32, false>(dz2b, 4, nullptr, 0, 2, wt + wt_off[2], nullptr, nullptr, gb, 0, st)));
    k_u3_skipadd<<<grid_of(cells(n[1]) * nb * 4), 256, 0, st>>>(gd1, 64, gb, 2, n[1][0], n[1][1], n[1][2], n[2][0],
                                                               n[2][1], n[2][2], nb, a1, dz1, dz1b), ::snac::count_launch();
    // E1: input p0 (1 group) at level 1
    SNAC_TRY(wgrad<32>(1, src(p0, 1, 1, 0), none(), 1, dz1, st));
    SNAC_TRY((conv<16, false>(dz1b, 2, nullptr, 0, 1, wt + wt_off[1], nullptr, nullptr, ge1, 0, st)));
    k_u3_skipadd<<<grid_of(cells(n[0]) * nb * 2), 256, 0, st>>>(gd0, 32, ge1, 1, n[0][0], n[0][1], n[0][2], n[1][0],
                                                               n[1][1], n[1][2], nb, a0, dz0, nullptr), ::snac::count_launch();
    // E0: input in (1 group) at level 0
    SNAC_TRY(wgrad<16>(0, src(in, 1, 0, 0), none(), 0, dz0, st));
    SNAC_CUDA(cudaGetLastError());
    return SNAC_OK;
  }
  int adam(float lr, cudaStream_t st) {
    adam_t++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)adam_t), c2 = 1.f - std::pow(b2, (float)adam_t);
    k_u3_adam<<<(NPAR + 255) / 256, 256, 0, st>>>(par, m, v, g, NPAR, lr, b1, b2, c1, c2), ::snac::count_launch();
    SNAC_CUDA(cudaGetLastError());
    return SNAC_OK;
  }
  int check_err() {
    int e = 0;
    SNAC_CUDA(cudaMemcpy(&e, err, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
      SNAC_CUDA(cudaMemset(err, 0, sizeof(int)));
      if (e == 2) { set_error("U-Net: shared-memory window not 1024-byte aligned"); return SNAC_ERR_CUDA; }
      set_error("tensor-core accumulator wait timed out (U-Net)");
      return SNAC_ERR_TIMEOUT;
    }
    return SNAC_OK;
  }
  // host FP32 planes (nb volumes of grid n: r, live as 0/1 floats) into the BF16 input
  int load_input(const float *hx, const int *nn, int nbv, bool training) {
    SNAC_TRY(ensure(nn, nbv, training));
    const long tot = cells(n[0]) * nb;
    float *dr = (float *)alloc(tot * 4);
    unsigned char *dl = (unsigned char *)alloc(tot);
    if (!dr || !dl) { set_error("device allocation failed"); return SNAC_ERR_NOMEM; }
    std::vector<float> r(tot);
    std::vector<unsigned char> l(tot);
    for (int b = 0; b < nb; b++)
      for (long i = 0; i < cells(n[0]); i++) {
        r[b * cells(n[0]) + i] = hx[((long)b * 2) * cells(n[0]) + i];
        l[b * cells(n[0]) + i] = hx[((long)b * 2 + 1) * cells(n[0]) + i] != 0.f;
      }
    SNAC_CUDA(cudaMemcpy(dr, r.data(), tot * 4, cudaMemcpyHostToDevice));
    SNAC_CUDA(cudaMemcpy(dl, l.data(), tot, cudaMemcpyHostToDevice));
    k_u3_input<<<(int)std::min<long>((tot + 255) / 256, 8192), 256>>>(dr, dl, tot, in), ::snac::count_launch();
    SNAC_CUDA(cudaDeviceSynchronize());
    void *pr = dr, *pl = dl;
    release(pr);
    release(pl);
    return SNAC_OK;
  }
};

// ---------------------------------------------------------------- the guess of the 3-D pressure solve
namespace g3 {

constexpr int CROP = 32;     // edge of a recorded training crop (cells)
constexpr int NCROP = 4;     // crops recorded per solve
constexpr int BATCH = 4;     // crops per training step
constexpr int RED = 1024;    // partial sums of the guess's reductions

// r = b - A x on level 0 of the 3-D problem (FP64), zero at dead cells
__global__ void __launch_bounds__(256) k_g3_resid(MgLevelD L, MgGeom G, const double *__restrict__ shift,
                                                  const double *__restrict__ x, const double *__restrict__ b,
                                                  double *__restrict__ r) {
  const long c = blockIdx.x * 256L + threadIdx.x;
  if (c >= L.ncell) return;
  if (L.code[c] & 0x8000) { r[c] = 0.0; return; }
  const int n0 = L.n[0], n1 = L.n[1];
  const int i = (int)(c % n0), j = (int)((c / n0) % n1), k = (int)(c / ((long)n0 * n1));
  const double sh = shift ? shift[0] : 0.0;
  const double acc = offdiag<double>(L, G, [&](int e) { return x[e]; }, (int)c, i, j, k);
  r[c] = b[c] - fmat(diag_of<double>(L, G, sh, (int)c), x[c], acc);
}

// per-CTA partials over the live cells: mode 0 (sum r0^2, count), mode 1 (sum r0 d, sum d^2) with d = r0 - r1
__global__ void __launch_bounds__(256) k_g3_sums(int mode, const double *__restrict__ r0, const double *__restrict__ r1,
                                                 const unsigned short *__restrict__ code, long n,
                                                 double *__restrict__ part) {
  double a = 0.0, b = 0.0;
  for (long c = blockIdx.x * 256L + threadIdx.x; c < n; c += (long)gridDim.x * 256) {
    if (code[c] & 0x8000) continue;
    if (mode == 0) { a += r0[c] * r0[c]; b += 1.0; }
    else { const double d = r0[c] - r1[c]; a += r0[c] * d; b += d * d; }
  }
  double ta, tb;
  block_sum2<double>(a, b, ta, tb);
  if (threadIdx.x == 0) { part[2 * blockIdx.x] = ta; part[2 * blockIdx.x + 1] = tb; }
}

// one warp, fixed order: scal[0] = RMS of r0, scal[1] = |r0|^2 (mode 0); scal[2] = alpha = <r0, d> / <d, d>,
// scal[3] = |r0 - alpha d| / |r0| (mode 1)
__global__ void k_g3_fin(int mode, const double *__restrict__ part, int np, double *__restrict__ scal) {
  double a = 0.0, b = 0.0;
  for (int q = threadIdx.x; q < np; q += 32) { a += part[2 * q]; b += part[2 * q + 1]; }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  if (threadIdx.x) return;
  if (mode == 0) {
    scal[0] = (a > 0.0 && b > 0.0) ? sqrt(a / b) : 0.0;
    scal[1] = a;
  } else {
    const double al = b > 0.0 ? a / b : 0.0, rr = scal[1];
    scal[2] = al;
    scal[3] = rr > 0.0 ? sqrt(fmax(0.0, rr - a * al) / rr) : 1.0;
  }
}

// network input: channel 0 = r / RMS, channel 1 = 1 at live cells (both 0 elsewhere)
__global__ void k_g3_input(const double *__restrict__ r, const unsigned short *__restrict__ code,
                           const double *__restrict__ scal, long n, __nv_bfloat16 *__restrict__ x) {
  const double m = scal[0];
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n; c += (long)gridDim.x * blockDim.x) {
    const bool live = m > 0.0 && !(code[c] & 0x8000);
    __align__(16) __nv_bfloat16 o[8];
    o[0] = __float2bfloat16(live ? (float)(r[c] / m) : 0.f);
    o[1] = __float2bfloat16(live ? 1.f : 0.f);
#pragma unroll
    for (int e = 2; e < 8; e++) o[e] = __float2bfloat16(0.f);
    *reinterpret_cast<uint4 *>(x + rec16(0, c, n) * 8) = *reinterpret_cast<const uint4 *>(o);
    *reinterpret_cast<uint4 *>(x + rec16(1, c, n) * 8) = make_uint4(0u, 0u, 0u, 0u);
  }
}

// correction RMS * net / D at live cells (D the operator's diagonal) and the trial x = x_prev + correction
__global__ void __launch_bounds__(256) k_g3_corr(const float *__restrict__ cn, MgLevelD L, MgGeom G,
                                                 const double *__restrict__ shift, const double *__restrict__ scal,
                                                 const double *__restrict__ xprev, double *__restrict__ corr,
                                                 double *__restrict__ x) {
  const long c = blockIdx.x * 256L + threadIdx.x;
  if (c >= L.ncell) return;
  double v = 0.0;
  if (!(L.code[c] & 0x8000) && scal[0] > 0.0) v = scal[0] * (double)cn[c] / diag_of<double>(L, G, shift ? shift[0] : 0.0, (int)c);
  corr[c] = v;
  x[c] = xprev[c] + v;
}

__global__ void k_g3_update(const double *__restrict__ xprev, const double *__restrict__ corr,
                            const double *__restrict__ scal, long n, double *__restrict__ x) {
  const double al = scal[2];
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n; c += (long)gridDim.x * blockDim.x)
    x[c] = fmat(al, corr[c], xprev[c]);
}

struct Crops {
  int o[NCROP][3];
  int slot[NCROP];
};

// one CTA per crop: the normalised residual, the live mask and the target D (x - x_prev) / RMS of the crop
// into its ring slot, with the target's squared norm
__global__ void __launch_bounds__(256) k_g3_record(Crops cr, int e0, int e1, int e2, MgLevelD L, MgGeom G,
                                                   const double *__restrict__ shift, const double *__restrict__ r,
                                                   const double *__restrict__ x, const double *__restrict__ xprev,
                                                   const double *__restrict__ scal, float *__restrict__ rec_r,
                                                   unsigned char *__restrict__ rec_live, float *__restrict__ rec_t,
                                                   float *__restrict__ rec_tn) {
  const int q = blockIdx.x;
  const long cc = (long)e0 * e1 * e2, base = (long)cr.slot[q] * cc;
  const double m = scal[0], sh = shift ? shift[0] : 0.0;
  double acc = 0.0;
  for (long e = threadIdx.x; e < cc; e += blockDim.x) {
    const int i = cr.o[q][0] + (int)(e % e0), j = cr.o[q][1] + (int)((e / e0) % e1), k = cr.o[q][2] + (int)(e / ((long)e0 * e1));
    const long c = i + (long)L.n[0] * (j + (long)L.n[1] * k);
    const bool live = m > 0.0 && !(L.code[c] & 0x8000);
    float rv = 0.f, tv = 0.f;
    if (live) {
      rv = (float)(r[c] / m);
      tv = (float)((x[c] - xprev[c]) * diag_of<double>(L, G, sh, (int)c) / m);
    }
    rec_r[base + e] = rv;
    rec_live[base + e] = live ? 1 : 0;
    rec_t[base + e] = tv;
    acc += (double)tv * tv;
  }
  const double t = block_sum1<double>(acc);
  if (threadIdx.x == 0) rec_tn[cr.slot[q]] = (float)t;
}

}  // namespace g3

struct Guess3 {
  UNet3 net;
  bool net_init = false;
  int n[3] = {}, crop[3] = {};
  long ncell = 0, ccell = 0;
  double *r = nullptr, *xprev = nullptr, *r1 = nullptr, *corr = nullptr, *part = nullptr, *scal = nullptr;
  float *rec_r = nullptr, *rec_t = nullptr, *rec_tn = nullptr, *bt_r = nullptr, *bt_t = nullptr, *bt_tn = nullptr;
  unsigned char *rec_live = nullptr, *bt_live = nullptr;
  int cap = 2048, count = 0, next = 0;
  bool packed = false;  // the forward weights match the masters
  std::mt19937 rng{4242};
  std::vector<void *> mem;
  void *alloc(size_t bytes) {
    void *p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
    cudaMemset(p, 0, bytes);
    mem.push_back(p);
    return p;
  }
  ~Guess3() { for (void *p : mem) cudaFree(p); }
};

Guess3 *guess3_create() { return new Guess3(); }
void guess3_destroy(Guess3 *g) { delete g; }

static int guess3_setup(const PoissonSolver &S, Guess3 &g) {
  if (g.r) return SNAC_OK;
  const MgLevelD &L = S.P.L[0];
  for (int a = 0; a < 3; a++) { g.n[a] = L.n[a]; g.crop[a] = std::min(g3::CROP, L.n[a]); }
  g.ncell = L.ncell;
  g.ccell = (long)g.crop[0] * g.crop[1] * g.crop[2];
  g.r = (double *)g.alloc(g.ncell * 8); g.xprev = (double *)g.alloc(g.ncell * 8);
  g.r1 = (double *)g.alloc(g.ncell * 8); g.corr = (double *)g.alloc(g.ncell * 8);
  g.part = (double *)g.alloc(2 * g3::RED * 8); g.scal = (double *)g.alloc(8 * 8);
  g.rec_r = (float *)g.alloc((size_t)g.cap * g.ccell * 4); g.rec_t = (float *)g.alloc((size_t)g.cap * g.ccell * 4);
  g.rec_live = (unsigned char *)g.alloc((size_t)g.cap * g.ccell); g.rec_tn = (float *)g.alloc(g.cap * 4);
  g.bt_r = (float *)g.alloc(g3::BATCH * g.ccell * 4); g.bt_t = (float *)g.alloc(g3::BATCH * g.ccell * 4);
  g.bt_live = (unsigned char *)g.alloc(g3::BATCH * g.ccell); g.bt_tn = (float *)g.alloc(g3::BATCH * 4);
  if (!g.r || !g.xprev || !g.r1 || !g.corr || !g.part || !g.scal || !g.rec_r || !g.rec_t || !g.rec_live || !g.rec_tn ||
      !g.bt_r || !g.bt_t || !g.bt_live || !g.bt_tn) {
    set_error("device allocation failed (learned guess, 3-D)");
    return SNAC_ERR_NOMEM;
  }
  if (!g.net_init) { SNAC_TRY(g.net.init(11)); g.net_init = true; }
  return SNAC_OK;
}

static MgGeom geom3(const MgProblem &P) {
  MgGeom G;
  G.mode3d = P.mode3d;
  for (int a = 0; a < 3; a++) G.periodic[a] = P.periodic[a];
  return G;
}

static int guess3_sums(Guess3 &g, const MgProblem &P, int mode, cudaStream_t st) {
  const int np = (int)std::min<long>(g3::RED, (g.ncell + 255) / 256);
  g3::k_g3_sums<<<np, 256, 0, st>>>(mode, g.r, g.r1, P.L[0].code, g.ncell, g.part), ::snac::count_launch();
  g3::k_g3_fin<<<1, 32, 0, st>>>(mode, g.part, np, g.scal), ::snac::count_launch();
  return SNAC_OK;
}

// before the 3-D solve: r0 = b - A x_prev and its RMS; mode 2 moves x_prev by the network's correction with the
// step that minimises the residual
int guess3_before(PoissonSolver &S, Guess3 &g, int mode, int measure, double *ratio, cudaStream_t st) {
  SNAC_TRY(guess3_setup(S, g));
  const MgProblem &P = S.P;
  const MgLevelD &L = P.L[0];
  const MgGeom G = geom3(P);
  const unsigned gb = (unsigned)((g.ncell + 255) / 256);
  g3::k_g3_resid<<<gb, 256, 0, st>>>(L, G, P.shift, S.box_x, S.box_b, g.r), ::snac::count_launch();
  SNAC_CUDA(cudaMemcpyAsync(g.xprev, S.box_x, g.ncell * 8, cudaMemcpyDeviceToDevice, st));
  SNAC_TRY(guess3_sums(g, P, 0, st));
  if (mode == 2) {
    SNAC_TRY(g.net.ensure(g.n, 1, false));
    if (!g.packed) { SNAC_TRY(g.net.pack(false, st)); g.packed = true; }
    g3::k_g3_input<<<(int)std::min<long>(gb, 8192), 256, 0, st>>>(g.r, L.code, g.scal, g.ncell, g.net.in), ::snac::count_launch();
    SNAC_TRY(g.net.forward(st));
    g3::k_g3_corr<<<gb, 256, 0, st>>>(g.net.c, L, G, P.shift, g.scal, g.xprev, g.corr, S.box_x), ::snac::count_launch();
    g3::k_g3_resid<<<gb, 256, 0, st>>>(L, G, P.shift, S.box_x, S.box_b, g.r1), ::snac::count_launch();
    SNAC_TRY(guess3_sums(g, P, 1, st));
    g3::k_g3_update<<<(int)std::min<long>(gb, 8192), 256, 0, st>>>(g.xprev, g.corr, g.scal, g.ncell, S.box_x), ::snac::count_launch();
    if (measure) {
      double sc[4];
      SNAC_CUDA(cudaMemcpyAsync(sc, g.scal, sizeof(sc), cudaMemcpyDeviceToHost, st));
      SNAC_CUDA(cudaStreamSynchronize(st));
      SNAC_TRY(g.net.check_err());
      if (ratio) *ratio = sc[3];
    }
  }
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

// after the 3-D solve (mode 1): NCROP random crops of (r0 / RMS, live, D (x - x_prev) / RMS) into the ring
int guess3_after(PoissonSolver &S, Guess3 &g, cudaStream_t st) {
  const MgProblem &P = S.P;
  g3::Crops cr = {};
  for (int q = 0; q < g3::NCROP; q++) {
    for (int a = 0; a < 3; a++) {
      std::uniform_int_distribution<int> pos(0, g.n[a] - g.crop[a]);
      cr.o[q][a] = pos(g.rng);
    }
    cr.slot[q] = g.next;
    g.next = (g.next + 1) % g.cap;
  }
  g3::k_g3_record<<<g3::NCROP, 256, 0, st>>>(cr, g.crop[0], g.crop[1], g.crop[2], P.L[0], geom3(P), P.shift, g.r, S.box_x,
                                             g.xprev, g.scal, g.rec_r, g.rec_live, g.rec_t, g.rec_tn), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  g.count = std::min(g.cap, g.count + g3::NCROP);
  return SNAC_OK;
}

// iters Adam steps on batches of BATCH recorded crops
int guess3_train(Guess3 &g, int iters, double lr, double *loss_first, double *loss_last, int *pairs, cudaStream_t st) {
  if (g.count == 0) { set_error("snac_guess_train: no recorded pairs"); return SNAC_ERR_STATE; }
  SNAC_TRY(g.net.ensure(g.crop, g3::BATCH, true));
  std::uniform_int_distribution<int> pick(0, g.count - 1);
  const int avg = std::min(10, std::max(1, iters / 2));
  double lf = 0.0, ll = 0.0;
  int nf = 0, nl = 0;
  std::vector<float> lp((size_t)g.net.lparts * g3::BATCH);
  const long cc = g.ccell;
  for (int it = 0; it < iters; it++) {
    for (int b = 0; b < g3::BATCH; b++) {
      const long s = pick(g.rng);
      SNAC_CUDA(cudaMemcpyAsync(g.bt_r + b * cc, g.rec_r + s * cc, cc * 4, cudaMemcpyDeviceToDevice, st));
      SNAC_CUDA(cudaMemcpyAsync(g.bt_t + b * cc, g.rec_t + s * cc, cc * 4, cudaMemcpyDeviceToDevice, st));
      SNAC_CUDA(cudaMemcpyAsync(g.bt_live + b * cc, g.rec_live + s * cc, cc, cudaMemcpyDeviceToDevice, st));
      SNAC_CUDA(cudaMemcpyAsync(g.bt_tn + b, g.rec_tn + s, 4, cudaMemcpyDeviceToDevice, st));
    }
    const long tot = cc * g3::BATCH;
    k_u3_input<<<(int)std::min<long>((tot + 255) / 256, 8192), 256, 0, st>>>(g.bt_r, g.bt_live, tot, g.net.in), ::snac::count_launch();
    SNAC_TRY(g.net.pack(true, st));
    SNAC_TRY(g.net.forward(st));
    SNAC_TRY(g.net.loss_backward(g.bt_t, g.bt_live, g.bt_tn, st));
    SNAC_TRY(g.net.adam((float)lr, st));
    if (it < avg || it >= iters - avg) {
      SNAC_CUDA(cudaMemcpyAsync(lp.data(), g.net.lpart, lp.size() * 4, cudaMemcpyDeviceToHost, st));
      SNAC_CUDA(cudaStreamSynchronize(st));
      double L = 0.0;
      for (float v : lp) L += v;
      if (it < avg) { lf += L; nf++; }
      if (it >= iters - avg) { ll += L; nl++; }
    }
  }
  g.packed = false;
  SNAC_CUDA(cudaStreamSynchronize(st));
  SNAC_TRY(g.net.check_err());
  if (loss_first) *loss_first = nf ? lf / nf : 0.0;
  if (loss_last) *loss_last = nl ? ll / nl : 0.0;
  if (pairs) *pairs = g.count;
  return SNAC_OK;
}

}  // namespace snac

using namespace snac;

int snac_unet_nparams(void) { return u3::NPAR; }

int snac_unet_set_poll_limit(long polls) {
  snac::g_u3_poll_limit = polls < 0 ? u3::MBAR_POLLS : polls;
  return SNAC_OK;
}

// forward of the network on host data: x nb x 2 x n2 x n1 x n0 (residual, live mask), params NPAR; out nb x n
int snac_unet_forward(const float *x, int nb, int n0, int n1, int n2, const float *params, float *out) {
  if (!x || !params || !out || nb < 1 || n0 < 1 || n1 < 1 || n2 < 1) { set_error("snac_unet_forward: bad argument"); return SNAC_ERR_ARG; }
  UNet3 net;
  SNAC_TRY(net.init(1));
  SNAC_TRY(net.set_params(params));
  const int nn[3] = {n0, n1, n2};
  SNAC_TRY(net.load_input(x, nn, nb, false));
  SNAC_TRY(net.pack(false, 0));
  SNAC_TRY(net.forward(0));
  SNAC_CUDA(cudaDeviceSynchronize());
  SNAC_TRY(net.check_err());
  SNAC_CUDA(cudaMemcpy(out, net.c, (size_t)nb * n0 * n1 * n2 * 4, cudaMemcpyDeviceToHost));
  return SNAC_OK;
}

// loss and gradients on host data (the gradient check): x as in snac_unet_forward, target nb x n (FP32, cells
// with live = 0 ignored); grads NPAR
int snac_unet_grad(const float *x, const float *target, int nb, int n0, int n1, int n2, const float *params,
                   float *grads, double *loss) {
  if (!x || !target || !params || !grads || nb < 1 || n0 < 1 || n1 < 1 || n2 < 1) { set_error("snac_unet_grad: bad argument"); return SNAC_ERR_ARG; }
  UNet3 net;
  SNAC_TRY(net.init(1));
  SNAC_TRY(net.set_params(params));
  const int nn[3] = {n0, n1, n2};
  SNAC_TRY(net.load_input(x, nn, nb, true));
  const long vol = (long)n0 * n1 * n2, tot = vol * nb;
  float *tg = (float *)net.alloc(tot * 4), *tn = (float *)net.alloc(nb * 4);
  unsigned char *live = (unsigned char *)net.alloc(tot);
  if (!tg || !tn || !live) { set_error("device allocation failed"); return SNAC_ERR_NOMEM; }
  std::vector<unsigned char> l(tot);
  std::vector<float> tnh(nb, 0.f);
  for (int b = 0; b < nb; b++)
    for (long i = 0; i < vol; i++) {
      l[b * vol + i] = x[((long)b * 2 + 1) * vol + i] != 0.f;
      if (l[b * vol + i]) tnh[b] += target[b * vol + i] * target[b * vol + i];
    }
  SNAC_CUDA(cudaMemcpy(tg, target, tot * 4, cudaMemcpyHostToDevice));
  SNAC_CUDA(cudaMemcpy(live, l.data(), tot, cudaMemcpyHostToDevice));
  SNAC_CUDA(cudaMemcpy(tn, tnh.data(), nb * 4, cudaMemcpyHostToDevice));
  SNAC_TRY(net.pack(true, 0));
  SNAC_TRY(net.forward(0));
  SNAC_TRY(net.loss_backward(tg, live, tn, 0));
  SNAC_CUDA(cudaDeviceSynchronize());
  SNAC_TRY(net.check_err());
  SNAC_CUDA(cudaMemcpy(grads, net.g, u3::NPAR * 4, cudaMemcpyDeviceToHost));
  std::vector<float> lp((size_t)net.lparts * nb);
  SNAC_CUDA(cudaMemcpy(lp.data(), net.lpart, lp.size() * 4, cudaMemcpyDeviceToHost));
  double L = 0.0;
  for (float v : lp) L += v;
  if (loss) *loss = L;
  return SNAC_OK;
}
