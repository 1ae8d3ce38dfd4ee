// k_mg_fused.cu -- fused multigrid kernels for the plane (2-D) systems.
//
// k_rbgs_tile2d: all 2*nu red-black half-sweeps of one plane level in one launch.
//   A CTA of 8 warps owns a 64 x 8R tile (a halo of TH = 4 cells on every side
//   around its 56 x (8R - 8) output cells).  Lane l of warp w owns the column
//   pair (2l, 2l+1) of rows w, w+8, ..., so in every half-sweep each thread
//   updates exactly one cell per row and no lane idles.  The tile lives in
//   shared memory split into even and odd columns (conflict-free neighbour
//   reads); b, 1/d and the four couplings of the owned cells stay in registers
//   for all sweeps.  After t half-sweeps only cells within t of the tile edge
//   can differ from a global sweep, so the output cells are exact after TH.
//   The pre-smoother starts from x = 0 without reading x; the post-smoother adds
//   the coarse-grid correction while loading (prolongation fused) and can emit
//   the partials of b.x (r.z of the Krylov iteration), one per warp.  Tiles overlap, so a
//   launch never reads the array it writes: the pre-smoother writes xp and the
//   post-smoother reads xp + correction and writes x.  The pre-smoother can also form the residual of its
//   output cells and restrict it to the next level (mode 2): from a zero start the first half-sweep is exact
//   everywhere in the tile (the cells outside it are still zero too), so after t half-sweeps only cells
//   within t - 1 of the tile edge differ from a global sweep and the neighbours of the output cells are
//   exact as well.  The children of a coarse cell (even-aligned pairs) always lie in one tile: along x they
//   are a thread's own column pair, along y the rows of warps w and w + 1, whose odd warp hands its residuals
//   over in shared memory; so the separate residual-restriction pass over the level goes away.  The first
//   half-sweep of a pre-smoother (zero neighbours) is done while its inputs are loaded.
// k_vcycle_coarse: one CTA of 1024 threads per system runs the V-cycle from
//   level l0 down to the coarsest solve and back, with x, b and 1/d of every
//   level in shared memory, and the couplings too where they fit (the top
//   level's may stay in global memory, shared by all systems and held in L2).
// Both follow the arithmetic of k_rbgs / k_resid_restrict / k_prolong / k_dense
// term by term, so fused and unfused V-cycles give identical results.
#include <algorithm>
#include <cstdlib>
#include <mutex>
#include <type_traits>
#include <utility>
#include <vector>

#include "snac_solver.h"
#include "snac_mgk.h"
#include "snac_mgdev.h"
#include "snac_prof.h"

namespace snac {

namespace {
constexpr int TH = 4;              // tile halo = most half-sweeps per launch (2 nu with nu <= 2)
constexpr int TSW = 64;            // tile width
// tile shapes: NW warps x R rows per warp = tile height SH (output rows SH - 2 TH)
struct TileShape { int nw, r; };
const TileShape SHAPES_F[] = {{8, 2}, {8, 3}, {16, 2}, {16, 3}, {8, 4}, {16, 4}};  // snac_options.mg_tile 1..6
constexpr int NSHAPES_F = 6;
const TileShape SHAPES_D[] = {{8, 2}};
constexpr int TBX = TSW - 2 * TH;  // output columns per tile
inline int tile_by(TileShape t) { return t.nw * t.r - 2 * TH; }
inline int tiles_for(const MgLevelD &L, TileShape t) {
  return ((L.n[0] + TBX - 1) / TBX) * ((L.n[1] + tile_by(t) - 1) / tile_by(t));
}
// the shape given by `pref` (1..6, FP32 only), else the one that processes the fewest tile rows (ties: the
// smaller tile), rows of the three-row shapes counted twice: they need more than 64 registers a thread, which
// halves the warps a multiprocessor holds (channel level 2, 256 x 36: 16 x 3 tiles sweep 48 rows, 16 x 2 tiles
// 64, and the step takes 17.05 against 16.52 ms)
TileShape choose_shape(const MgLevelD &L, int prec, int pref) {
  if (!prec && pref >= 1 && pref <= NSHAPES_F) return SHAPES_F[pref - 1];
  const TileShape *opts = prec ? SHAPES_D : SHAPES_F;
  const int nopt = prec ? 1 : 4;  // the default choice among the first four (the 4-row shapes are tuning options)
  TileShape best = opts[0];
  long bestc = -1;
  for (int q = 0; q < nopt; q++) {
    const TileShape t = opts[q];
    const long cost = (long)((L.n[1] + tile_by(t) - 1) / tile_by(t)) * t.nw * t.r * (t.r >= 3 ? 2 : 1);
    if (bestc < 0 || cost < bestc) { bestc = cost; best = t; }
  }
  return best;
}
__device__ __forceinline__ int wrap(int g, int n) {
  if (g >= 0 && g < n) return g;
  g %= n;
  return g < 0 ? g + n : g;
}
}  // namespace

// partial sums per system written by the post-smoother: one per warp of every tile, over all tile shapes
// the FP32 tile shape level l of P uses, as snac_options.mg_tile (1..4)
int tile2d_shape_index(const MgProblem &P, int l) {
  const TileShape t = choose_shape(P.L[l], 0, P.tile_shape);
  for (int q = 0; q < NSHAPES_F; q++)
    if (SHAPES_F[q].nw == t.nw && SHAPES_F[q].r == t.r) return q + 1;
  return 0;
}

int tile2d_max_parts(const MgLevelD &L) {
  int m = 0;
  for (const TileShape &t : SHAPES_F) m = std::max(m, tiles_for(L, t) * t.nw);
  for (const TileShape &t : SHAPES_D) m = std::max(m, tiles_for(L, t) * t.nw);
  return m;
}

bool tile2d_geometry_ok(const MgProblem &P, int l) {
  if (P.mode3d || l >= P.nlev - 1 || 2 * mg_nu(P, l) > TH) return false;
  const MgLevelD &L = P.L[l];
  if (L.n[0] & 1) return false;  // column pairs are copied as one aligned unit
  for (int a = 0; a < 2; a++)
    if (P.periodic[a] && L.n[a] > 1 && (L.n[a] & 1)) return false;  // red-black colouring must wrap consistently
  return true;
}

bool tile2d_ok(const MgProblem &P, int l, int prec) {
  (void)prec;
  if (!tile2d_geometry_ok(P, l)) return false;
  const MgLevelD &L = P.L[l];
  return L.xp && L.xpf && L.invd && L.invdf;
}

// shared-memory row of the even/odd x tile: 32 column pairs plus a zero pad on each side, so that the
// edge lanes read a zero neighbour instead of testing their lane
constexpr int TRS = 34;

// dynamic shared memory of one tile CTA: the even/odd x tile (SH rows plus a zero pad row above and
// below), two stages of the staged inputs (b and 1/d; in mode 1 also the pre-smoothed x and the coarse
// correction), [stage][array][row][64], and in mode 2 the residuals the odd warps hand over (SH 64 entries)
// and the owned cells' cc and w01, [2][2R][thread] (2 SH 64 entries)
template <typename T>
inline size_t tile_smem_bytes(int sh, int mode) {
  return (2 * (size_t)(sh + 2) * TRS + 2 * (size_t)(mode == 1 ? 4 : 2) * sh * 64 + (mode == 2 ? 3 * (size_t)sh * 64 : 0)) *
         sizeof(T);
}

// Every per-cell address, mask and coupling is set up once per CTA and reused for all its systems.  The
// cells on the tile's outermost ring are updated with zero neighbours from the pads; like any cell within
// TH of the tile edge they may differ from a global sweep, and none of them is stored.
template <typename T, int NW, int R, int MODE>
__device__ __forceinline__ void rbgs_tile2d(MgLevelD L, MgLevelD C, int per0, int per1, const int *__restrict__ active,
                                            int nsys, int sb, int first_color, int nhalf, T *__restrict__ x,
                                            const T *__restrict__ b, const T *__restrict__ xin,
                                            const T *__restrict__ xc, double *__restrict__ part_bx,
                                            const int *__restrict__ singular, double *__restrict__ part_x,
                                            double *__restrict__ part_b, int part_stride, const T *__restrict__ shift,
                                            int inv_inline, T *__restrict__ bco, T *__restrict__ xcz) {
  static_assert(NW % 2 == 0, "rows w + NW q of a thread must share their colour parity");
  using V2 = typename std::conditional<sizeof(T) == 4, float2, double2>::type;
  constexpr int SH = NW * R, BY = SH - 2 * TH;
  static_assert(TBX % 2 == 0 && TH % 2 == 0 && BY % 2 == 0, "coarse cells must not straddle tiles");
  constexpr int NA = MODE == 1 ? 4 : 2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *const xe = reinterpret_cast<T *>(smem_raw);  // [SH + 2][TRS], tile row r at r + 1, pair l at l + 1
  T *const xo = xe + (SH + 2) * TRS;
  T *const stg = xo + (SH + 2) * TRS;
  T *const res = stg + 2 * NA * SH * 64;          // mode 2: residuals handed from odd to even warps
  T *const dtab = res + SH * 64;                  // mode 2: cc, w01 of the owned cells, [2][2R][thread]
  const int n0 = L.n[0], n1 = L.n[1];
  const int ntx = (n0 + TBX - 1) / TBX;
  const int i0 = (int)(blockIdx.x % ntx) * TBX - TH, j0 = (int)(blockIdx.x / ntx) * BY - TH;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const bool skip0 = per0 && n0 == 1, skip1 = per1 && n1 == 1;
  for (int e = threadIdx.x; e < 2 * (SH + 2) * TRS; e += NW * 32) xe[e] = T(0);  // pads stay zero
  // wrapped global coordinates of the owned cells (-1: outside a non-periodic boundary); with n0 even
  // and i0 even the pair (2 lane, 2 lane + 1) is never split by a boundary or a wrap
  int gi0;
  {
    const int g = i0 + 2 * lane;
    gi0 = (g >= 0 && g < n0) ? g : (per0 ? wrap(g, n0) : -1);
  }
  int cidx[R];          // global index of the even cell of the owned pair of row q (0 when outside)
  int cidxc[R];         // modes 1, 2: index of the coarse cell of that pair
  unsigned live = 0;    // bit 2q+p: active cell
  unsigned inb = 0;     // bit q: the pair of row q lies inside the level (staged from global memory)
  unsigned store = 0;   // bit 2q+p: an output cell of this tile
  unsigned outq = 0;    // mode 2: bit q: the pair of row q lies in the output region and inside the level
  const T *__restrict__ cp0 = LA<T>::cp(L, 0);
  const T *__restrict__ cp1 = LA<T>::cp(L, 1);
  const T *__restrict__ invd = LA<T>::invd(L);
  const bool xhalf = C.coarsened[0] != 0, yhalf = C.coarsened[1] != 0;
  T ce[R][2], cw[R][2], cn[R][2], cs[R][2];
  T dcc[R][2], dwt[R][2];  // inv_inline: the cell's cc and w01 (1 / diagonal = rcpt(fma(shift, w01, cc)), as the table)
#pragma unroll
  for (int q = 0; q < R; q++) {
    const int r = w + NW * q;
    const int g = j0 + r;
    const int gj = (g >= 0 && g < n1) ? g : (per1 ? wrap(g, n1) : -1);
    const bool in = gi0 >= 0 && gj >= 0;
    cidx[q] = in ? gi0 + n0 * gj : 0;
    cidxc[q] = in ? (xhalf ? gi0 / 2 : gi0) + C.n[0] * (yhalf ? gj / 2 : gj) : 0;
    if (in) inb |= 1u << q;
#pragma unroll
    for (int p = 0; p < 2; p++) {
      T e_ = 0, w_ = 0, n_ = 0, s_ = 0;
      if (in) {
        const int ii = gi0 + p, c = cidx[q] + p;
        if (!(L.code[c] & 0x8000)) {
          live |= 1u << (2 * q + p);
          if (!skip0) {
            e_ = cp0[c];
            w_ = ii > 0 ? cp0[c - 1] : (per0 ? cp0[c + n0 - 1] : T(0));
          }
          if (!skip1) {
            n_ = cp1[c];
            s_ = gj > 0 ? cp1[c - n0] : (per1 ? cp1[c + n0 * (n1 - 1)] : T(0));
          }
        }
      }
      ce[q][p] = e_;
      cw[q][p] = w_;
      cn[q][p] = n_;
      cs[q][p] = s_;
      dcc[q][p] = (inv_inline && (live >> (2 * q + p) & 1)) ? LA<T>::cc(L)[cidx[q] + p] : T(0);
      dwt[q][p] = (inv_inline && (live >> (2 * q + p) & 1)) ? LA<T>::w01(L)[cidx[q] + p] : T(0);
      if (MODE == 2 && !inv_inline) {  // each thread reads back only its own entries: no barrier needed
        const int dq = (2 * q + p) * NW * 32 + (int)threadIdx.x;
        const bool lv = live >> (2 * q + p) & 1;
        dtab[dq] = lv ? LA<T>::cc(L)[cidx[q] + p] : T(0);
        dtab[2 * R * NW * 32 + dq] = lv ? LA<T>::w01(L)[cidx[q] + p] : T(0);
      }
      // unwrapped: each global cell is stored by one tile only (stored cells are never wrapped)
      const int col = 2 * lane + p, ui = i0 + col, uj = j0 + r;
      const bool outc = r >= TH && r < TH + BY && col >= TH && col < TH + TBX && ui < n0 && uj < n1;
      if (outc && (live >> (2 * q + p) & 1)) store |= 1u << (2 * q + p);
      if (p == 0 && outc) outq |= 1u << q;
    }
  }
  // this thread's cells in the tile and the staging area
  const int tpos = (w + 1) * TRS + lane + 1;  // row q adds (NW * q) * TRS
  const int spos = w * 64 + 2 * lane;         // row q adds (NW * q) * 64; array a of stage k adds (k * NA + a) * SH * 64
  // parity of the even column of the owned pairs (the same for every row of this thread, NW being even)
  const int par = (i0 + j0 + w) & 1;
  // stage the inputs of system `sys` (each thread copies exactly the cells it owns)
  auto issue = [&](int sys, int k) {
    const long off = L.ncell * (long)sys, offc = C.ncell * (long)sys;
    T *sk = stg + (size_t)k * NA * SH * 64 + spos;
#pragma unroll
    for (int q = 0; q < R; q++) {
      const bool in = inb >> q & 1;
      T *sq = sk + NW * q * 64;
      cp_async_zfill<2 * sizeof(T)>(sq, b + off + cidx[q], in);
      if (!inv_inline) cp_async_zfill<2 * sizeof(T)>(sq + SH * 64, invd + off + cidx[q], in);
      if (MODE == 1) {
        cp_async_zfill<2 * sizeof(T)>(sq + 2 * SH * 64, xin + off + cidx[q], in);
        if (xhalf) cp_async_zfill<sizeof(T)>(sq + 3 * SH * 64, xc + offc + cidxc[q], in);
        else cp_async_zfill<2 * sizeof(T)>(sq + 3 * SH * 64, xc + offc + cidxc[q], in);
      }
    }
    cp_async_commit();
  };
  // systems strided over the CTA groups: systems still active late in a solve (often neighbouring
  // wavenumbers) spread over many CTAs instead of queueing in one
  const int sstep = (int)gridDim.y;
  auto next_active = [&](int from) {
    for (int q = from; q < nsys; q += sstep)
      if (!active || active[q]) return q;
    return -1;
  };
  pdl_enter();  // everything above reads constant tables only
  int cur = next_active((int)blockIdx.y), k = 0;
  if (cur >= 0) issue(cur, 0);
  while (cur >= 0) {
    const int nxt = next_active(cur + sstep);
    if (nxt >= 0) {
      issue(nxt, k ^ 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();  // the staged inputs are complete and the previous system's sweeps are over
    T bv[R][2], iv[R][2];
    // the pre-smoother's first half-sweep sees only zero neighbours (x = 0 everywhere, pads included): its
    // sum of neighbour terms is +0, so (b - 0) / d = b (1/d) exactly, and it is done while loading
    const int t0 = MODE != 1 && nhalf > 0 ? 1 : 0;
    const int pfirst = (first_color + par) & 1;  // the column of the pair that half-sweep 0 updates
    {
      const T sh = inv_inline ? shift[cur] : T(0);
      const T *sk = stg + (size_t)k * NA * SH * 64 + spos;
#pragma unroll
      for (int q = 0; q < R; q++) {
        const T *sq = sk + NW * q * 64;
        // the staged pairs of b, 1/d and the pre-smoothed x read as vectors (a 2-way bank conflict less per
        // array; spos is even and every staged array starts on a 16-byte boundary)
        const V2 b2 = *reinterpret_cast<const V2 *>(sq);
        const V2 i2 = inv_inline ? V2{} : *reinterpret_cast<const V2 *>(sq + SH * 64);
        const V2 p2 = MODE == 1 ? *reinterpret_cast<const V2 *>(sq + 2 * SH * 64) : V2{};
#pragma unroll
        for (int p = 0; p < 2; p++) {
          const bool lv = live >> (2 * q + p) & 1;
          bv[q][p] = lv ? (p ? b2.y : b2.x) : T(0);
          iv[q][p] = lv ? (inv_inline ? rcpt(fmat(sh, dwt[q][p], dcc[q][p])) : (p ? i2.y : i2.x)) : T(0);
          T x_ = 0;
          if (MODE == 1 && lv) x_ = (p ? p2.y : p2.x) + sq[3 * SH * 64 + (xhalf ? 0 : p)];
          if (MODE != 1 && t0 && p == pfirst) x_ = bv[q][p] * iv[q][p];
          (p ? xo : xe)[tpos + NW * q * TRS] = x_;
        }
      }
    }
    for (int t = t0; t < nhalf; t++) {
      __syncthreads();
      if (((first_color + t + par) & 1) == 0) {  // even columns 2 lane: E = odd(lane), W = odd(lane - 1)
#pragma unroll
        for (int q = 0; q < R; q++) {
          T *o = xe + tpos + NW * q * TRS;
          const T *e = xo + tpos + NW * q * TRS;
          T acc = fmat(ce[q][0], e[0], T(0));
          acc = fmat(cw[q][0], e[-1], acc);
          acc = fmat(cn[q][0], o[TRS], acc);
          acc = fmat(cs[q][0], o[-TRS], acc);
          o[0] = (bv[q][0] - acc) * iv[q][0];
        }
      } else {                                   // odd columns 2 lane + 1: E = even(lane + 1), W = even(lane)
#pragma unroll
        for (int q = 0; q < R; q++) {
          T *o = xo + tpos + NW * q * TRS;
          const T *e = xe + tpos + NW * q * TRS;
          T acc = fmat(ce[q][1], e[1], T(0));
          acc = fmat(cw[q][1], e[0], acc);
          acc = fmat(cn[q][1], o[TRS], acc);
          acc = fmat(cs[q][1], o[-TRS], acc);
          o[0] = (bv[q][1] - acc) * iv[q][1];
        }
      }
    }
    // every thread stores only cells it updated itself: no barrier needed here
    const long off = L.ncell * (long)cur;
    T bx = 0, sx = 0, sb = 0;
#pragma unroll
    for (int q = 0; q < R; q++) {
#pragma unroll
      for (int p = 0; p < 2; p++) {
        if (!(store >> (2 * q + p) & 1)) continue;
        const T v = (p ? xo : xe)[tpos + NW * q * TRS];
        x[off + cidx[q] + p] = v;
        bx = fmat(bv[q][p], v, bx);
        sx += v;
        sb += bv[q][p];
      }
    }
    if (part_bx) {  // one partial per warp (shuffles only: no barrier in the system loop)
      const long e = (long)cur * part_stride + (long)blockIdx.x * NW + w;
      double t = (double)bx;
      for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
      if (lane == 0) part_bx[e] = t;
      if (singular && singular[cur]) {
        double tx = (double)sx, tb = (double)sb;
        for (int o = 16; o > 0; o >>= 1) {
          tx += __shfl_down_sync(0xffffffffu, tx, o);
          tb += __shfl_down_sync(0xffffffffu, tb, o);
        }
        if (lane == 0) { part_x[e] = tx; part_b[e] = tb; }
      }
    }
    if constexpr (MODE == 2) {
      // residual of every owned output cell, term by term as the level kernels form it (the off-diagonal
      // sum in the order E, W, N, S, then b - (shift w01 + cc) x - sum); 0 for every other cell.  The cells'
      // cc and w01 (the same for every system) were put in shared memory at set-up
      __syncthreads();  // the last half-sweep of every thread is complete
      const T sh = shift[cur];
      T rv[R][2];
#pragma unroll
      for (int q = 0; q < R; q++) {
#pragma unroll
        for (int p = 0; p < 2; p++) {
          rv[q][p] = 0;
          if (store >> (2 * q + p) & 1) {
            const T *o = (p ? xo : xe) + tpos + NW * q * TRS;  // the cell's colour array
            const T *e = (p ? xe : xo) + tpos + NW * q * TRS;  // the other colour
            T acc = fmat(ce[q][p], p ? e[1] : e[0], T(0));
            acc = fmat(cw[q][p], p ? e[0] : e[-1], acc);
            acc = fmat(cn[q][p], o[TRS], acc);
            acc = fmat(cs[q][p], o[-TRS], acc);
            const int dq = (2 * q + p) * NW * 32 + (int)threadIdx.x;
            const T dv = inv_inline ? fmat(sh, dwt[q][p], dcc[q][p]) : fmat(sh, dtab[2 * R * NW * 32 + dq], dtab[dq]);
            rv[q][p] = bv[q][p] - fmat(dv, o[0], acc);
          }
        }
      }
      // summed restriction, children in the order (dj outer, di inner) of the level kernels.  The children of
      // a coarse cell along x are the thread's own pair; along y, rows 2J and 2J + 1 of the tile belong to
      // warps w and w + 1 (same lane, same q: NW and the tile's first row are even), so the odd warps hand
      // their residuals over in shared memory and the even warps store the coarse cells
      T *__restrict__ bcs = bco + C.ncell * (long)cur;
      T *__restrict__ xcs = xcz ? xcz + C.ncell * (long)cur : nullptr;
      const bool oddw = w & 1;
      if (yhalf) {
        T *const hand = res + (w >> 1) * 32 + lane;  // [q][p][NW / 2][32 lanes]
        if (oddw) {
#pragma unroll
          for (int q = 0; q < R; q++) {
            hand[q * NW * 32] = rv[q][0];
            hand[q * NW * 32 + NW * 16] = rv[q][1];
          }
        }
        __syncthreads();
        if (!oddw) {
#pragma unroll
          for (int q = 0; q < R; q++) {
            if (!(outq >> q & 1)) continue;
            const T u0 = hand[q * NW * 32], u1 = hand[q * NW * 32 + NW * 16];
            if (xhalf) {
              T sum = 0;
              sum += rv[q][0];
              sum += rv[q][1];
              sum += u0;
              sum += u1;
              bcs[cidxc[q]] = sum;
              if (xcs) xcs[cidxc[q]] = T(0);
            } else {
              T s0 = 0, s1 = 0;
              s0 += rv[q][0];
              s0 += u0;
              s1 += rv[q][1];
              s1 += u1;
              bcs[cidxc[q]] = s0;
              bcs[cidxc[q] + 1] = s1;
              if (xcs) { xcs[cidxc[q]] = T(0); xcs[cidxc[q] + 1] = T(0); }
            }
          }
        }
      } else {
#pragma unroll
        for (int q = 0; q < R; q++) {
          if (!(outq >> q & 1)) continue;
          if (xhalf) {
            T sum = 0;
            sum += rv[q][0];
            sum += rv[q][1];
            bcs[cidxc[q]] = sum;
            if (xcs) xcs[cidxc[q]] = T(0);
          } else {  // no axis halved (not built by the hierarchy; kept general)
            T s0 = 0, s1 = 0;
            s0 += rv[q][0];
            s1 += rv[q][1];
            bcs[cidxc[q]] = s0;
            bcs[cidxc[q] + 1] = s1;
            if (xcs) { xcs[cidxc[q]] = T(0); xcs[cidxc[q] + 1] = T(0); }
          }
        }
      }
    }
    cur = nxt;
    k ^= 1;
  }
}

// modes 0 (pre-smoother) and 1 (post-smoother)
template <typename T, int NW, int R, int MODE>
__global__ void __launch_bounds__(NW * 32) k_rbgs_tile2d(MgLevelD L, MgLevelD C, int per0, int per1,
                                                         const int *__restrict__ active, int nsys, int sb,
                                                         int first_color, int nhalf, T *__restrict__ x,
                                                         const T *__restrict__ b, const T *__restrict__ xin,
                                                         const T *__restrict__ xc, double *__restrict__ part_bx,
                                                         const int *__restrict__ singular, double *__restrict__ part_x,
                                                         double *__restrict__ part_b, int part_stride,
                                                         const T *__restrict__ shift, int inv_inline) {
  rbgs_tile2d<T, NW, R, MODE>(L, C, per0, per1, active, nsys, sb, first_color, nhalf, x, b, xin, xc, part_bx, singular,
                              part_x, part_b, part_stride, shift, inv_inline, nullptr, nullptr);
}

// mode 2 (pre-smoother restricting its residual into bco, zeroing xcz when given); with two rows per thread
// at most 64 registers, so that 2048 threads' worth of CTAs fit on a multiprocessor as in mode 0
template <typename T, int NW, int R>
__global__ void __launch_bounds__(NW * 32, R == 2 ? 1024 / (NW * 32) : 1)
    k_rbgs_tile2d_restrict(MgLevelD L, MgLevelD C, int per0, int per1, const int *__restrict__ active, int nsys, int sb,
                           int nhalf, T *__restrict__ x, const T *__restrict__ b, const T *__restrict__ shift,
                           int inv_inline, T *__restrict__ bco, T *__restrict__ xcz) {
  rbgs_tile2d<T, NW, R, 2>(L, C, per0, per1, active, nsys, sb, 0, nhalf, x, b, nullptr, nullptr, nullptr, nullptr,
                           nullptr, nullptr, 0, shift, inv_inline, bco, xcz);
}

// ---------------------------------------------------------------- whole coarse V-cycle in one CTA
constexpr int COARSE_THREADS = 1024;

// where the coarse V-cycle kernel keeps each level: x, b and 1/d in shared memory; the couplings too when
// they fit (else they are read from global memory, where every system shares them and L2 holds them)
struct CoarseLev {
  int ox, ob, oi;  // shared-memory offsets (elements) of x, b, 1/d
  int oc;          // couplings c0 | c1 at oc, oc + ncell; -1: global memory
  int od;          // the system's diagonal shift w01 + cc (the residual's); -1: formed from global memory
  int hdj, hdi;    // walker steps over the half rows of a colour: COARSE_THREADS / h0, % h0 (h0 = (n0+1)/2)
  int fdj, fdi;    // walker steps over full rows: COARSE_THREADS / n0, % n0
};
struct CoarsePlan {
  CoarseLev lev[MG_MAXLEV];
};

// the layout for levels l0.. : x, b and 1/d of every level (the dense coarsest level only x and b) in
// shared memory, then the couplings of as many levels as still fit, the coarsest first; false when even
// x, b and 1/d do not fit
template <typename T>
static bool coarse_plan(const MgProblem &P, int l0, CoarsePlan *plan, size_t *bytes) {
  const int last = P.nlev - 1;
  const bool dense = LA<T>::dinv(P.L[last]) != nullptr;
  size_t o = 0;
  CoarsePlan pl{};
  for (int l = l0; l < P.nlev; l++) {
    const MgLevelD &L = P.L[l];
    const int n = (int)L.ncell, n0 = L.n[0], h0 = (n0 + 1) / 2;
    CoarseLev &e = pl.lev[l];
    e.hdj = COARSE_THREADS / h0;
    e.hdi = COARSE_THREADS % h0;
    e.fdj = COARSE_THREADS / n0;
    e.fdi = COARSE_THREADS % n0;
    e.ox = (int)o;
    e.ob = (int)o + n;
    o += 2 * (size_t)n;
    e.oi = e.oc = e.od = -1;
    if (l == last && dense) continue;
    e.oi = (int)o;
    o += n;
  }
  if (o * sizeof(T) > MG_COARSE_SMEM_MAX) return false;
  // couplings of the coarsest levels first: their sweeps have about one cell per thread, so a global load
  // there is an exposed L2 latency per phase, while the finest level's many cells per thread overlap theirs
  for (int l = last; l >= l0; l--) {
    if (l == last && dense) continue;
    const size_t need = 2 * (size_t)P.L[l].ncell;
    if ((o + need) * sizeof(T) > MG_COARSE_SMEM_MAX) break;
    pl.lev[l].oc = (int)o;
    o += need;
  }
  // then the diagonals the restriction's residual uses, where room is left (coarsest first): formed once per
  // launch instead of two L2 reads per child in every restriction phase
  for (int l = last - 1; l >= l0; l--) {
    const size_t need = (size_t)P.L[l].ncell;
    if ((o + need) * sizeof(T) > MG_COARSE_SMEM_MAX) break;
    pl.lev[l].od = (int)o;
    o += need;
  }
  if (plan) *plan = pl;
  if (bytes) *bytes = o * sizeof(T);
  return true;
}

// one half-sweep of a level held in shared memory (inactive cells have 1/d = 0); the walker visits the
// cells of one colour without a division per cell
template <typename T>
__device__ __forceinline__ void cta_sweep_xy(int n0, int n1, int per0, int per1, T *x, const T *b, const T *id,
                                             const T *c0, const T *c1, int color, int hdj, int hdi) {
  const int h0 = (n0 + 1) >> 1;
  int j = (int)threadIdx.x / h0, ih = (int)threadIdx.x - j * h0;
  while (j < n1) {
    const int i = 2 * ih + ((color + j) & 1);
    if (i < n0) {
      const int c = i + n0 * j;
      const T iv = id[c];
      if (iv != T(0)) {
        const T acc = offdiag_xy<T>(n0, n1, per0, per1, c0, c1, [&](int e) { return x[e]; }, c, i, j);
        x[c] = (b[c] - acc) * iv;
      }
    }
    ih += hdi;
    j += hdj;
    if (ih >= h0) { ih -= h0; j++; }
  }
  __syncthreads();
}

// The same half-sweep for an even n0 with a fixed cell ownership: thread t owns the column pair (2p, 2p+1),
// p = t % (n0/2), in the rows j = g, g + G, ... (g = t / (n0/2), G = COARSE_THREADS / (n0/2)), and in each of
// them updates the one cell of the pair that has the sweep's colour.  The east/west offsets (wrapped on a
// periodic axis, 0 with a zero coupling at a wall) are fixed per thread, so a cell costs its ten shared loads,
// four FMAs and a store.  Same terms in the same order as cta_sweep_xy: a missing neighbour contributes a
// zero coupling times the cell's own value.
template <typename T>
__device__ __forceinline__ void cta_sweep_pairs(int n0, int n1, int per0, int per1, T *x, const T *b, const T *id,
                                                const T *c0, const T *c1, int color) {
  const int np = n0 >> 1;
  const int G = COARSE_THREADS / np;
  const int t = (int)threadIdx.x;
  if (t < G * np) {
    const int g = t / np, p = t - g * np;
    const int we0 = p > 0 ? -1 : (per0 ? n0 - 1 : 0);       // west of the even cell 2p
    const int ee1 = p < np - 1 ? 1 : (per0 ? 1 - n0 : 0);   // east of the odd cell 2p + 1
    const bool hw0 = p > 0 || per0;                          // the even cell has a west neighbour
    const int wrap_n = per1 ? n0 - n0 * n1 : 0, wrap_s = per1 ? n0 * (n1 - 1) : 0;
    // a missing east/north neighbour has a zero (folded) coupling c0[c] / c1[c]; a missing west/south one
    // has none to read, so its coupling is taken as zero here
    for (int j = g; j < n1; j += G) {
      const int e = (color + j) & 1;
      const int c = j * n0 + 2 * p + e;
      const int oe = e ? ee1 : 1, ow = e ? -1 : we0;
      const int on = j + 1 < n1 ? n0 : wrap_n, os = j > 0 ? -n0 : wrap_s;
      const T iv = id[c];
      if (iv != T(0)) {
        const T cwv = (e || hw0) ? c0[c + ow] : T(0);
        const T csv = (j > 0 || per1) ? c1[c + os] : T(0);
        T acc = fmat(c0[c], x[c + oe], T(0));
        acc = fmat(cwv, x[c + ow], acc);
        acc = fmat(c1[c], x[c + on], acc);
        acc = fmat(csv, x[c + os], acc);
        x[c] = (b[c] - acc) * iv;
      }
    }
  }
  __syncthreads();
}

// one half-sweep of level (n0, n1): the pair-owned form where it applies, else the walker
template <typename T>
__device__ __forceinline__ void cta_sweep(int n0, int n1, int per0, int per1, T *x, const T *b, const T *id,
                                          const T *c0, const T *c1, int color, int hdj, int hdi) {
  if (!(n0 & 1) && n0 >= 4 && (n0 >> 1) <= COARSE_THREADS) cta_sweep_pairs<T>(n0, n1, per0, per1, x, b, id, c0, c1, color);
  else cta_sweep_xy<T>(n0, n1, per0, per1, x, b, id, c0, c1, color, hdj, hdi);
}

// Coarsest level x = Dinv b by all threads: row r is split into KS contiguous column chunks summed by KS
// threads (KS = COARSE_THREADS / n), then the chunk sums of each row are added in chunk order.  Every load of
// the (global, L2-resident) inverse then waits behind a few others instead of n.
template <typename T>
__device__ __forceinline__ void cta_dense(int n, const T *__restrict__ M, const T *bv, T *xv, T *red) {
  const int KS = COARSE_THREADS / n;
  const int chunk = (n + KS - 1) / KS;
  const int t = (int)threadIdx.x, k = t / n, r = t - k * n;
  if (k < KS) {
    const int ca = k * chunk, cb = min(n, ca + chunk);
    T acc = 0;
#pragma unroll 4
    for (int c = ca; c < cb; c++) acc = fmat(M[(size_t)c * n + r], bv[c], acc);
    red[k * n + r] = acc;
  }
  __syncthreads();
  if (t < n) {
    T v = red[t];
    for (int q = 1; q < KS; q++) v += red[q * n + t];
    xv[t] = v;
  }
  __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(COARSE_THREADS, 1) k_vcycle_coarse(MgProblem P, CoarsePlan plan, int l0,
                                                                     const T *__restrict__ shift,
                                                                     const int *__restrict__ active,
                                                                     T *__restrict__ xout, const T *__restrict__ bin) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ T red[COARSE_THREADS];  // chunk sums of the dense coarsest solve
  pdl_enter();
  const int s = blockIdx.x;
  if (active && !active[s]) return;
  const int last = P.nlev - 1;
  const bool dense = LA<T>::dinv(P.L[last]) != nullptr;
  const int per0 = P.periodic[0], per1 = P.periodic[1];
  T *const base = (T *)smem_raw;
  auto X = [&](int l) { return base + plan.lev[l].ox; };
  auto B = [&](int l) { return base + plan.lev[l].ob; };
  auto ID = [&](int l) { return base + plan.lev[l].oi; };
  // f(c0, c1) with the couplings of level l: two inlined copies, one reading shared memory and one global
  // memory, so that neither goes through generic loads
  auto with_c = [&](int l, auto &&f) {
    if (plan.lev[l].oc >= 0) {
      const T *c0 = base + plan.lev[l].oc;
      f(c0, c0 + (int)P.L[l].ncell);
    } else {
      f(LA<T>::cp(P.L[l], 0), LA<T>::cp(P.L[l], 1));
    }
  };
  const T sh = shift[s];
  for (int l = l0; l < P.nlev; l++) {
    if (l == last && dense) break;
    const MgLevelD &L = P.L[l];
    const int n = (int)L.ncell;
    const T *__restrict__ invd = LA<T>::invd(L) + (long)n * s;
    const T *__restrict__ cp0 = LA<T>::cp(L, 0);
    const T *__restrict__ cp1 = LA<T>::cp(L, 1);
    T *id = ID(l);
    const bool cs = plan.lev[l].oc >= 0, ds = plan.lev[l].od >= 0;
    T *c0 = base + plan.lev[l].oc, *c1 = c0 + n;
    T *dg = base + plan.lev[l].od;
    const T *__restrict__ ccl = LA<T>::cc(L);
    const T *__restrict__ wtl = LA<T>::w01(L);
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
      id[c] = invd[c];
      if (cs) {
        c0[c] = cp0[c];
        c1[c] = cp1[c];
      }
      if (ds) dg[c] = fmat(sh, wtl[c], ccl[c]);  // the diagonal of the unfused residual, term by term
    }
  }
  {
    const int n = (int)P.L[l0].ncell;
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
      B(l0)[c] = bin[(long)n * s + c];
      X(l0)[c] = 0;
    }
  }
  __syncthreads();
  // down: pre-smoothing and restriction of the residual
  for (int l = l0; l < last; l++) {
    const MgLevelD &L = P.L[l];
    const MgLevelD &C = P.L[l + 1];
    const CoarseLev &E = plan.lev[l], &EC = plan.lev[l + 1];
    const int n0 = L.n[0], n1 = L.n[1];
    T *x = X(l);
    const T *b = B(l), *id = ID(l);
    const T *__restrict__ cc = LA<T>::cc(L);
    const T *__restrict__ w01 = LA<T>::w01(L);
    with_c(l, [&](const T *c0, const T *c1) {
      for (int it = 0; it < 2 * mg_nu(P, l); it++) cta_sweep<T>(n0, n1, per0, per1, x, b, id, c0, c1, it & 1, E.hdj, E.hdi);
      const int cn0 = C.n[0], cn1 = C.n[1];
      const int e0 = C.coarsened[0] ? 2 : 1, e1 = C.coarsened[1] ? 2 : 1;
      T *bc = B(l + 1), *xc = X(l + 1);
      int J = (int)threadIdx.x / cn0, I = (int)threadIdx.x - J * cn0;
      while (J < cn1) {
        T sum = 0;
        for (int dj = 0; dj < e1; dj++)
          for (int di = 0; di < e0; di++) {
            const int i = C.coarsened[0] ? 2 * I + di : I, j = C.coarsened[1] ? 2 * J + dj : J;
            const int c = i + n0 * j;
            if (id[c] == T(0)) continue;
            const T dv = E.od >= 0 ? base[E.od + c] : fmat(sh, w01[c], cc[c]);  // the unfused residual's diagonal
            const T acc = offdiag_xy<T>(n0, n1, per0, per1, c0, c1, [&](int e) { return x[e]; }, c, i, j);
            sum += b[c] - fmat(dv, x[c], acc);
          }
        bc[I + cn0 * J] = sum;
        xc[I + cn0 * J] = 0;
        I += EC.fdi;
        J += EC.fdj;
        if (I >= cn0) { I -= cn0; J++; }
      }
    });
    __syncthreads();
  }
  // coarsest level
  {
    const MgLevelD &L = P.L[last];
    const int n = (int)L.ncell;
    if (dense) {
      // the inverse is stored by columns (as for k_dense)
      cta_dense<T>(n, LA<T>::dinv(L) + (size_t)n * n * s, B(last), X(last), red);
    } else {
      const CoarseLev &E = plan.lev[last];
      with_c(last, [&](const T *c0, const T *c1) {
        for (int it = 0; it < 40; it++)
          for (int col = 0; col < 4; col++)
            cta_sweep<T>(L.n[0], L.n[1], per0, per1, X(last), B(last), ID(last), c0, c1,
                         (col == 1 || col == 2) ? 1 : 0, E.hdj, E.hdi);
      });
    }
  }
  // up: prolongation and post-smoothing
  for (int l = last - 1; l >= l0; l--) {
    const MgLevelD &L = P.L[l];
    const MgLevelD &C = P.L[l + 1];
    const CoarseLev &E = plan.lev[l];
    const int n0 = L.n[0], n1 = L.n[1], cn0 = C.n[0];
    T *x = X(l);
    const T *xc = X(l + 1), *id = ID(l);
    int j = (int)threadIdx.x / n0, i = (int)threadIdx.x - j * n0;
    while (j < n1) {
      const int c = i + n0 * j;
      if (id[c] != T(0)) {
        const int I = C.coarsened[0] ? i / 2 : i, J = C.coarsened[1] ? j / 2 : j;
        x[c] += xc[I + cn0 * J];
      }
      i += E.fdi;
      j += E.fdj;
      if (i >= n0) { i -= n0; j++; }
    }
    __syncthreads();
    with_c(l, [&](const T *c0, const T *c1) {
      for (int it = 0; it < 2 * mg_nu(P, l); it++)
        cta_sweep<T>(n0, n1, per0, per1, x, B(l), id, c0, c1, 1 - (it & 1), E.hdj, E.hdi);
    });
  }
  const int n = (int)P.L[l0].ncell;
  for (int c = threadIdx.x; c < n; c += blockDim.x) xout[(long)n * s + c] = X(l0)[c];
}

// ---------------------------------------------------------------- 3-D coarse end of a V-cycle in one CTA
// 3-D mode has one system, so its coarse levels (and the 160 half-sweeps of an iterative coarsest level)
// would be launch after launch of a few hundred cells.  Here one CTA of 1024 threads runs the V-cycle from
// level l0 down and back with x and b of every level in shared memory; the operator (shared by every
// system, L2-resident) is read from global memory.  Same arithmetic as k_rbgs, k_resid_restrict,
// k_prolong and k_dense, term by term.

// cells of a 3-D index space of extents m[3] visited by COARSE_THREADS threads without a division per cell
struct Walk3 {
  int a[3], s[3], m[3];
  __device__ void start(int m0, int m1, int m2) {
    m[0] = m0; m[1] = m1; m[2] = m2;
    const int t = threadIdx.x, S = COARSE_THREADS;
    a[0] = t % m0; a[1] = (t / m0) % m1; a[2] = t / (m0 * m1);
    s[0] = S % m0; s[1] = (S / m0) % m1; s[2] = S / (m0 * m1);
  }
  __device__ bool ok() const { return a[2] < m[2]; }
  __device__ void next() {
    a[0] += s[0];
    if (a[0] >= m[0]) { a[0] -= m[0]; a[1]++; }
    a[1] += s[1];
    if (a[1] >= m[1]) { a[1] -= m[1]; a[2]++; }
    a[2] += s[2];
  }
};

template <typename T>
__device__ __forceinline__ void cta_sweep3(const MgLevelD &L, const MgGeom &G, T sh, T *x, const T *b, int color) {
  const int n0 = L.n[0], h0 = (n0 + 1) >> 1;
  Walk3 w;
  for (w.start(h0, L.n[1], L.n[2]); w.ok(); w.next()) {
    const int j = w.a[1], k = w.a[2], i = 2 * w.a[0] + ((color + j + k) & 1);
    if (i >= n0) continue;
    const int c = i + n0 * (j + L.n[1] * k);
    if (L.code[c] & 0x8000) continue;
    const T d = diag_of<T>(L, G, sh, c);
    const T acc = offdiag<T>(L, G, [&](int e) { return x[e]; }, c, i, j, k);
    x[c] = (b[c] - acc) * rcpt(d);
  }
  __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(COARSE_THREADS, 1) k_vcycle_coarse3d(MgProblem P, MgGeom G, int l0,
                                                                       const T *__restrict__ shift,
                                                                       const int *__restrict__ active,
                                                                       T *__restrict__ xout, const T *__restrict__ bin) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int s = blockIdx.x;
  if (active && !active[s]) return;
  const int last = P.nlev - 1;
  const bool dense = LA<T>::dinv(P.L[last]) != nullptr;
  __shared__ int off[MG_MAXLEV];
  if (threadIdx.x == 0) {
    int o = 0;
    for (int l = l0; l < P.nlev; l++) { off[l] = o; o += 2 * (int)P.L[l].ncell; }
  }
  __syncthreads();
  T *const base = (T *)smem_raw;
  auto X = [&](int l) { return base + off[l]; };
  auto B = [&](int l) { return base + off[l] + (int)P.L[l].ncell; };
  const T sh = shift[s];
  {
    const int n = (int)P.L[l0].ncell;
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
      B(l0)[c] = bin[(long)n * s + c];
      X(l0)[c] = 0;
    }
  }
  __syncthreads();
  for (int l = l0; l < last; l++) {
    const MgLevelD &F = P.L[l], &C = P.L[l + 1];
    T *x = X(l);
    const T *b = B(l);
    for (int it = 0; it < 2 * mg_nu(P, l); it++) cta_sweep3<T>(F, G, sh, x, b, it & 1);
    const int e0 = C.coarsened[0] ? 2 : 1, e1 = C.coarsened[1] ? 2 : 1, e2 = C.coarsened[2] ? 2 : 1;
    T *bc = B(l + 1), *xc = X(l + 1);
    Walk3 w;
    for (w.start(C.n[0], C.n[1], C.n[2]); w.ok(); w.next()) {
      const int I = w.a[0], J = w.a[1], K = w.a[2];
      T sum = 0;
      for (int dk = 0; dk < e2; dk++)
        for (int dj = 0; dj < e1; dj++)
          for (int di = 0; di < e0; di++) {
            const int i = C.coarsened[0] ? 2 * I + di : I, j = C.coarsened[1] ? 2 * J + dj : J,
                      k = C.coarsened[2] ? 2 * K + dk : K;
            const int c = i + F.n[0] * (j + F.n[1] * k);
            if (F.code[c] & 0x8000) continue;
            const T acc = offdiag<T>(F, G, [&](int e) { return x[e]; }, c, i, j, k);
            sum += b[c] - fmat(diag_of<T>(F, G, sh, c), x[c], acc);
          }
      const int cc = I + C.n[0] * (J + C.n[1] * K);
      bc[cc] = sum;
      xc[cc] = 0;
    }
    __syncthreads();
  }
  {
    const MgLevelD &L = P.L[last];
    const int n = (int)L.ncell;
    if (dense) {
      const T *__restrict__ M = LA<T>::dinv(L) + (size_t)n * n * s;
      for (int r = threadIdx.x; r < n; r += blockDim.x) {  // the inverse is stored by columns (as k_dense)
        T acc = 0;
#pragma unroll 8
        for (int c = 0; c < n; c++) acc = fmat(M[(size_t)c * n + r], B(last)[c], acc);
        X(last)[r] = acc;
      }
      __syncthreads();
    } else {
      for (int it = 0; it < 40; it++)
        for (int col = 0; col < 4; col++) cta_sweep3<T>(L, G, sh, X(last), B(last), (col == 1 || col == 2) ? 1 : 0);
    }
  }
  for (int l = last - 1; l >= l0; l--) {
    const MgLevelD &F = P.L[l], &C = P.L[l + 1];
    T *x = X(l);
    const T *xc = X(l + 1);
    Walk3 w;
    for (w.start(F.n[0], F.n[1], F.n[2]); w.ok(); w.next()) {
      const int i = w.a[0], j = w.a[1], k = w.a[2];
      const int c = i + F.n[0] * (j + F.n[1] * k);
      if (F.code[c] & 0x8000) continue;
      const int I = C.coarsened[0] ? i / 2 : i, J = C.coarsened[1] ? j / 2 : j, K = C.coarsened[2] ? k / 2 : k;
      x[c] += xc[I + C.n[0] * (J + C.n[1] * K)];
    }
    __syncthreads();
    for (int it = 0; it < 2 * mg_nu(P, l); it++) cta_sweep3<T>(F, G, sh, x, B(l), 1 - (it & 1));
  }
  const int n = (int)P.L[l0].ncell;
  for (int c = threadIdx.x; c < n; c += blockDim.x) xout[(long)n * s + c] = X(l0)[c];
}

// ---------------------------------------------------------------- launchers
// opt in to more than 48 KB of dynamic shared memory, once per kernel and device
static int allow_smem(const void *fn, size_t bytes) {
  // the default limit of 48 KB covers static and dynamic shared memory together: the kernels here keep at most
  // 8 KB of static shared memory, so up to 40 KB of dynamic shared memory needs no opt-in
  if (bytes <= 40 * 1024) return SNAC_OK;
  static std::mutex mu;
  static std::vector<std::pair<const void *, int>> done;
  int dev = 0;
  SNAC_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  for (auto &e : done)
    if (e.first == fn && e.second == dev) return SNAC_OK;
  // the opt-in limit less the kernel's own static shared memory (the coarse kernels keep some)
  int optin = 0;
  SNAC_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  cudaFuncAttributes fa;
  SNAC_CUDA(cudaFuncGetAttributes(&fa, fn));
  const size_t room = (size_t)optin > fa.sharedSizeBytes ? (size_t)optin - fa.sharedSizeBytes : 0;
  if (bytes > room) {
    set_error("kernel needs %zu bytes of dynamic shared memory, %zu available", bytes, room);
    return SNAC_ERR_ARG;
  }
  SNAC_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::min(room, MG_SMEM_OPT_IN)));
  done.push_back({fn, dev});
  return SNAC_OK;
}

// the per-system shifts in the tile's precision (the 1 / diagonal formed in registers needs them)
template <typename T>
static const T *shift_of_tile(const MgProblem &P) {
  if constexpr (sizeof(T) == 8) return P.shift;
  else return P.shiftf;
}

template <typename T, int NW, int R>
static int launch_tile(const MgProblem &P, const MgLevelD &L, const MgLevelD &C, int nt, int nhalf, const int *active,
                       int first_color, int mode, T *x, const T *b, const T *xin, const T *xc, double *part_bx,
                       double *part_x, double *part_b, int part_stride, cudaStream_t st, T *bco = nullptr,
                       T *xcz = nullptr) {
  const int *sing = P.any_singular && part_bx ? P.singular : nullptr;
  const int inv = sizeof(T) == 4 && P.tile_inv ? 1 : 0;  // FP64 keeps the table (its reciprocal is costly)
  const size_t smem = tile_smem_bytes<T>(NW * R, mode);
  const int sb = plane_batch(P, nt, NW == 16 ? 2 : 4);
  const dim3 g((unsigned)nt, (unsigned)((P.nsys + sb - 1) / sb));
  if (mode == 2) {
    if constexpr (sizeof(T) == 4) {
      SNAC_TRY(allow_smem((const void *)k_rbgs_tile2d_restrict<T, NW, R>, smem));
      SNAC_CUDA(launch_k(k_rbgs_tile2d_restrict<T, NW, R>, g, dim3(NW * 32), smem, st, L, C, P.periodic[0],
                         P.periodic[1], active, P.nsys, sb, nhalf, x, b, shift_of_tile<T>(P), inv, bco, xcz));
    } else {
      set_error("the restricting tiled pre-smoother is FP32 only");
      return SNAC_ERR_ARG;
    }
  } else if (mode == 1) {
    SNAC_TRY(allow_smem((const void *)k_rbgs_tile2d<T, NW, R, 1>, smem));
    SNAC_CUDA(launch_k(k_rbgs_tile2d<T, NW, R, 1>, g, dim3(NW * 32), smem, st, L, C, P.periodic[0], P.periodic[1],
                       active, P.nsys, sb, first_color, nhalf, x, b, xin, xc, part_bx, sing, part_x, part_b,
                       part_stride, shift_of_tile<T>(P), inv));
  } else {
    SNAC_TRY(allow_smem((const void *)k_rbgs_tile2d<T, NW, R, 0>, smem));
    SNAC_CUDA(launch_k(k_rbgs_tile2d<T, NW, R, 0>, g, dim3(NW * 32), smem, st, L, C, P.periodic[0], P.periodic[1],
                       active, P.nsys, sb, first_color, nhalf, x, b, xin, xc, part_bx, sing, part_x, part_b,
                       part_stride, shift_of_tile<T>(P), inv));
  }
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

template <typename T>
int launch_rbgs_tile2d(const MgProblem &P, int l, const int *active, int first_color, int mode, T *x, const T *b,
                       const T *xin, const T *xc, double *part_bx, double *part_x, double *part_b, int part_stride,
                       int *nchunk, cudaStream_t st) {
  if (mode == 1 && (xin == x || !xin || !xc)) { set_error("tiled post-smoother needs separate input and output"); return SNAC_ERR_ARG; }
  const MgLevelD &L = P.L[l];
  const MgLevelD &C = l + 1 < P.nlev ? P.L[l + 1] : P.L[l];
  const TileShape t = choose_shape(L, sizeof(T) == 8 ? 1 : 0, P.tile_shape);
  const int nt = tiles_for(L, t);
  if (part_bx && nt * t.nw > part_stride) { set_error("partial-sum area too small for the tiled smoother"); return SNAC_ERR_ARG; }
  prof_begin(KID_RBGS, st);
  int rc;
  if constexpr (sizeof(T) == 8) {
    rc = launch_tile<T, 8, 2>(P, L, C, nt, 2 * mg_nu(P, l), active, first_color, mode, x, b, xin, xc, part_bx, part_x, part_b, part_stride, st);
  } else {
    if (t.nw == 8 && t.r == 2)
      rc = launch_tile<T, 8, 2>(P, L, C, nt, 2 * mg_nu(P, l), active, first_color, mode, x, b, xin, xc, part_bx, part_x, part_b, part_stride, st);
    else if (t.nw == 16 && t.r == 2)
      rc = launch_tile<T, 16, 2>(P, L, C, nt, 2 * mg_nu(P, l), active, first_color, mode, x, b, xin, xc, part_bx, part_x, part_b, part_stride, st);
    else if (t.nw == 8 && t.r == 3)
      rc = launch_tile<T, 8, 3>(P, L, C, nt, 2 * mg_nu(P, l), active, first_color, mode, x, b, xin, xc, part_bx, part_x, part_b, part_stride, st);
    else if (t.nw == 16 && t.r == 3)
      rc = launch_tile<T, 16, 3>(P, L, C, nt, 2 * mg_nu(P, l), active, first_color, mode, x, b, xin, xc, part_bx, part_x, part_b, part_stride, st);
    else if (t.nw == 8)
      rc = launch_tile<T, 8, 4>(P, L, C, nt, 2 * mg_nu(P, l), active, first_color, mode, x, b, xin, xc, part_bx, part_x, part_b, part_stride, st);
    else
      rc = launch_tile<T, 16, 4>(P, L, C, nt, 2 * mg_nu(P, l), active, first_color, mode, x, b, xin, xc, part_bx, part_x, part_b, part_stride, st);
  }
  prof_end(KID_RBGS, st);
  SNAC_TRY(rc);
  if (nchunk) *nchunk = part_bx ? nt * t.nw : 0;
  return SNAC_OK;
}

// The FP32 pre-smoother of level l (x = 0 in, 2 nu half-sweeps, xp out) that also writes the restricted
// residual b_{l+1} of its output cells, and zeroes x_{l+1} when xcz is given: the pre-smoother and
// plane_restrict of an unfused V-cycle in one pass, with the same values and the same tiles.
template <typename T>
int launch_rbgs_tile2d_restrict(const MgProblem &P, int l, const int *active, T *xp, const T *b, T *bc, T *xcz,
                                cudaStream_t st) {
  if constexpr (sizeof(T) != 4) {
    set_error("the restricting tiled pre-smoother is FP32 only");
    return SNAC_ERR_ARG;
  } else {
    if (l + 1 >= P.nlev || !bc) { set_error("restricting pre-smoother: level %d has no coarser level", l); return SNAC_ERR_ARG; }
    const MgLevelD &L = P.L[l];
    const MgLevelD &C = P.L[l + 1];
    const TileShape t = choose_shape(L, 0, P.tile_shape);
    const int nt = tiles_for(L, t);
    const int nhalf = 2 * mg_nu(P, l);
    prof_begin(KID_RBGS, st);
    int rc;
    if (t.nw == 8 && t.r == 2)
      rc = launch_tile<T, 8, 2>(P, L, C, nt, nhalf, active, 0, 2, xp, b, nullptr, nullptr, nullptr, nullptr, nullptr, 0, st, bc, xcz);
    else if (t.nw == 16 && t.r == 2)
      rc = launch_tile<T, 16, 2>(P, L, C, nt, nhalf, active, 0, 2, xp, b, nullptr, nullptr, nullptr, nullptr, nullptr, 0, st, bc, xcz);
    else if (t.nw == 8 && t.r == 3)
      rc = launch_tile<T, 8, 3>(P, L, C, nt, nhalf, active, 0, 2, xp, b, nullptr, nullptr, nullptr, nullptr, nullptr, 0, st, bc, xcz);
    else if (t.nw == 16 && t.r == 3)
      rc = launch_tile<T, 16, 3>(P, L, C, nt, nhalf, active, 0, 2, xp, b, nullptr, nullptr, nullptr, nullptr, nullptr, 0, st, bc, xcz);
    else if (t.nw == 8)
      rc = launch_tile<T, 8, 4>(P, L, C, nt, nhalf, active, 0, 2, xp, b, nullptr, nullptr, nullptr, nullptr, nullptr, 0, st, bc, xcz);
    else
      rc = launch_tile<T, 16, 4>(P, L, C, nt, nhalf, active, 0, 2, xp, b, nullptr, nullptr, nullptr, nullptr, nullptr, 0, st, bc, xcz);
    prof_end(KID_RBGS, st);
    return rc;
  }
}

template <typename T>
size_t coarse_smem_bytes(const MgProblem &P, int l0) {
  size_t bytes = 0;
  return coarse_plan<T>(P, l0, nullptr, &bytes) ? bytes : (size_t)-1;
}

template <typename T>
int launch_vcycle_coarse(const MgProblem &P, int l0, const T *shift, const int *active, T *x, const T *b,
                         cudaStream_t st) {
  CoarsePlan plan;
  size_t smem = 0;
  if (!coarse_plan<T>(P, l0, &plan, &smem)) { set_error("coarse levels exceed the shared-memory budget"); return SNAC_ERR_ARG; }
  for (int l = l0; l < P.nlev; l++)
    if (!LA<T>::invd(P.L[l]) && !(l == P.nlev - 1 && LA<T>::dinv(P.L[l]))) {
      set_error("coarse V-cycle needs the 1/diagonal tables");
      return SNAC_ERR_STATE;
    }
  SNAC_TRY(allow_smem((const void *)k_vcycle_coarse<T>, smem));
  prof_begin(KID_COARSE, st);
  SNAC_CUDA(launch_k(k_vcycle_coarse<T>, dim3(P.nsys), dim3(COARSE_THREADS), smem, st, P, plan, l0, shift, active, x, b));
  prof_end(KID_COARSE, st);
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

template <typename T>
size_t coarse3d_smem_bytes(const MgProblem &P, int l0) {
  size_t n = 0;
  for (int l = l0; l < P.nlev; l++) n += 2 * (size_t)P.L[l].ncell;
  return n * sizeof(T);
}

template <typename T>
int launch_vcycle_coarse3d(const MgProblem &P, const MgGeom &G, int l0, const T *shift, const int *active, T *x,
                           const T *b, cudaStream_t st) {
  const size_t smem = coarse3d_smem_bytes<T>(P, l0);
  if (smem > MG_COARSE3D_SMEM_MAX) { set_error("coarse levels exceed the shared-memory budget"); return SNAC_ERR_ARG; }
  SNAC_TRY(allow_smem((const void *)k_vcycle_coarse3d<T>, smem));
  prof_begin(KID_COARSE, st);
  k_vcycle_coarse3d<T><<<P.nsys, COARSE_THREADS, smem, st>>>(P, G, l0, shift, active, x, b), ::snac::count_launch();
  prof_end(KID_COARSE, st);
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

template size_t coarse3d_smem_bytes<double>(const MgProblem &, int);
template size_t coarse3d_smem_bytes<float>(const MgProblem &, int);
template int launch_vcycle_coarse3d<double>(const MgProblem &, const MgGeom &, int, const double *, const int *,
                                            double *, const double *, cudaStream_t);
template int launch_vcycle_coarse3d<float>(const MgProblem &, const MgGeom &, int, const float *, const int *, float *,
                                           const float *, cudaStream_t);

template int launch_rbgs_tile2d<double>(const MgProblem &, int, const int *, int, int, double *, const double *,
                                        const double *, const double *, double *, double *, double *, int, int *,
                                        cudaStream_t);
template int launch_rbgs_tile2d<float>(const MgProblem &, int, const int *, int, int, float *, const float *,
                                       const float *, const float *, double *, double *, double *, int, int *,
                                       cudaStream_t);
template int launch_rbgs_tile2d_restrict<float>(const MgProblem &, int, const int *, float *, const float *, float *,
                                                float *, cudaStream_t);
template size_t coarse_smem_bytes<double>(const MgProblem &, int);
template size_t coarse_smem_bytes<float>(const MgProblem &, int);
template int launch_vcycle_coarse<double>(const MgProblem &, int, const double *, const int *, double *,
                                          const double *, cudaStream_t);
template int launch_vcycle_coarse<float>(const MgProblem &, int, const float *, const int *, float *, const float *,
                                         cudaStream_t);

}  // namespace snac
