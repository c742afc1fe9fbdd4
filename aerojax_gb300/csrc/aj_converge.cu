// Converging multigrid: solves the reference's discrete pressure operator
// (5-point Laplacian with edge ghosts, outlet row pinned at 0; the operator of
// pressure_solvers/multigrid_solver.py:173-183) to ||b - A p||_2 <= rtol ||b||_2.
//
// Structure of one refinement iteration (one body of the graph's while node):
//   levels 0 .. lc-1   k_cv_down: 2 red-black sweeps from e = 0 in a shared-
//                      memory tile, residual, 2x2 restriction
//   levels lc .. D     k_cv_block: one 1024-thread block holding the smallest
//                      levels (<= 16384 cells) in shared memory: sweeps,
//                      restriction, the FP64 dense solve of the coarsest grid,
//                      prolongation, sweeps
//   levels lc-1 .. 1   k_cv_up: e += P(e_coarse), 2 red-black sweeps
//   level 0            k_cv_up0: e += P(e_coarse), 1 red-black sweep (a
//                      V(2,1) cycle on the fine grid: from the warm starts of
//                      a developed flow it ends in as many cycles as V(2,2)
//                      with a halo of 3 instead of 5), then p += e, the
//                      residual r = b - A p for the next iteration, its FP64
//                      norm, and (last block) the convergence test that sets
//                      the while node's condition with cudaGraphSetConditional
//
// Precision.  The V-cycle runs in FP32.  The refinement state p and the
// refinement residual are kept in double-FP32 ("double-single") arithmetic:
// p = hi + lo with |lo| <= ulp(hi)/2, updated and applied with the error-free
// transformations TwoSum (Knuth) and TwoProd (Dekker, via fma), which carry a
// ~48-bit significand on the FP32 pipes.  GB300 executes FP64 at 1/64 of the
// FP32 rate, and a plain-FP64 residual cost ~25 us per cycle at 2048x512.
// FP64 proper is kept where it is cheap: the coarsest-grid dense solve and the
// global norms that decide termination.
// The pressure state ping-pongs between two buffers (a tile's halo must see the
// old values while neighbouring tiles write the new ones).
// Coarse operators are rediscretised at spacing 2^l h; the outlet Dirichlet
// point stays where the fine grid has it (ghost g * e_last with
// g = (theta - 1) / theta, theta = (1 - 2^-l) / 2).  The oracle is
// oracle/ref_np.py mg_converge (FP64 throughout).
#include "aj_internal.cuh"
#include <math.h>
#include <string.h>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

namespace aj {

constexpr int CV_NS = 2;                         // red-black sweeps per smoothing phase
constexpr int CV_BLOCK_THREADS = 1024;
constexpr int CV_BLOCK_MAX_CELLS = 16384;        // levels handled by the one-block kernel

struct CvLvl {
  int n, m, level;
  float ax, ay, g;   // g: outlet ghost factor of this level (level >= 1)
};

static double ghost_factor(int level) {
  double th = 0.5 * (1.0 - pow(2.0, -level));
  return (th - 1.0) / th;
}

static CvLvl cv_level(const AjStepParams& p, const Layout& L, int l) {
  CvLvl c;
  c.n = L.ln[l];
  c.m = L.lm[l];
  c.level = l;
  double hx = p.dx * (double)(1 << l), hy = p.dy * (double)(1 << l);
  c.ax = (float)(1.0 / (hx * hx));
  c.ay = (float)(1.0 / (hy * hy));
  c.g = l > 0 ? (float)ghost_factor(l) : 0.f;
  return c;
}

// ---------------------------------------------------------------- double-FP32
// (df, two_sum, quick_two_sum, two_prod, df_add: aj_internal.cuh)
__device__ __forceinline__ df df_neg(df a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ df df_mul(df a, df b) {
  df p = two_prod(a.hi, b.hi);
  p.lo += a.hi * b.lo + a.lo * b.hi;
  return quick_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ df df_add_f(df a, float b) {
  df s = two_sum(a.hi, b);
  s.lo += a.lo;
  return quick_two_sum(s.hi, s.lo);
}
// Dekker's addition with one TwoSum: error <= ~2^-47 max(|a|, |b|), which in
// the residual below stays ~1e-14 |p| ax, far under the 1e-6 |b| targets
__device__ __forceinline__ df df_add_s(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  s.lo += a.lo + b.lo;
  return quick_two_sum(s.hi, s.lo);
}
// r = b - (ax ((xp + xm) - 2c) + ay ((yp + ym) - 2c)), all double-FP32 (-2c is
// exact, so each second difference costs two additions, not three)
__device__ __forceinline__ df df_residual(float b, df c, df xp, df xm, df yp, df ym, df ax, df ay) {
  const df c2{-2.f * c.hi, -2.f * c.lo};
  const df sx = df_add_s(df_add_s(xp, xm), c2);
  const df sy = df_add_s(df_add_s(yp, ym), c2);
  const df ap = df_add_s(df_mul(ax, sx), df_mul(ay, sy));
  return df_add_f(df_neg(ap), b);
}

// ---------------------------------------------------------------- paired double-FP32
// Two double-FP32 values side by side (a thread's two columns of a tile row)
// through the same error-free transformations on the paired FP32
// instructions (f2, add2, sub2: aj_internal.cuh).
struct df2 {
  float2 hi, lo;
};
__device__ __forceinline__ df2 two_sum2(float2 a, float2 b) {
  const float2 s = add2(a, b);
  const float2 bb = sub2(s, a);
  return {s, add2(sub2(a, sub2(s, bb)), sub2(b, bb))};
}
__device__ __forceinline__ df2 quick_two_sum2(float2 a, float2 b) {
  const float2 s = add2(a, b);
  return {s, sub2(b, sub2(s, a))};
}
__device__ __forceinline__ df2 df2_add_s(df2 a, df2 b) {   // as df_add_s
  df2 s = two_sum2(a.hi, b.hi);
  s.lo = add2(s.lo, add2(a.lo, b.lo));
  return quick_two_sum2(s.hi, s.lo);
}
__device__ __forceinline__ df2 df2_add_f(df2 a, float2 b) {   // as df_add_f
  df2 s = two_sum2(a.hi, b);
  s.lo = add2(s.lo, a.lo);
  return quick_two_sum2(s.hi, s.lo);
}
// a * b for one double-FP32 a: TwoProd by fma, whose error term is formed
// negated (fma(-a, b, p) = -(a b - p) exactly) and subtracted
__device__ __forceinline__ df2 df2_mul_u(df a, df2 b) {
  const float2 ah = f2(a.hi);
  const float2 p = __fmul2_rn(ah, b.hi);
  const float2 en = __ffma2_rn(f2(-a.hi), b.hi, p);
  const float2 cross = __ffma2_rn(ah, b.lo, __fmul2_rn(f2(a.lo), b.hi));
  return quick_two_sum2(p, sub2(cross, en));
}
// b - a: df_add_f(df_neg(a), b) with the signs carried through (negation
// is exact, so every rounding is the scalar form's)
__device__ __forceinline__ df2 df2_rsub_f(float2 b, df2 a) {
  const float2 s = sub2(b, a.hi);
  const float2 bb = add2(s, a.hi);
  const float2 e = sub2(sub2(b, bb), add2(a.hi, sub2(s, bb)));
  return quick_two_sum2(s, sub2(e, a.lo));
}
// df_residual for two cells
__device__ __forceinline__ df2 df2_residual(float2 b, df2 c, df2 xp, df2 xm, df2 yp, df2 ym,
                                            df ax, df ay) {
  const df2 c2{__fmul2_rn(c.hi, f2(-2.f)), __fmul2_rn(c.lo, f2(-2.f))};
  const df2 sx = df2_add_s(df2_add_s(xp, xm), c2);
  const df2 sy = df2_add_s(df2_add_s(yp, ym), c2);
  return df2_rsub_f(b, df2_add_s(df2_mul_u(ax, sx), df2_mul_u(ay, sy)));
}

struct DfCoef {
  float axh, axl, ayh, ayl;   // 1/dx^2 and 1/dy^2 split into hi + lo
};
static DfCoef df_coef(double ax, double ay) {
  DfCoef c;
  c.axh = (float)ax;
  c.axl = (float)(ax - (double)c.axh);
  c.ayh = (float)ay;
  c.ayl = (float)(ay - (double)c.ayh);
  return c;
}

// ---------------------------------------------------------------- tiles
// A tile is SI x SJ cells of shared memory: the TI x TJ interior plus a halo
// of H = 2 NS + 1 cells (NS red-black sweeps, one cell for the residual).
// Threads form a (SJ/2) x RG grid: thread (tx, ty) owns the column pair
// {2tx, 2tx+1} and walks the rows ty, ty+RG, ...; in a red-black half-sweep
// exactly one cell of its pair per row has the colour being updated, so no
// index needs a division.
// VEC tiles (k_cv_up0 on a level whose rows are a multiple of 4 floats) are
// staged in 16-byte chunks: their shared rows start at the 16-byte column at
// or left of the tile's first one and are SJS = SJ + 4 floats long (the
// pressure window's rows, PJS, cover its TJ + 2 columns from the 16-byte
// column at or left of its first, in whole chunks), and the kernel indexes
// them through base pointers shifted by the offsets from those columns.
template <int SI_, int SJ_, int NTH_, int NS_ = CV_NS, bool VEC_ = false>
struct TileCfg {
  static constexpr int SI = SI_, SJ = SJ_, NTH = NTH_, NS = NS_, H = 2 * NS_ + 1;
  static constexpr bool VEC = VEC_;
  static constexpr int TI = SI - 2 * H, TJ = SJ - 2 * H;
  static constexpr int SJS = VEC ? SJ + 4 : SJ;
  static constexpr int PJS = VEC ? (TJ + 2 + 3 + 3) / 4 * 4 : TJ + 2;
  static constexpr int PAIRS = SJ / 2, RG = NTH / PAIRS, NT = SI * SJS;
  static_assert(!VEC || SJ % 4 == 0, "a 16-byte staged row is whole chunks");
  static_assert(TI % 2 == 0 && TJ % 2 == 0, "tile interiors must align with the coarse grid");
  static_assert(NTH % PAIRS == 0, "threads must fill whole rows of column pairs");
};
using T0 = TileCfg<48, 64, 256>;   // level 0: 38 x 54 interior (default)
using T0b = TileCfg<32, 64, 256>;  // level 0: 22 x 54 interior (more, shorter tiles)
using T0c = TileCfg<64, 32, 256>;  // level 0: 54 x 22 interior (narrow tiles)
using T1 = TileCfg<32, 32, 256>;   // coarser levels: 22 x 22 interior
// Level 0 post-smooths with one sweep (a V(2,1) cycle on the fine grid,
// V(2,2) below it): the same tiles with a halo of 3
constexpr int CV_NS_UP0 = 1;
using T0u = TileCfg<48, 64, 256, CV_NS_UP0>;    // 42 x 58 interior
using T0bu = TileCfg<32, 64, 256, CV_NS_UP0>;   // 26 x 58 interior
using T0cu = TileCfg<64, 32, 256, CV_NS_UP0>;   // 58 x 26 interior
using T0uv = TileCfg<48, 64, 256, CV_NS_UP0, true>;
using T0buv = TileCfg<32, 64, 256, CV_NS_UP0, true>;
using T0cuv = TileCfg<64, 32, 256, CV_NS_UP0, true>;
constexpr int CV_TILE_VARIANTS = 3;

__device__ __forceinline__ float cv_diag(const CvLvl& L, int gi, int gj) {
  float d = -2.f * (L.ax + L.ay);
  if (gi == 0) d += L.ax;
  if (gj == 0) d += L.ay;
  if (gj == L.m - 1) d += L.ay;
  if (gi == L.n - 1) d += (L.level == 0) ? L.ax : L.ax * L.g;
  return d;
}

// red-black half-sweeps over the whole shared-memory tile; cells outside the
// domain hold 0 and never change (the diagonal carries the ghost rule).  After
// half-sweep h the cells at distance >= h+1 from the tile border hold exact
// red-black values; the cells nearer the border are never stored.  Tiles start
// at even global coordinates, so a cell's colour is (ti + tj) & 1.
template <class TC, bool INTERIOR>
__device__ __forceinline__ void cv_sweeps_t(float* E, const float* R, const CvLvl& L, int gi0,
                                            int gj0) {
  constexpr int SJ = TC::SJ, SI = TC::SI;
  constexpr int ROWS = (SI - 2 + TC::RG - 1) / TC::RG;   // rows of a thread per half-sweep
  const int tx = threadIdx.x, ty = threadIdx.y;
  const float inv_int = 1.f / (-2.f * (L.ax + L.ay));
  for (int h = 0; h < 2 * TC::NS; ++h) {
    const int color = h & 1;
    // every new value of this thread's rows first, then the stores: a
    // half-sweep reads only the other colour, so no store can feed a load of
    // the same half-sweep, and the loads of all rows are in flight together
    float val[ROWS];
    int cc[ROWS];
#pragma unroll
    for (int q = 0; q < ROWS; ++q) {
      const int ti = 1 + ty + q * TC::RG;
      const int tj = 2 * tx + ((color + ti) & 1);
      const int gi = gi0 + ti, gj = gj0 + tj;
      const bool upd = ti < SI - 1 &&
                       (INTERIOR ? (tj >= 1 && tj < SJ - 1)
                                 : (tj >= 1 && tj < SJ - 1 && (unsigned)gi < (unsigned)L.n &&
                                    (unsigned)gj < (unsigned)L.m &&
                                    !(L.level == 0 && gi == L.n - 1)));
      cc[q] = -1;
      val[q] = 0.f;
      if (upd) {
        const int c = ti * TC::SJS + tj;
        const float nb = L.ax * (E[c + TC::SJS] + E[c - TC::SJS]) + L.ay * (E[c + 1] + E[c - 1]);
        float inv = inv_int;
        if (!INTERIOR && (gi == 0 || gj == 0 || gi == L.n - 1 || gj == L.m - 1))
          inv = 1.f / cv_diag(L, gi, gj);
        val[q] = (R[c] - nb) * inv;
        cc[q] = c;
      }
    }
#pragma unroll
    for (int q = 0; q < ROWS; ++q)
      if (cc[q] >= 0) E[cc[q]] = val[q];
    __syncthreads();
  }
}
// A tile whose every cell is an interior cell of the level (no boundary row
// or column, not the pinned outlet row) takes the sweep without the checks.
template <class TC>
__device__ __forceinline__ void cv_sweeps(float* E, const float* R, const CvLvl& L, int gi0,
                                          int gj0) {
  if (gi0 >= 1 && gj0 >= 1 && gi0 + TC::SI <= L.n - 1 && gj0 + TC::SJ <= L.m - 1)
    cv_sweeps_t<TC, true>(E, R, L, gi0, gj0);
  else
    cv_sweeps_t<TC, false>(E, R, L, gi0, gj0);
}

// The coarse cells a tile's cell-centred bilinear prolongation reads, with the
// ghost rules folded in: row -1 copies row 0 (inlet Neumann), row nc is
// g * row nc-1 (outlet ghost), columns clamp (wall Neumann).
template <class TC>
struct CoarseWin {
  static constexpr int R = TC::SI / 2 + 3, C = TC::SJ / 2 + 3;
};

template <class TC>
__device__ __forceinline__ void cv_load_coarse(float* W, int gi0, int gj0,
                                               const float* __restrict__ ec, int nc, int mc,
                                               float g) {
  using CW = CoarseWin<TC>;
  const int I0 = (gi0 >> 1) - 1, J0 = (gj0 >> 1) - 1;
  for (int t = threadIdx.y * blockDim.x + threadIdx.x; t < CW::R * CW::C;
       t += blockDim.x * blockDim.y) {
    const int a = t / CW::C, b = t - a * CW::C;
    int I = I0 + a;
    const int J = min(max(J0 + b, 0), mc - 1);
    float f = 1.f;
    if (I < 0) I = 0;
    if (I >= nc) {
      I = nc - 1;
      f = g;
    }
    float v = 0.f;
    if (I0 + a >= -1 && I0 + a <= nc) v = ldg(ec + (long)I * mc + J);
    W[t] = f == 1.f ? v : f * v;
  }
}

// tile + halo load for a pre-smoothing: E = 0, R = r; each row is read as
// two coalesced runs of SJ/2 floats
template <class TC>
__device__ __forceinline__ void cv_load_r(float* E, float* R, const CvLvl& L, int gi0, int gj0,
                                          const float* __restrict__ r) {
  constexpr int SJ = TC::SJ;
  const int tx = threadIdx.x, ty = threadIdx.y;
#pragma unroll
  for (int ti = ty; ti < TC::SI; ti += TC::RG) {
    const int gi = gi0 + ti;
    const bool row_in = (unsigned)gi < (unsigned)L.n;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int tj = tx + q * TC::PAIRS;
      const int gj = gj0 + tj;
      const bool in = row_in && (unsigned)gj < (unsigned)L.m;
      E[ti * SJ + tj] = 0.f;
      R[ti * SJ + tj] = in ? ldg(r + (long)gi * L.m + gj) : 0.f;
    }
  }
  __syncthreads();
}

// 4-byte asynchronous global-to-shared copy; zero-fill when !in (the source
// is then not read)
__device__ __forceinline__ void cv_cp4(float* dst, const float* src, bool in) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src),
               "r"(in ? 4 : 0));
}

// tile + halo of a post-smoothing, requested without waiting: R = r and
// E = e_in by cp.async (zero outside the level, e also on level 0's pinned
// outlet row), so that their round trip overlaps the coarse window's; the
// caller commits, waits, synchronises and then adds the prolongation
template <class TC>
__device__ __forceinline__ void cv_stage_async(float* E, float* R, const CvLvl& L, int gi0,
                                               int gj0, const float* __restrict__ r,
                                               const float* __restrict__ e_in) {
  const int tx = threadIdx.x, ty = threadIdx.y;
#pragma unroll
  for (int ti = ty; ti < TC::SI; ti += TC::RG) {
    const int gi = gi0 + ti;
    const bool row_in = (unsigned)gi < (unsigned)L.n;
    const bool row_e = row_in && !(L.level == 0 && gi == L.n - 1);
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int tj = tx + q * TC::PAIRS;
      const int gj = gj0 + tj;
      const bool in = row_in && (unsigned)gj < (unsigned)L.m;
      const long k = in ? (long)gi * L.m + gj : 0;
      cv_cp4(R + ti * TC::SJS + tj, r + k, in);
      cv_cp4(E + ti * TC::SJS + tj, e_in + k, in && row_e);
    }
  }
}

// 16-byte asynchronous copy, zero-filled when !in; both addresses 16-byte
// aligned (the caller's VEC tiles guarantee it)
__device__ __forceinline__ void cv_cp16(float* dst, const float* src, bool in) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src),
               "r"(in ? 16 : 0));
}

// cv_stage_async of a VEC tile: rows of SJS floats from global column x0 (a
// multiple of 4; the level's row length m is one too, so a chunk is wholly
// inside or outside the level)
template <class TC>
__device__ __forceinline__ void cv_stage_async_v(float* E, float* R, const CvLvl& L, int gi0,
                                                 int x0, const float* __restrict__ r,
                                                 const float* __restrict__ e_in, int tid) {
  constexpr int CH = TC::SJS / 4;
  for (int t = tid; t < TC::SI * CH; t += TC::NTH) {
    const int ti = t / CH, ch = t - ti * CH;
    const int gi = gi0 + ti, gx = x0 + 4 * ch;
    const bool in = (unsigned)gi < (unsigned)L.n && gx >= 0 && gx < L.m;
    const bool ine = in && !(L.level == 0 && gi == L.n - 1);
    const long k = in ? (long)gi * L.m + gx : 0;
    cv_cp16(R + ti * TC::SJS + 4 * ch, r + k, in);
    cv_cp16(E + ti * TC::SJS + 4 * ch, e_in + k, ine);
  }
}

// e += P(e_coarse) on the cells this thread staged: the cell-centred
// bilinear prolongation (weights 9/16, 3/16, 3/16, 1/16) from the coarse
// window W (after cv_load_coarse, the copies' wait and a barrier)
template <class TC>
__device__ __forceinline__ void cv_add_prolong(float* E, const CvLvl& L, int gi0, int gj0,
                                               const float* W) {
  using CW = CoarseWin<TC>;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int I0 = (gi0 >> 1) - 1, J0 = (gj0 >> 1) - 1;
#pragma unroll
  for (int ti = ty; ti < TC::SI; ti += TC::RG) {
    const int gi = gi0 + ti;
    if ((unsigned)gi >= (unsigned)L.n || (L.level == 0 && gi == L.n - 1)) continue;
    const int a = (gi >> 1) - I0, ai = (gi & 1) ? a + 1 : a - 1;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int tj = tx + q * TC::PAIRS;
      const int gj = gj0 + tj;
      if ((unsigned)gj >= (unsigned)L.m) continue;
      const int b = (gj >> 1) - J0, bj = (gj & 1) ? b + 1 : b - 1;
      const float c0 = W[a * CW::C + b], cx = W[ai * CW::C + b];
      const float cy = W[a * CW::C + bj], cxy = W[ai * CW::C + bj];
      float* e = E + ti * TC::SJS + tj;
      *e = *e + (9.f * c0 + 3.f * cx + 3.f * cy + cxy) * (1.f / 16.f);
    }
  }
}

// pre-smoothing from e = 0, residual, 2x2 average onto the coarse rhs.  On
// level 0 the residual alternates between two buffers (r0, r1) with the
// pressure state: *cur selects the one the last iteration wrote.
template <class TC>
__global__ void __launch_bounds__(TC::NTH) k_cv_down(CvLvl L, const float* r0, const float* r1,
                                                     const int* cur, float* __restrict__ e_out,
                                                     float* __restrict__ rc, const int* done) {
  pdl_wait();
  constexpr int SJ = TC::SJ, TI = TC::TI, TJ = TC::TJ;
  static_assert(!TC::VEC, "the pre-smoothing indexes its tile with stride SJ");
  if (*done) return;
  __shared__ float E[TC::NT];
  __shared__ float R[TC::NT];
  const int i0 = blockIdx.y * TI, j0 = blockIdx.x * TJ;
  const int gi0 = i0 - TC::H, gj0 = j0 - TC::H;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const float* r = (r1 && *cur) ? r1 : r0;
  cv_load_r<TC>(E, R, L, gi0, gj0, r);
  cv_sweeps<TC>(E, R, L, gi0, gj0);
  // store e and compute the residual on the tile interior (in place in R:
  // every residual of this thread first, then the stores, so that no store
  // holds back the next cell's loads)
  constexpr int DR = (TI + TC::RG - 1) / TC::RG;
  float res[DR][2];
  int rc_[DR][2];
#pragma unroll
  for (int it = 0; it < DR; ++it) {
    const int ti = TC::H + ty + it * TC::RG;
    const int gi = gi0 + ti;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int tj = TC::H + tx + q * TC::PAIRS;
      const int gj = gj0 + tj;
      rc_[it][q] = -1;
      res[it][q] = 0.f;
      if (ti >= TC::H + TI || gi >= L.n || tj >= TC::H + TJ || gj >= L.m) continue;
      const int c = ti * SJ + tj;
      e_out[(long)gi * L.m + gj] = E[c];
      if (!(L.level == 0 && gi == L.n - 1)) {
        const float nb = L.ax * (E[c + SJ] + E[c - SJ]) + L.ay * (E[c + 1] + E[c - 1]);
        res[it][q] = R[c] - (nb + cv_diag(L, gi, gj) * E[c]);
      }
      rc_[it][q] = c;
    }
  }
#pragma unroll
  for (int it = 0; it < DR; ++it)
#pragma unroll
    for (int q = 0; q < 2; ++q)
      if (rc_[it][q] >= 0) R[rc_[it][q]] = res[it][q];
  __syncthreads();
  const int mc = L.m >> 1, nc = L.n >> 1;
  for (int ci = ty; ci < TI / 2; ci += TC::RG) {
    const int I = (i0 >> 1) + ci;
    if (I >= nc) break;
    for (int cj = tx; cj < TJ / 2; cj += TC::PAIRS) {
      const int J = (j0 >> 1) + cj;
      if (J >= mc) break;
      const int c = (TC::H + 2 * ci) * SJ + TC::H + 2 * cj;
      rc[(long)I * mc + J] = 0.25f * (R[c] + R[c + SJ] + R[c + 1] + R[c + SJ + 1]);
    }
  }
}

// e + P(e_coarse), post-smoothing, store (levels >= 1)
template <class TC>
__global__ void __launch_bounds__(TC::NTH) k_cv_up(CvLvl L, const float* __restrict__ r,
                                                   const float* __restrict__ e_in,
                                                   const float* __restrict__ ec, int nc, int mc,
                                                   float gc, float* __restrict__ e_out,
                                                   const int* done) {
  pdl_wait();
  constexpr int SJ = TC::SJ, TI = TC::TI, TJ = TC::TJ;
  static_assert(!TC::VEC, "the level >= 1 post-smoothing indexes its tile with stride SJ");
  if (*done) return;
  __shared__ float E[TC::NT];
  __shared__ float R[TC::NT];
  const int i0 = blockIdx.y * TI, j0 = blockIdx.x * TJ;
  const int gi0 = i0 - TC::H, gj0 = j0 - TC::H;
  const int tx = threadIdx.x, ty = threadIdx.y;
  cv_stage_async<TC>(E, R, L, gi0, gj0, r, e_in);
  asm volatile("cp.async.commit_group;\n" ::);
  __shared__ float W[CoarseWin<TC>::R * CoarseWin<TC>::C];
  cv_load_coarse<TC>(W, gi0, gj0, ec, nc, mc, gc);
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  __syncthreads();
  cv_add_prolong<TC>(E, L, gi0, gj0, W);
  __syncthreads();
  cv_sweeps<TC>(E, R, L, gi0, gj0);
  for (int ti = TC::H + ty; ti < TC::H + TI; ti += TC::RG) {
    const int gi = gi0 + ti;
    if (gi >= L.n) break;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int tj = TC::H + tx + q * TC::PAIRS;
      const int gj = gj0 + tj;
      if (tj >= TC::H + TJ || gj >= L.m) continue;
      e_out[(long)gi * L.m + gj] = E[ti * SJ + tj];
    }
  }
}

struct CvCheck {
  double rtol;
  int max_cycles;
  int use_handle;
  cudaGraphConditionalHandle h;
};

// convergence bookkeeping after a V-cycle (device scalars; one thread).  All
// fields are loaded before any is stored: interleaved, every load waited for
// the store before it (a chain of dependent round trips at the end of the
// cycle's last kernel).
__device__ void cv_check_body(DevScalars* sc, const CvCheck& ck) {
  int done = sc->mg_done, cycles = sc->mg_cycles, err = sc->err, loops = sc->loops;
  const double bnorm = sc->bnorm, a0 = sc->acc[0];
  const int was_done = done;
  if (!was_done) {
    cycles += 1;
    const double nb = bnorm > 0.0 ? bnorm : 1.0;
    const double rel = sqrt(a0) / nb;
    sc->rel = rel;
    sc->abs_sq = a0;
    if (!isfinite(rel)) {
      err = AJ_ERR_NONFINITE;
      done = 1;
    } else if (rel <= ck.rtol) {
      done = 1;
    } else if (cycles >= ck.max_cycles) {
      err = AJ_ERR_NOT_CONVERGED;
      done = 1;
    }
  }
  sc->acc[0] = 0.0;
  if (ck.use_handle) {
    // independent bound on the while node: never more bodies than max_cycles + 1
    loops += 1;
    if (loops > ck.max_cycles + 1 && !done) {
      err = AJ_ERR_NOT_CONVERGED;
      done = 1;
    }
    sc->loops = loops;
  }
  sc->mg_cycles = cycles;
  sc->err = err;
  sc->mg_done = done;
  if (ck.use_handle) cudaGraphSetConditional(ck.h, done ? 0u : 1u);
}

// a ping-pong pair: the pressure state (each buffer N hi values followed by N
// lo values) or the level-0 residual (N floats each)
struct PState {
  float* a;   // buffer 0
  float* b;   // buffer 1
};

// level 0: e + P(e_coarse), post-smoothing, p += e (double-FP32, ping-pong), the
// residual of the reference operator for the next iteration (double-FP32), its
// FP64 norm, and the convergence test in the last block to finish.  The
// residual ping-pongs with the pressure (rs.a pairs with ps.a): a block reads
// the current residual over its tile and halo while its neighbours write the
// next one, so the two must never share a buffer.
template <class TC>
__global__ void __launch_bounds__(TC::NTH, 4) k_cv_up0(
    CvLvl L, PState rs, const float* __restrict__ e_in,
    const float* __restrict__ ec, int nc, int mc, float gc, PState ps, const float* __restrict__ b,
    DevScalars* sc, DfCoef co, CvCheck ck, int profile) {
  pdl_wait();
  constexpr int TI = TC::TI, TJ = TC::TJ, SJS = TC::SJS;
  constexpr int PI = TI + 2, PJ = TJ + 2, PJS = TC::PJS;
  static_assert(PJ <= 2 * TC::PAIRS, "the pressure window must fit two column runs");
  if (!profile && sc->mg_done) {
    // met before this body ran (the initial guess already satisfied the
    // tolerance, or the rhs is zero): every kernel of the body skipped its
    // work and no block reaches the convergence test, so end the loop here
    // (a body after a converged one never runs: the test set the condition)
    if (ck.use_handle && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 &&
        threadIdx.y == 0)
      cudaGraphSetConditional(ck.h, 0u);
    return;
  }
  __shared__ __align__(16) float E[TC::NT];
  __shared__ __align__(16) float R[TC::NT];
  __shared__ __align__(16) float PH[PI * PJS];
  __shared__ __align__(16) float PL[PI * PJS];
  __shared__ int am_last;
  const int i0 = blockIdx.y * TI, j0 = blockIdx.x * TJ;
  const int gi0 = i0 - TC::H, gj0 = j0 - TC::H;
  // the tile's and the window's first logical cells (VEC: the shared rows
  // start at the 16-byte column at or left of them)
  const int xe = TC::VEC ? (gj0 & ~3) : gj0;
  const int xw = TC::VEC ? ((j0 - 1) & ~3) : j0 - 1;
  float* const Es = E + (gj0 - xe);
  float* const Rs = R + (gj0 - xe);
  float* const PHs = PH + (j0 - 1 - xw);
  float* const PLs = PL + (j0 - 1 - xw);
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int tid = ty * TC::PAIRS + tx;
  const long N = (long)L.n * L.m;
  const int cur = sc->pcur;
  const float* __restrict__ pin = cur ? ps.b : ps.a;
  float* __restrict__ pout = cur ? ps.a : ps.b;
  const float* __restrict__ r = cur ? rs.b : rs.a;
  float* __restrict__ r_next = cur ? rs.a : rs.b;
  // Every global read is requested before the first wait, so that the block
  // pays one round trip: the tile of r and e (tile and halo) and the pressure
  // window (interior + 1) by cp.async straight into R, E, PH and PL, b into
  // registers (this thread's residual cells: rows ty + RG q, columns tx and
  // tx + PAIRS), the coarse window by plain loads; the prolongation is then
  // added to E in shared memory.
  if constexpr (TC::VEC) {
    cv_stage_async_v<TC>(E, R, L, gi0, xe, r, e_in, tid);
    constexpr int PCH = PJS / 4;
    for (int t = tid; t < PI * PCH; t += TC::NTH) {
      const int pi = t / PCH, ch = t - pi * PCH;
      const int gi = i0 - 1 + pi, gx = xw + 4 * ch;
      const bool in = (unsigned)gi < (unsigned)L.n && gi != L.n - 1 && gx >= 0 && gx < L.m;
      const long k = in ? (long)gi * L.m + gx : 0;
      cv_cp16(PH + pi * PJS + 4 * ch, pin + k, in);
      cv_cp16(PL + pi * PJS + 4 * ch, pin + N + k, in);
    }
  } else {
    cv_stage_async<TC>(E, R, L, gi0, gj0, r, e_in);
    for (int pi = ty; pi < PI; pi += TC::RG) {
      const int gi = i0 - 1 + pi;
      const bool row_in = (unsigned)gi < (unsigned)L.n && gi != L.n - 1;
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int pj = tx + q * TC::PAIRS;
        if (pj >= PJ) continue;
        const int gj = j0 - 1 + pj;
        const bool in = row_in && (unsigned)gj < (unsigned)L.m;
        const long k = in ? (long)gi * L.m + gj : 0;
        cv_cp4(PH + pi * PJS + pj, pin + k, in);
        cv_cp4(PL + pi * PJS + pj, pin + N + k, in);
      }
    }
  }
  asm volatile("cp.async.commit_group;\n" ::);
  constexpr int RQ = (TI + TC::RG - 1) / TC::RG;
  float bpre[RQ][2];
#pragma unroll
  for (int it = 0; it < RQ; ++it) {
    const int ti = ty + it * TC::RG, gi = i0 + ti;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int tj = tx + q * TC::PAIRS, gj = j0 + tj;
      bpre[it][q] = (ti < TI && gi < L.n && tj < TJ && gj < L.m) ? ldg(b + (long)gi * L.m + gj) : 0.f;
    }
  }
  __shared__ float W[CoarseWin<TC>::R * CoarseWin<TC>::C];
  cv_load_coarse<TC>(W, gi0, gj0, ec, nc, mc, gc);
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  __syncthreads();
  cv_add_prolong<TC>(Es, L, gi0, gj0, W);
  __syncthreads();
  cv_sweeps<TC>(Es, Rs, L, gi0, gj0);
  // new pressure on the interior and one cell around it, the thread's two
  // columns of a row as one pair (all of this thread's sums first, then the
  // stores)
  constexpr int PR = (PI + TC::RG - 1) / TC::RG;
  df2 pv[PR];
  int pt[PR][2];
#pragma unroll
  for (int it = 0; it < PR; ++it) {
    const int pi = ty + it * TC::RG;
    const int gi = i0 - 1 + pi;
    const bool row_in = pi < PI && (unsigned)gi < (unsigned)L.n && gi != L.n - 1;
    float h[2], l[2], e[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int pj = tx + q * TC::PAIRS;
      const int gj = j0 - 1 + pj;
      pt[it][q] = -1;
      h[q] = l[q] = e[q] = 0.f;
      if (row_in && pj < PJ && (unsigned)gj < (unsigned)L.m) {
        const int t = pi * PJS + pj;
        h[q] = PHs[t];
        l[q] = PLs[t];
        e[q] = Es[(TC::H - 1 + pi) * SJS + (TC::H - 1 + pj)];
        pt[it][q] = t;
      }
    }
    pv[it] = df2_add_f(df2{make_float2(h[0], h[1]), make_float2(l[0], l[1])},
                       make_float2(e[0], e[1]));
  }
#pragma unroll
  for (int it = 0; it < PR; ++it) {
    if (pt[it][0] >= 0) {
      PHs[pt[it][0]] = pv[it].hi.x;
      PLs[pt[it][0]] = pv[it].lo.x;
    }
    if (pt[it][1] >= 0) {
      PHs[pt[it][1]] = pv[it].hi.y;
      PLs[pt[it][1]] = pv[it].lo.y;
    }
  }
  __syncthreads();
  const df ax{co.axh, co.axl}, ay{co.ayh, co.ayl};
  float acc = 0.f;
#pragma unroll
  for (int it = 0; it < RQ; ++it) {
    const int ti = ty + it * TC::RG;
    const int gi = i0 + ti;
    if (ti >= TI || gi >= L.n) break;
    // the row's two columns tx and tx + PAIRS; a column outside the tile or
    // the grid reads the row's first window cell (in bounds) and stores nothing
    bool ok[2];
    long k[2];
    df pc[2], xp[2], xm[2], yp[2], ym[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int tj = tx + q * TC::PAIRS;
      const int gj = j0 + tj;
      ok[q] = tj < TJ && gj < L.m;
      k[q] = (long)gi * L.m + gj;
      const int c = (ti + 1) * PJS + (ok[q] ? tj + 1 : 1);
      pc[q] = df{PHs[c], PLs[c]};
      xp[q] = df{PHs[c + PJS], PLs[c + PJS]};                    // row n-1 holds the pinned 0
      xm[q] = gi > 0 ? df{PHs[c - PJS], PLs[c - PJS]} : pc[q];   // Neumann ghosts
      yp[q] = gj < L.m - 1 ? df{PHs[c + 1], PLs[c + 1]} : pc[q];
      ym[q] = gj > 0 ? df{PHs[c - 1], PLs[c - 1]} : pc[q];
      if (ok[q]) {
        pout[k[q]] = pc[q].hi;
        pout[N + k[q]] = pc[q].lo;
      }
    }
    float rr[2] = {0.f, 0.f};
    if (gi != L.n - 1) {
      auto pair = [](const df* v) {
        return df2{make_float2(v[0].hi, v[1].hi), make_float2(v[0].lo, v[1].lo)};
      };
      const df2 res = df2_residual(make_float2(bpre[it][0], bpre[it][1]), pair(pc), pair(xp),
                                   pair(xm), pair(yp), pair(ym), ax, ay);
      const float2 s = add2(res.hi, res.lo);
      rr[0] = s.x;
      rr[1] = s.y;
    }
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      if (!ok[q]) continue;
      if (!profile) r_next[k[q]] = rr[q];
      acc = fmaf(rr[q], rr[q], acc);
    }
  }
  if (profile) return;
  block_sum_atomic_f(acc, &sc->acc[0]);
  if (tid == 0) {
    __threadfence();
    unsigned int ticket = atomicAdd(&sc->red_count, 1u);
    am_last = ticket == gridDim.x * gridDim.y - 1;
  }
  __syncthreads();
  if (am_last && tid == 0) {
    __threadfence();
    sc->red_count = 0u;
    sc->pcur = 1 - cur;
    cv_check_body(sc, ck);
  }
}

struct CvBlock {
  int lc, D, ncoarse, pre;
  int n[AJ_MAX_LEVELS + 1], m[AJ_MAX_LEVELS + 1];
  int eoff[AJ_MAX_LEVELS + 1], roff[AJ_MAX_LEVELS + 1], voff;   // shared-memory float offsets
  float ax[AJ_MAX_LEVELS + 1], ay[AJ_MAX_LEVELS + 1], g[AJ_MAX_LEVELS + 1];
  const float* r_in;      // rhs of level lc (global)
  float* e_out;           // correction of level lc (global)
  const double* Ainv;     // coarsest inverse, row-major ncoarse^2
  const int* done;
};

// shared-memory footprint of levels lc..D: e with a one-cell zero border and
// r, per level, plus the FP64 vector of the dense coarsest solve
static size_t block_levels_smem(const Layout& L, int lc) {
  size_t s = 0;
  for (int k = lc; k <= L.nlev; ++k)
    s += ((size_t)(L.ln[k] + 2) * (L.lm[k] + 2) + (size_t)L.ln[k] * L.lm[k]) * 4;
  s = (s + 15) & ~(size_t)15;
  const size_t N = (size_t)L.ln[L.nlev] * L.lm[L.nlev];
  return s + N * 8;
}
// whether the coarsest inverse is copied to shared memory (when it fits)
static bool block_prefetch(const Layout& L, int lc) {
  const size_t N = (size_t)L.ln[L.nlev] * L.lm[L.nlev];
  return N <= AJ_MAX_COARSE && block_levels_smem(L, lc) + N * N * 8 <= kBlockSmemMax;
}
size_t converge_block_smem(const Layout& L, int lc) {
  const size_t N = (size_t)L.ln[L.nlev] * L.lm[L.nlev];
  return block_levels_smem(L, lc) + (block_prefetch(L, lc) ? N * N * 8 : 0);
}

// A thread's place in a (rows x w) sweep of the block: column tx, first row
// ty, row stride rs (threads beyond rs * w rows idle).
struct Lane2 {
  int tx, ty, rs;
};
__device__ __forceinline__ Lane2 lane2(int w) {
  Lane2 l;
  l.tx = threadIdx.x % w;
  l.ty = threadIdx.x / w;
  l.rs = blockDim.x / w;
  return l;
}

__device__ __forceinline__ float blk_inv_diag(int i, int j, int n, int m, float ax, float ay,
                                              float g, float inv_int) {
  if (i > 0 && i < n - 1 && j > 0 && j < m - 1) return inv_int;
  float dd = -2.f * (ax + ay);
  if (i == 0) dd += ax;
  if (j == 0) dd += ay;
  if (j == m - 1) dd += ay;
  if (i == n - 1) dd += ax * g;
  return __frcp_rn(dd);
}

// red-black sweeps of one level held in shared memory (E bordered, R not)
__device__ __forceinline__ void blk_sweeps(float* E, const float* R, int n, int m, float ax,
                                           float ay, float g) {
  const int W = m + 2, hw = (m + 1) >> 1;
  const Lane2 q = lane2(hw);
  const float inv_int = 1.f / (-2.f * (ax + ay));
  for (int h = 0; h < 2 * CV_NS; ++h) {
    const int color = h & 1;
    if (q.ty < q.rs) {
      for (int i = q.ty; i < n; i += q.rs) {
        const int j = ((color + i) & 1) + 2 * q.tx;
        if (j >= m) continue;
        const int c = (i + 1) * W + (j + 1);
        const float nb = ax * (E[c + W] + E[c - W]) + ay * (E[c + 1] + E[c - 1]);
        E[c] = (R[i * m + j] - nb) * blk_inv_diag(i, j, n, m, ax, ay, g, inv_int);
      }
    }
    __syncthreads();
  }
}

// Levels lc..D in one block of CV_BLOCK_THREADS threads, every level resident
// in shared memory: pre-smoothing, residual and restriction down to the
// coarsest grid, its FP64 dense solve, prolongation and post-smoothing back
// to level lc.  Replaces 2 (D - lc) launches of the tile kernels by one.
__global__ void __launch_bounds__(CV_BLOCK_THREADS) k_cv_block(CvBlock a) {
  pdl_wait();
  if (*a.done) return;
  extern __shared__ __align__(16) float smf[];
  // level arrays are addressed from smf directly so that every access is a
  // shared-memory access
  auto E = [&](int k) { return smf + a.eoff[k]; };
  auto R = [&](int k) { return smf + a.roff[k]; };
  double* V = reinterpret_cast<double*>(smf + a.voff);
  double* Ainv_s = V + a.ncoarse;
  // start loading the coarsest inverse now, so its latency hides behind the
  // smoothing of the finer levels
  if (a.pre)
    for (int t = threadIdx.x; t < a.ncoarse * a.ncoarse; t += blockDim.x) Ainv_s[t] = a.Ainv[t];
  for (int k = a.lc; k <= a.D; ++k) {
    float* e = E(k);
    const int cnt = (a.n[k] + 2) * (a.m[k] + 2);
    for (int t = threadIdx.x; t < cnt; t += blockDim.x) e[t] = 0.f;
  }
  {
    const int cnt = a.n[a.lc] * a.m[a.lc];
    float* r0 = R(a.lc);
    for (int t = threadIdx.x; t < cnt; t += blockDim.x) r0[t] = ldg(a.r_in + t);
  }
  __syncthreads();
  // down: smooth, residual, restrict (coarse cell = average of 4 fine residuals)
  for (int k = a.lc; k < a.D; ++k) {
    const int n = a.n[k], m = a.m[k], W = m + 2;
    const float ax = a.ax[k], ay = a.ay[k], g = a.g[k];
    blk_sweeps(E(k), R(k), n, m, ax, ay, g);
    const int nc = n >> 1, mc = m >> 1;
    const Lane2 q = lane2(mc);
    const float* e = E(k);
    const float* rk = R(k);
    float* rk1 = R(k + 1);
    if (q.ty < q.rs) {
      for (int I = q.ty; I < nc; I += q.rs) {
        const int J = q.tx;
        float s = 0.f;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int i = 2 * I + (u & 1), j = 2 * J + (u >> 1);
          const int c = (i + 1) * W + (j + 1);
          float dd = -2.f * (ax + ay);
          if (i == 0) dd += ax;
          if (j == 0) dd += ay;
          if (j == m - 1) dd += ay;
          if (i == n - 1) dd += ax * g;
          const float Ae = ax * (e[c + W] + e[c - W]) + ay * (e[c + 1] + e[c - 1]) + dd * e[c];
          s += rk[i * m + j] - Ae;
        }
        rk1[I * mc + J] = 0.25f * s;
      }
    }
    __syncthreads();
  }
  // coarsest: e = A^-1 r in FP64 (one warp per row)
  {
    const int m = a.m[a.D], W = m + 2, N = a.ncoarse;
    const float* rD = R(a.D);
    float* eD = E(a.D);
    for (int t = threadIdx.x; t < N; t += blockDim.x) V[t] = (double)rD[t];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int row = warp; row < N; row += nw) {
      const double* arow = (a.pre ? Ainv_s : a.Ainv) + (long)row * N;
      double s = 0.0;
      for (int c = lane; c < N; c += 32) s += arow[c] * V[c];
      s = warp_sum(s);
      if (lane == 0) {
        const int i = row / m, j = row - i * m;
        eD[(i + 1) * W + (j + 1)] = (float)s;
      }
    }
    __syncthreads();
  }
  // up: prolong, smooth
  for (int k = a.D - 1; k >= a.lc; --k) {
    const int n = a.n[k], m = a.m[k], W = m + 2;
    const int nc = a.n[k + 1], mc = a.m[k + 1], Wc = mc + 2;
    const float gc = a.g[k + 1];
    const float* Ec = E(k + 1);
    float* Ek = E(k);
    const Lane2 q = lane2(m);
    if (q.ty < q.rs) {
      for (int gi = q.ty; gi < n; gi += q.rs) {
        const int gj = q.tx;
        const int I = gi >> 1, J = gj >> 1;
        const int Ii = (gi & 1) ? I + 1 : I - 1;
        int Jj = (gj & 1) ? J + 1 : J - 1;
        Jj = Jj < 0 ? 0 : (Jj >= mc ? mc - 1 : Jj);
        const float c0 = Ec[(I + 1) * Wc + (J + 1)], cy = Ec[(I + 1) * Wc + (Jj + 1)];
        float cx, cxy;
        if (Ii < 0) {
          cx = c0;
          cxy = cy;
        } else if (Ii >= nc) {
          cx = gc * c0;
          cxy = gc * cy;
        } else {
          cx = Ec[(Ii + 1) * Wc + (J + 1)];
          cxy = Ec[(Ii + 1) * Wc + (Jj + 1)];
        }
        Ek[(gi + 1) * W + (gj + 1)] += (9.f * c0 + 3.f * cx + 3.f * cy + cxy) * (1.f / 16.f);
      }
    }
    __syncthreads();
    blk_sweeps(Ek, R(k), n, m, a.ax[k], a.ay[k], a.g[k]);
  }
  {
    const int n = a.n[a.lc], m = a.m[a.lc], W = m + 2;
    const Lane2 q = lane2(m);
    const float* e0 = E(a.lc);
    if (q.ty < q.rs)
      for (int i = q.ty; i < n; i += q.rs) a.e_out[(long)i * m + q.tx] = e0[(i + 1) * W + q.tx + 1];
  }
}

// ---------------------------------------------------------------- direct coarse solve
// The rediscretised operator of level ld is separable: A = ax Tx (x) I +
// ay I (x) Ty, with Ty the 1-D Neumann-Neumann Laplacian (edge ghosts at both
// walls) and Tx the 1-D operator with an edge ghost at the inlet and the
// outlet ghost g * e_last.  The orthonormal DCT-II basis diagonalises Ty
// (eigenvalues -4 sin^2(pi k / 2m)), so A e = r splits into m independent
// tridiagonal systems (ax Tx + ay lambda_k) e_k = r_k in x, one per cosine
// mode, solved here by parallel cyclic reduction.  The whole coarse part of
// the V-cycle below level ld is replaced by this exact solve: a cosine
// transform (k_cv_dfwd), the m tridiagonal solves (k_cv_dpcr) and the inverse
// transform (k_cv_dbwd).
constexpr int CV_DIRECT_MAX_CELLS = 65536;
constexpr int CV_DIRECT_MAX_M = 128;
constexpr int CV_DIRECT_MAX_N = 1024;

struct CvDirect {
  int n, m;
  float ax, g;
  const float* r;      // level-ld rhs [n][m]
  const float* cy;     // cosine basis Cy[k][j] (orthonormal DCT-II)
  const float* ly;     // ay * lambda_k
  float* rhat;         // mode coefficients of r, transposed [m][n]
  float* ehat;         // mode coefficients of e, transposed [m][n]
  float* e;            // level-ld correction [n][m]
  const int* done;
};

int converge_direct_level(const Layout& L) {
  for (int l = 1; l <= L.nlev; ++l) {
    const long cells = (long)L.ln[l] * L.lm[l];
    if (cells <= CV_DIRECT_MAX_CELLS && L.lm[l] <= CV_DIRECT_MAX_M && L.ln[l] <= CV_DIRECT_MAX_N &&
        L.ln[l] >= 2)
      return l;
  }
  return 0;
}

// rhat[k][i] = sum_j Cy[k][j] r[i][j]: 32 x 32 output tiles; both operand
// panels (32 x m, m <= 128) are staged whole, so the block waits for global
// memory once; thread (tx, ty) owns i = i0 + tx and the modes k0 + ty + 8q
constexpr int CV_DT = 32;
constexpr int CV_DK = CV_DIRECT_MAX_M + 1;
__global__ void __launch_bounds__(256) k_cv_dfwd(CvDirect a) {
  pdl_wait();
  if (*a.done) return;
  __shared__ float Cs[CV_DT][CV_DK];
  __shared__ float Rs[CV_DT][CV_DK];
  const int n = a.n, m = a.m;
  const int i0 = blockIdx.x * CV_DT, k0 = blockIdx.y * CV_DT;
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int rr = ty; rr < CV_DT; rr += 8) {
    const int k = k0 + rr, i = i0 + rr;
    for (int j = tx; j < m; j += CV_DT) {
      Cs[rr][j] = k < m ? ldg(a.cy + (long)k * m + j) : 0.f;
      Rs[rr][j] = i < n ? ldg(a.r + (long)i * m + j) : 0.f;
    }
  }
  __syncthreads();
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 8
  for (int j = 0; j < m; ++j) {
    const float rv = Rs[tx][j];
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[q] = fmaf(Cs[ty + 8 * q][j], rv, acc[q]);
  }
  const int i = i0 + tx;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int k = k0 + ty + 8 * q;
    if (i < n && k < m) a.rhat[(long)k * n + i] = acc[q];
  }
}

// one block per cosine mode k: parallel cyclic reduction of
// (ax Tx + ay lambda_k) ehat_k = rhat_k, n unknowns along x
__global__ void __launch_bounds__(1024) k_cv_dpcr(CvDirect a) {
  pdl_wait();
  if (*a.done) return;
  extern __shared__ __align__(16) float sh[];
  const int n = a.n, k = blockIdx.x;
  float* A0 = sh;
  float* B0 = A0 + n;
  float* C0 = B0 + n;
  float* D0 = C0 + n;
  float* A1 = D0 + n;
  float* B1 = A1 + n;
  float* C1 = B1 + n;
  float* D1 = C1 + n;
  const int i = threadIdx.x;
  const float lyk = ldg(a.ly + k);
  if (i < n) {
    float dx = -2.f;
    if (i == 0) dx += 1.f;
    if (i == n - 1) dx += a.g;
    A0[i] = i > 0 ? a.ax : 0.f;
    C0[i] = i < n - 1 ? a.ax : 0.f;
    B0[i] = fmaf(a.ax, dx, lyk);
    D0[i] = ldg(a.rhat + (long)k * n + i);
  }
  __syncthreads();
  float *Ac = A0, *Bc = B0, *Cc = C0, *Dc = D0, *An = A1, *Bn = B1, *Cn = C1, *Dn = D1;
  for (int st = 1; st < n; st <<= 1) {
    if (i < n) {
      const float ai = Ac[i], bi = Bc[i], ci = Cc[i], di = Dc[i];
      float an = 0.f, bn = bi, cn = 0.f, dn = di;
      if (i - st >= 0) {
        const float k1 = ai / Bc[i - st];
        an = -Ac[i - st] * k1;
        bn -= Cc[i - st] * k1;
        dn -= Dc[i - st] * k1;
      }
      if (i + st < n) {
        const float k2 = ci / Bc[i + st];
        cn = -Cc[i + st] * k2;
        bn -= Ac[i + st] * k2;
        dn -= Dc[i + st] * k2;
      }
      An[i] = an;
      Bn[i] = bn;
      Cn[i] = cn;
      Dn[i] = dn;
    }
    __syncthreads();
    float* t;
    t = Ac; Ac = An; An = t;
    t = Bc; Bc = Bn; Bn = t;
    t = Cc; Cc = Cn; Cn = t;
    t = Dc; Dc = Dn; Dn = t;
  }
  if (i < n) a.ehat[(long)k * n + i] = Dc[i] / Bc[i];
}

// e[i][j] = sum_k ehat[k][i] Cy[k][j]: 32 x 32 output tiles, both m x 32
// operand panels staged whole; thread (tx, ty) owns j = j0 + tx and the rows
// i0 + ty + 8q
__global__ void __launch_bounds__(256) k_cv_dbwd(CvDirect a) {
  pdl_wait();
  if (*a.done) return;
  __shared__ float Es[CV_DIRECT_MAX_M][CV_DT + 1];
  __shared__ float Cs[CV_DIRECT_MAX_M][CV_DT + 1];
  const int n = a.n, m = a.m;
  const int j0 = blockIdx.x * CV_DT, i0 = blockIdx.y * CV_DT;
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int k = ty; k < m; k += 8) {
    const int i = i0 + tx, j = j0 + tx;
    Es[k][tx] = i < n ? ldg(a.ehat + (long)k * n + i) : 0.f;
    Cs[k][tx] = j < m ? ldg(a.cy + (long)k * m + j) : 0.f;
  }
  __syncthreads();
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 8
  for (int k = 0; k < m; ++k) {
    const float cv = Cs[k][tx];
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[q] = fmaf(Es[k][ty + 8 * q], cv, acc[q]);
  }
  const int j = j0 + tx;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int i = i0 + ty + 8 * q;
    if (i < n && j < m) a.e[(long)i * m + j] = acc[q];
  }
}

static void direct_launch(const CvDirect& d, cudaStream_t st) {
  launch_pdl(true, k_cv_dfwd, dim3(cdiv(d.n, CV_DT), cdiv(d.m, CV_DT)), dim3(CV_DT, 8), 0, st, d);
  launch_pdl(true, k_cv_dpcr, dim3(d.m), dim3(cdiv(d.n, 32) * 32), 8 * d.n * sizeof(float), st, d);
  launch_pdl(true, k_cv_dbwd, dim3(cdiv(d.m, CV_DT), cdiv(d.n, CV_DT)), dim3(CV_DT, 8), 0, st, d);
}

static CvDirect direct_args(const AjStepParams& p, const Layout& L, void* ws, const int* done);

// ---------------------------------------------------------------- set-up / solve
// The initial double-FP32 state, outlet row pinned; a block per 8 rows.
// With a history (warm start AJ_WARM_EXTRAPOLATE) of two solutions
// p = p1 + (dt / dt1) (p1 - p2), of one solution p = p1; else p0 (or 0).
struct CvHist {
  const float* h;   // two slots of N hi values followed by N lo values; null: none
  long N;
};
constexpr int CV_ROWS = 8;   // rows per block of the whole-grid kernels (unrolled)

// The extrapolation history as this solve sees it: a solve that finished
// since the last commit (hist_pending) has filed its solution in the other
// slot.  The last block of k_cv_resid commits the rotation.
struct HistView {
  int cur, n;
  float dtp;
};
__device__ __forceinline__ HistView hist_view(const DevScalars* sc) {
  // all five fields loaded unconditionally (one round trip), then selected
  const int pend = sc->hist_pending, cur = sc->hist_cur, n = sc->hist_n;
  const float dtl = sc->dt_last, dtp = sc->dt_prev;
  HistView h;
  if (pend) {
    h.cur = 1 - cur;
    h.n = n < 2 ? n + 1 : 2;
    h.dtp = dtl;
  } else {
    h.cur = cur;
    h.n = n;
    h.dtp = dtp;
  }
  return h;
}
__global__ void __launch_bounds__(256) k_cv_init(const float* __restrict__ p0,
                                                 float* __restrict__ ps, int n, int m, CvHist hs,
                                                 const DevScalars* sc) {
  pdl_wait();
  const long N = (long)n * m;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  const HistView hv = hist_view(sc);
  const int hn = hs.h ? hv.n : 0;
  const float* __restrict__ h1 = hs.h ? hs.h + (long)hv.cur * 2 * N : nullptr;
  const float* __restrict__ h2 = hs.h ? hs.h + (long)(1 - hv.cur) * 2 * N : nullptr;
  float ratio = 1.f;
  if (hn >= 2 && sc->dt > 0.f && hv.dtp > 0.f) ratio = sc->dt / hv.dtp;
  const int i0 = blockIdx.y * CV_ROWS;
  // every row's loads first (the stores below would otherwise hold each
  // row's loads back behind the previous row's stores)
  float a_hi[CV_ROWS], a_lo[CV_ROWS], b_hi[CV_ROWS], b_lo[CV_ROWS];
#pragma unroll
  for (int r = 0; r < CV_ROWS; ++r) {
    const int i = i0 + r;
    const long k = (long)i * m + j;
    a_hi[r] = a_lo[r] = b_hi[r] = b_lo[r] = 0.f;
    if (i < n - 1) {
      if (hn >= 1) {
        a_hi[r] = h1[k];
        a_lo[r] = h1[N + k];
      } else if (p0) {
        a_hi[r] = p0[k];
      }
      if (hn >= 2) {
        b_hi[r] = h2[k];
        b_lo[r] = h2[N + k];
      }
    }
  }
#pragma unroll
  for (int r = 0; r < CV_ROWS; ++r) {
    const int i = i0 + r;
    if (i < n) {
      const long k = (long)i * m + j;
      df v{a_hi[r], a_lo[r]};
      if (hn >= 2 && i != n - 1) {
        const df a = v, b{b_hi[r], b_lo[r]};
        v = df_add(a, df_mul(df{ratio, 0.f}, df_add(a, df_neg(b))));
      }
      ps[k] = v.hi;
      ps[N + k] = v.lo;
    }
  }
}

// residual of the reference operator before the first cycle (double-FP32)
// and the FP64 norms of r and b; a block per 8 rows
__global__ void __launch_bounds__(256) k_cv_resid(const float* __restrict__ ps,
                                                  const float* __restrict__ b,
                                                  float* __restrict__ r, int n, int m, DfCoef co,
                                                  DevScalars* sc, double rtol) {
  pdl_wait();
  const long N = (long)n * m;
  const df ax{co.axh, co.axl}, ay{co.ayh, co.ayl};
  float acc = 0.f, accb = 0.f;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < m) {
    const int i0 = blockIdx.y * CV_ROWS;
    // all loads first: the state at rows i0-1 .. i0+CV_ROWS (column j), the
    // column neighbours j-1, j+1 and b at rows i0 .. i0+CV_ROWS-1
    float ch[CV_ROWS + 2], cl[CV_ROWS + 2], yph[CV_ROWS], ypl[CV_ROWS], ymh[CV_ROWS],
        yml[CV_ROWS], bv[CV_ROWS];
#pragma unroll
    for (int q = 0; q < CV_ROWS + 2; ++q) {
      const int i = i0 - 1 + q;
      ch[q] = cl[q] = 0.f;
      if (i >= 0 && i < n) {
        const long k = (long)i * m + j;
        ch[q] = ps[k];
        cl[q] = ps[N + k];
      }
    }
#pragma unroll
    for (int q = 0; q < CV_ROWS; ++q) {
      const int i = i0 + q;
      yph[q] = ypl[q] = ymh[q] = yml[q] = bv[q] = 0.f;
      if (i < n - 1) {
        const long k = (long)i * m + j;
        if (j + 1 < m) {
          yph[q] = ps[k + 1];
          ypl[q] = ps[N + k + 1];
        }
        if (j > 0) {
          ymh[q] = ps[k - 1];
          yml[q] = ps[N + k - 1];
        }
        bv[q] = b[k];
      }
    }
#pragma unroll
    for (int q = 0; q < CV_ROWS; ++q) {
      const int i = i0 + q;
      if (i >= n) break;
      const long k = (long)i * m + j;
      float rr = 0.f;
      if (i != n - 1) {
        const df c{ch[q + 1], cl[q + 1]};
        const df xp{ch[q + 2], cl[q + 2]};
        const df xm = i > 0 ? df{ch[q], cl[q]} : c;
        const df yp = j + 1 < m ? df{yph[q], ypl[q]} : c;
        const df ym = j > 0 ? df{ymh[q], yml[q]} : c;
        const df res = df_residual(bv[q], c, xp, xm, yp, ym, ax, ay);
        rr = res.hi + res.lo;
        accb = fmaf(bv[q], bv[q], accb);
      }
      r[k] = rr;
      acc = fmaf(rr, rr, acc);
    }
  }
  block_sum_atomic_f(acc, &sc->acc[0]);
  block_sum_atomic_f(accb, &sc->acc[1]);
  // the last block: commit the history rotation, reset the solve's counters
  // and run the test before the first cycle (the guess may already satisfy rtol)
  __shared__ int am_last;
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned int ticket = atomicAdd(&sc->red_count, 1u);
    am_last = ticket == gridDim.x * gridDim.y - 1;
  }
  __syncthreads();
  if (am_last && threadIdx.x == 0) {
    __threadfence();
    // every field first, then the stores (see cv_check_body)
    const HistView hv = hist_view(sc);
    const double a0 = sc->acc[0], a1 = sc->acc[1];
    const double bnorm = sqrt(a1);
    const double nb = bnorm > 0.0 ? bnorm : 1.0;
    const double rel = sqrt(a0) / nb;
    int err = AJ_OK, done = 0;
    if (!isfinite(rel)) {
      err = AJ_ERR_NONFINITE;
      done = 1;
    } else if (rel <= rtol) {
      done = 1;
    }
    sc->hist_cur = hv.cur;
    sc->hist_n = hv.n;
    sc->dt_prev = hv.dtp;
    sc->hist_pending = 0;
    sc->red_count = 0u;
    sc->mg_cycles = 0;
    sc->loops = 0;
    sc->pcur = 0;
    sc->bnorm = bnorm;
    sc->rel = rel;
    sc->abs_sq = a0;
    sc->acc[0] = 0.0;
    sc->acc[1] = 0.0;
    sc->err = err;
    sc->mg_done = done;
  }
}

// p = hi + lo; with a history, the state also goes to the free slot (the
// next solve's k_cv_resid makes it the latest); thread 0 files the statistics
__global__ void k_cv_out(PState ps, DevScalars* sc, float* __restrict__ p, long N, float* hist,
                         AjStats* stats) {
  pdl_wait();
  long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const float* src = sc->pcur ? ps.b : ps.a;
  if (k < N) {
    const float hi = src[k], lo = src[N + k];
    p[k] = hi + lo;
    if (hist) {
      float* dst = hist + (long)(1 - sc->hist_cur) * 2 * N;
      dst[k] = hi;
      dst[N + k] = lo;
    }
  }
  if (k == 0) {
    // every field first, then the stores (stats may alias nothing the
    // compiler can prove, so interleaved each load waited for a store)
    const int cycles = sc->mg_cycles, done = sc->mg_done, err = sc->err;
    const double rel = sc->rel, bnorm = sc->bnorm, abs_sq = sc->abs_sq;
    const float dt = sc->dt;
    if (hist) {
      sc->hist_pending = 1;
      sc->dt_last = dt;
    }
    if (stats) {
      stats->cycles = cycles;
      stats->converged = done && err == AJ_OK;   // the tolerance met, not just the loop ended
      stats->err = err;
      stats->pad = 0;
      stats->rel_residual = rel;
      stats->rhs_norm = bnorm;
      stats->dt = dt;
      stats->abs_residual_sq = abs_sq;
    }
  }
}

static CvBlock block_args(const AjStepParams& p, const Layout& L, void* ws, const int* done) {
  CvBlock a;
  memset(&a, 0, sizeof(a));
  a.lc = L.lc;
  a.D = L.nlev;
  a.ncoarse = L.ncoarse;
  a.pre = block_prefetch(L, L.lc) ? 1 : 0;
  size_t off = 0;   // floats; the same order as block_levels_smem
  for (int k = L.lc; k <= L.nlev; ++k) {
    a.eoff[k] = (int)off;
    off += (size_t)(L.ln[k] + 2) * (L.lm[k] + 2);
    a.roff[k] = (int)off;
    off += (size_t)L.ln[k] * L.lm[k];
  }
  a.voff = (int)((off + 3) & ~(size_t)3);
  for (int k = 0; k <= L.nlev; ++k) {
    CvLvl c = cv_level(p, L, k);
    a.n[k] = c.n;
    a.m[k] = c.m;
    a.ax[k] = c.ax;
    a.ay[k] = c.ay;
    a.g[k] = c.g;
  }
  a.r_in = at<float>(ws, L.B[L.lc]);
  a.e_out = at<float>(ws, L.T[L.lc]);
  a.Ainv = at<double>(ws, L.cinv);
  a.done = done;
  return a;
}

static CvDirect direct_args(const AjStepParams& p, const Layout& L, void* ws, const int* done) {
  CvDirect d;
  const CvLvl c = cv_level(p, L, L.ld);
  d.n = c.n;
  d.m = c.m;
  d.ax = c.ax;
  d.g = c.g;
  d.r = at<float>(ws, L.B[L.ld]);
  d.cy = at<float>(ws, L.dcy);
  d.ly = at<float>(ws, L.dly);
  d.rhat = at<float>(ws, L.X[L.ld]);
  d.ehat = at<float>(ws, L.dtmp);
  d.e = at<float>(ws, L.T[L.ld]);
  d.done = done;
  return d;
}

static PState pstate(const Layout& L, void* ws) {
  return PState{at<float>(ws, L.p64), at<float>(ws, L.p64b)};
}

template <class TC>
static dim3 tiles(const CvLvl& c) {
  return dim3(cdiv(c.m, TC::TJ), cdiv(c.n, TC::TI));
}
template <class TC>
static dim3 tile_threads() {
  return dim3(TC::PAIRS, TC::RG);
}

// level-0 kernels of tile variant v (chosen per grid shape by the autotuner)
template <class TC>
static void level0_down(const CvLvl& c, const Layout& L, void* ws, const int* done,
                        cudaStream_t st) {
  const DevScalars* sc = at<DevScalars>(ws, 0);
  launch_pdl(true, k_cv_down<TC>, dim3(tiles<TC>(c)), dim3(tile_threads<TC>()), 0, st, c,
             at<float>(ws, L.B[0]), at<float>(ws, L.T[0]), &sc->pcur, at<float>(ws, L.X[0]),
             at<float>(ws, L.B[1]), done);
}
template <class TC>
static void level0_up(const AjStepParams& p, const CvLvl& c, const Layout& L, void* ws,
                      DevScalars* sc, const CvCheck& ck, int profile, cudaStream_t st) {
  launch_pdl(true, k_cv_up0<TC>, dim3(tiles<TC>(c)), dim3(tile_threads<TC>()), 0, st, c,
             PState{at<float>(ws, L.B[0]), at<float>(ws, L.T[0])}, at<float>(ws, L.X[0]),
             at<float>(ws, L.T[1]), L.ln[1], L.lm[1], (float)ghost_factor(1), pstate(L, ws),
             at<float>(ws, L.b0), sc, df_coef(1.0 / (p.dx * p.dx), 1.0 / (p.dy * p.dy)), ck,
             profile);
}
static void level0_down_v(int v, const CvLvl& c, const Layout& L, void* ws, const int* done,
                          cudaStream_t st) {
  if (v == 1) level0_down<T0b>(c, L, ws, done, st);
  else if (v == 2) level0_down<T0c>(c, L, ws, done, st);
  else level0_down<T0>(c, L, ws, done, st);
}
// the 16-byte staged tiles need rows of a multiple of 4 floats and every
// staged buffer 16-byte aligned (workspace offsets are multiples of 256)
static bool level0_vec_ok(const CvLvl& c, const void* ws) {
  return c.m % 4 == 0 && (reinterpret_cast<uintptr_t>(ws) & 15) == 0;
}
static void level0_up_v(int v, const AjStepParams& p, const CvLvl& c, const Layout& L, void* ws,
                        DevScalars* sc, const CvCheck& ck, int profile, cudaStream_t st) {
  const bool vec = level0_vec_ok(c, ws);
  if (v == 1) vec ? level0_up<T0buv>(p, c, L, ws, sc, ck, profile, st)
                  : level0_up<T0bu>(p, c, L, ws, sc, ck, profile, st);
  else if (v == 2) vec ? level0_up<T0cuv>(p, c, L, ws, sc, ck, profile, st)
                       : level0_up<T0cu>(p, c, L, ws, sc, ck, profile, st);
  else vec ? level0_up<T0uv>(p, c, L, ws, sc, ck, profile, st)
           : level0_up<T0u>(p, c, L, ws, sc, ck, profile, st);
}

// one refinement iteration
static void cv_body(const AjStepParams& p, const Layout& L, void* ws,
                    cudaGraphConditionalHandle h, int use_handle, cudaStream_t st) {
  DevScalars* sc = at<DevScalars>(ws, 0);
  const int* done = &sc->mg_done;
  const int lc = L.lc;
  for (int l = 0; l < lc; ++l) {
    CvLvl c = cv_level(p, L, l);
    if (l == 0)
      level0_down_v(tile_variant(p.nx, p.ny), c, L, ws, done, st);
    else
      launch_pdl(true, k_cv_down<T1>, dim3(tiles<T1>(c)), dim3(tile_threads<T1>()), 0, st, c,
                 at<float>(ws, L.B[l]), nullptr, done, at<float>(ws, L.X[l]),
                 at<float>(ws, L.B[l + 1]), done);
  }
  if (L.ld > 0) {
    direct_launch(direct_args(p, L, ws, done), st);
  } else {
    k_cv_block<<<1, CV_BLOCK_THREADS, converge_block_smem(L, lc), st>>>(block_args(p, L, ws, done));
  }
  for (int l = lc - 1; l >= 1; --l) {
    CvLvl c = cv_level(p, L, l);
    launch_pdl(true, k_cv_up<T1>, dim3(tiles<T1>(c)), dim3(tile_threads<T1>()), 0, st, c,
               at<float>(ws, L.B[l]), at<float>(ws, L.X[l]), at<float>(ws, L.T[l + 1]), L.ln[l + 1],
               L.lm[l + 1], (float)ghost_factor(l + 1), at<float>(ws, L.T[l]), done);
  }
  CvLvl c0 = cv_level(p, L, 0);
  CvCheck ck{p.mg_rtol, p.max_cycles, use_handle, h};
  level0_up_v(tile_variant(p.nx, p.ny), p, c0, L, ws, sc, ck, 0, st);
}

static cudaStream_t side_stream() {
  static cudaStream_t s = nullptr;
  if (!s) cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  return s;
}

// the initial double-FP32 state (needs the step's dt and the history, not
// the rhs: the step runs it beside the predictor)
int converge_init(const AjStepParams& p, const Layout& L, void* ws, const float* p0,
                  cudaStream_t st) {
  DevScalars* sc = at<DevScalars>(ws, 0);
  const long N = (long)p.nx * p.ny;
  const PState ps = pstate(L, ws);
  const dim3 rgrid(cdiv(p.ny, 256), cdiv(p.nx, CV_ROWS));
  const bool extrap = p.warm_start == AJ_WARM_EXTRAPOLATE && L.hist;
  CvHist hs{extrap ? at<float>(ws, L.hist) : nullptr, N};
  launch_pdl(true, k_cv_init, dim3(rgrid), dim3(256), 0, st, p.warm_start ? p0 : nullptr, ps.a,
             p.nx, p.ny, hs, (const DevScalars*)sc);
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

int converge_solve(const AjStepParams& p, const Layout& L, void* ws, const float* p0,
                   float* pout, cudaStream_t st, const NnWarm* nn, AjStats* stats,
                   bool init_done) {
  DevScalars* sc = at<DevScalars>(ws, 0);
  const long N = (long)p.nx * p.ny;
  const PState ps = pstate(L, ws);
  const dim3 rgrid(cdiv(p.ny, 256), cdiv(p.nx, CV_ROWS));
  const bool extrap = p.warm_start == AJ_WARM_EXTRAPOLATE && L.hist;
  if (!init_done) {
    const int rc = converge_init(p, L, ws, p0, st);
    if (rc != AJ_OK) return rc;
  }
  if (nn && nn->packed) {
    const int rc = nn_correct_state(p, L, ws, at<float>(ws, L.b0), *nn, ps.a, st);
    if (rc != AJ_OK) return rc;
  }
  launch_pdl(true, k_cv_resid, dim3(rgrid), dim3(256), 0, st, ps.a, at<float>(ws, L.b0),
             at<float>(ws, L.B[0]), p.nx, p.ny, df_coef(1.0 / (p.dx * p.dx), 1.0 / (p.dy * p.dy)),
             sc, p.mg_rtol);

  cudaStreamCaptureStatus cs;
  unsigned long long id;
  cudaGraph_t g;
  const cudaGraphNode_t* deps;
  const cudaGraphEdgeData* ed;
  size_t nd;
  if (cudaStreamGetCaptureInfo(st, &cs, &id, &g, &deps, &ed, &nd) != cudaSuccess)
    return AJ_ERR_CUDA;
  if (cs != cudaStreamCaptureStatusActive) {
    // eager launches (profiling mode): a fixed number of loop bodies, each
    // skipping its work once the target is met
    int unroll = eager_unroll(p.max_cycles);
    for (int k = 0; k < unroll; ++k) cv_body(p, L, ws, 0, 0, st);
  } else {
    // the refinement loop: a while node appended to the graph being captured
    cudaGraphConditionalHandle h;
    if (cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault) != cudaSuccess)
      return AJ_ERR_CUDA;
    // the params union has no default constructor: zero-initialised storage
    alignas(cudaGraphNodeParams) unsigned char npbuf[sizeof(cudaGraphNodeParams)];
    memset(npbuf, 0, sizeof(npbuf));
    cudaGraphNodeParams& np = *reinterpret_cast<cudaGraphNodeParams*>(npbuf);
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    if (cudaGraphAddNode(&node, g, deps, ed, nd, &np) != cudaSuccess) return AJ_ERR_CUDA;
    if (cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1,
                                            cudaStreamSetCaptureDependencies) != cudaSuccess)
      return AJ_ERR_CUDA;
    cudaGraph_t body = np.conditional.phGraph_out[0];
    cudaStream_t side = side_stream();
    if (cudaStreamBeginCaptureToGraph(side, body, nullptr, nullptr, 0,
                                      cudaStreamCaptureModeRelaxed) != cudaSuccess)
      return AJ_ERR_CUDA;
    cv_body(p, L, ws, h, 1, side);
    cudaGraph_t out;
    if (cudaStreamEndCapture(side, &out) != cudaSuccess) return AJ_ERR_CUDA;
  }
  launch_pdl(true, k_cv_out, dim3(cdiv(N, 256)), dim3(256), 0, st, ps, sc, pout, N,
             extrap ? at<float>(ws, L.hist) : nullptr, stats);
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

// dense matrix of the coarsest converging-mode operator, inverted on the host
static bool coarse_inverse(const AjStepParams& p, const Layout& L, std::vector<double>& inv) {
  const int l = L.nlev, n = L.ln[l], m = L.lm[l], N = n * m;
  double hx = p.dx * (double)(1 << l), hy = p.dy * (double)(1 << l);
  double ax = 1.0 / (hx * hx), ay = 1.0 / (hy * hy), g = ghost_factor(l);
  std::vector<double> A((size_t)N * N, 0.0);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < m; ++j) {
      int r = i * m + j;
      double d = -2.0 * (ax + ay);
      if (i == 0) d += ax; else A[(size_t)r * N + (i - 1) * m + j] += ax;
      if (i == n - 1) d += ax * g; else A[(size_t)r * N + (i + 1) * m + j] += ax;
      if (j == 0) d += ay; else A[(size_t)r * N + i * m + j - 1] += ay;
      if (j == m - 1) d += ay; else A[(size_t)r * N + i * m + j + 1] += ay;
      A[(size_t)r * N + r] += d;
    }
  inv.assign((size_t)N * N, 0.0);
  for (int i = 0; i < N; ++i) inv[(size_t)i * N + i] = 1.0;
  for (int c = 0; c < N; ++c) {          // Gauss-Jordan with partial pivoting
    int piv = c;
    for (int r = c + 1; r < N; ++r)
      if (fabs(A[(size_t)r * N + c]) > fabs(A[(size_t)piv * N + c])) piv = r;
    if (fabs(A[(size_t)piv * N + c]) < 1e-300) return false;
    if (piv != c)
      for (int k = 0; k < N; ++k) {
        std::swap(A[(size_t)c * N + k], A[(size_t)piv * N + k]);
        std::swap(inv[(size_t)c * N + k], inv[(size_t)piv * N + k]);
      }
    double s = 1.0 / A[(size_t)c * N + c];
    for (int k = 0; k < N; ++k) {
      A[(size_t)c * N + k] *= s;
      inv[(size_t)c * N + k] *= s;
    }
    for (int r = 0; r < N; ++r) {
      if (r == c) continue;
      double f = A[(size_t)r * N + c];
      if (f == 0.0) continue;
      for (int k = 0; k < N; ++k) {
        A[(size_t)r * N + k] -= f * A[(size_t)c * N + k];
        inv[(size_t)r * N + k] -= f * inv[(size_t)c * N + k];
      }
    }
  }
  return true;
}

int converge_first_block_level(const Layout& L) {
  // the coarsest level always; finer ones while they are small enough and fit
  int lc = L.nlev;
  for (int l = L.nlev - 1; l >= 1; --l) {
    if ((long)L.ln[l] * L.lm[l] > CV_BLOCK_MAX_CELLS) break;
    if (L.lm[l] > CV_BLOCK_THREADS) break;      // one row per pass of the block
    if (converge_block_smem(L, l) > kBlockSmemMax) break;
    lc = l;
  }
  return lc;
}

int converge_prepare(const AjStepParams& p, const Layout& L, void* ws, cudaStream_t st) {
  std::vector<double> inv;
  if (!coarse_inverse(p, L, inv)) return AJ_ERR_PARAM;
  std::vector<float> cy, ly;
  if (L.ld > 0) {
    // orthonormal DCT-II basis of the level-ld Neumann-Neumann y operator and
    // its eigenvalues times 1/hy^2
    const int m = L.lm[L.ld];
    const double hy = p.dy * (double)(1 << L.ld), ay = 1.0 / (hy * hy);
    const double pi = 3.14159265358979323846;
    cy.resize((size_t)m * m);
    ly.resize(m);
    for (int k = 0; k < m; ++k) {
      const double sk = k == 0 ? sqrt(1.0 / m) : sqrt(2.0 / m);
      for (int j = 0; j < m; ++j) cy[(size_t)k * m + j] = (float)(sk * cos(pi * k * (2 * j + 1) / (2.0 * m)));
      const double sn = sin(pi * k / (2.0 * m));
      ly[k] = (float)(-4.0 * ay * sn * sn);
    }
    if (cudaMemcpyAsync(at<float>(ws, L.dcy), cy.data(), cy.size() * 4, cudaMemcpyHostToDevice,
                        st) != cudaSuccess ||
        cudaMemcpyAsync(at<float>(ws, L.dly), ly.data(), ly.size() * 4, cudaMemcpyHostToDevice,
                        st) != cudaSuccess)
      return AJ_ERR_CUDA;
  }
  if (cudaFuncSetAttribute(k_cv_block, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)kBlockSmemMax + 1024) != cudaSuccess)
    return AJ_ERR_CUDA;
  if (cudaMemcpyAsync(at<double>(ws, L.cinv), inv.data(), inv.size() * sizeof(double),
                      cudaMemcpyHostToDevice, st) != cudaSuccess)
    return AJ_ERR_CUDA;
  return cudaStreamSynchronize(st) == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

// One launch of a converging-mode kernel on the workspace's current contents
// (instrumentation: lets a caller time the kernel on its own).  which:
// 0 = level-0 smoothing + residual + restriction, 1 = level-0 prolongation +
// smoothing + pressure update + residual (the solver state is left untouched),
// 2 = the coarse solve (the separable direct solve, or the one-block kernel).
int profile_pressure_kernel(const AjStepParams& p, const Layout& L, void* ws, int which,
                            cudaStream_t st) {
  if (p.mg_mode != AJ_MG_CONVERGE) return AJ_ERR_PARAM;
  DevScalars* sc = at<DevScalars>(ws, 0);
  const int* never = reinterpret_cast<const int*>(&sc->pad_[0]);   // always 0
  CvLvl c = cv_level(p, L, 0);
  const int v = tile_variant(p.nx, p.ny);
  if (which == 0) {
    level0_down_v(v, c, L, ws, never, st);
  } else if (which == 1) {
    CvCheck ck{p.mg_rtol, p.max_cycles, 0, 0};
    // profile mode reads the current state buffer and writes only the other one
    level0_up_v(v, p, c, L, ws, sc, ck, 1, st);
  } else if (which == 2) {
    if (L.ld > 0) {
      direct_launch(direct_args(p, L, ws, never), st);
    } else {
      k_cv_block<<<1, CV_BLOCK_THREADS, converge_block_smem(L, L.lc), st>>>(
          block_args(p, L, ws, never));
    }
  } else {
    return AJ_ERR_PARAM;
  }
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

// ---------------------------------------------------------------- autotuner
// The level-0 tile shape per grid shape.  converge_autotune times every
// candidate (level-0 pre-smoothing + post-smoothing kernels, profile mode, on
// a prepared workspace) and keeps the fastest (the default unless another is
// 5 % faster); the choice is cached per
// (nx, ny, SM count) for the life of the process and is part of every graph
// key, so graphs captured before and after a tuning never mix.
namespace {
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int>, int> g_tune;
int sm_count() {
  static int n = -1;
  if (n < 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) n = 0;
  }
  return n;
}
}  // namespace

int tile_variant(int nx, int ny) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tune.find({nx, ny, sm_count()});
  return it == g_tune.end() ? 0 : it->second;
}

int converge_autotune(const AjStepParams& p, const Layout& L, void* ws, int reps, float* times_ms,
                      int* chosen, cudaStream_t st) {
  if (p.mg_mode != AJ_MG_CONVERGE) return AJ_ERR_PARAM;
  DevScalars* sc = at<DevScalars>(ws, 0);
  const int* never = reinterpret_cast<const int*>(&sc->pad_[0]);   // always 0
  const CvLvl c = cv_level(p, L, 0);
  const CvCheck ck{p.mg_rtol, p.max_cycles, 0, 0};
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    return AJ_ERR_CUDA;
  int best = 0;
  float best_ms = 1e30f;
  for (int v = 0; v < CV_TILE_VARIANTS; ++v) {
    for (int w = 0; w < 2; ++w) {   // warm-up
      level0_down_v(v, c, L, ws, never, st);
      level0_up_v(v, p, c, L, ws, sc, ck, 1, st);
    }
    cudaEventRecord(e0, st);
    for (int r = 0; r < reps; ++r) {
      level0_down_v(v, c, L, ws, never, st);
      level0_up_v(v, p, c, L, ws, sc, ck, 1, st);
    }
    cudaEventRecord(e1, st);
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return AJ_ERR_CUDA;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    ms /= (float)(reps > 0 ? reps : 1);
    if (times_ms) times_ms[v] = ms;
    // another shape must beat the default by 5 % to be taken (the candidates
    // are often within run-to-run noise of each other)
    if (v == 0 || ms < 0.95f * best_ms) {
      best_ms = ms;
      best = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[{p.nx, p.ny, sm_count()}] = best;
  }
  if (chosen) *chosen = best;
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

}  // namespace aj

