// Reverse mode (vector-Jacobian product) of the collocated step_pure: what
// jax.grad computes through the reference's rollouts (solver/solver.py:34-114;
// inverse_design_WIP/optimizer_autodiff.py:113-205 differentiates the same
// scan).  From cotangents of the step's outputs (u, v, p) it produces the
// cotangents of its inputs (u, v) and of the parameters a design loss
// differentiates: the SDF (through the Brinkman chi), nu and U_inf.
//
// The reverse pass follows the forward in reverse order:
//   correction + interface projection + boundary rows + hard masks
//     (solver/pure_functions/step.py:259-397)       -> k_adj_correct, k_adj_grad
//   parity multigrid (pressure_solvers/multigrid_solver.py:173-241)
//                                                    -> k_adj_pair/prolong/coarsest
//   rhs = div*mask/dt (step.py:182-199)              -> k_adj_div
//   RK3/RK2 upwind predictor with implicit Brinkman (rk3_simple_new.py:284-358)
//                                                    -> k_adj_rk_out, k_adj_rk_stage
// JAX's rules: where(c, x, y) sends the cotangent to the selected branch (the
// condition has none), .at[].set drops the overwritten entries' cotangent,
// lax.cond in the V-cycle scan differentiates only the cycles that ran.
//
// Structure: the Jacobi sweep (p <- (N p - b)/d) and the edge-ghost Laplacian
// are symmetric, so each reversed sweep is h = pbar/d, bbar -= h, pbar = N h;
// restriction and prolongation swap into each other's transposes; each
// level's two reversed pre- or post-sweeps run as one tiled kernel.  The
// boundary rows are gathers (each output cell copies one source cell), so
// their transposes are gathers at the source.  The two boundary passes of the
// predictor (rk3_simple_new.py:262-275, then step.py:182-191) compose to the
// first, so one transpose covers both.  Forward stage states are recomputed
// by the forward predictor kernels (stage buffers of the step workspace).
#include "aj_internal.cuh"

#include <cooperative_groups.h>
#include <mutex>

namespace aj {

// ------------------------------------------------------------------ layout
struct AdjLayout {
  size_t gus = 0, gvs = 0;           // cotangent of the predictor output
  size_t gdpx = 0, gdpy = 0;         // cotangent of the projected pressure gradient
  size_t wnu = 0, wnv = 0;           // forward predictor output (recomputed)
  size_t kAu = 0, kAv = 0, kBu = 0, kBv = 0, kEu = 0, kEv = 0;   // stage-slope cotangents
  size_t w1u = 0, w1v = 0, dbar = 0; // cotangent of u, v through the stages; of den
  size_t pscr = 0;                   // forward pressure (only to count V-cycles)
  size_t GX[AJ_MAX_LEVELS + 1] = {0}, GT[AJ_MAX_LEVELS + 1] = {0}, GB[AJ_MAX_LEVELS + 1] = {0};
  size_t part = 0;                   // per-block FP64 partial sums of d/d nu
  int nblk = 0;                      // blocks of one cell kernel
  size_t total = 0;
};

constexpr int kAdjBX = 32, kAdjBY = 8;

static bool make_adj_layout(const AjStepParams& p, const Layout& L, AdjLayout& A) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off += (bytes + 255) & ~(size_t)255;
    return o;
  };
  const size_t N = (size_t)p.nx * p.ny * 4;
  A.gus = take(N);
  A.gvs = take(N);
  A.gdpx = take(N);
  A.gdpy = take(N);
  A.wnu = take(N);
  A.wnv = take(N);
  A.kAu = take(N);
  A.kAv = take(N);
  A.kBu = take(N);
  A.kBv = take(N);
  if (p.fast_mode) {
    A.kEu = take(N);
    A.kEv = take(N);
  }
  A.w1u = take(N);
  A.w1v = take(N);
  A.dbar = take(N);
  if (p.v_cycles > 1) A.pscr = take(N);
  for (int l = 0; l <= L.nlev; ++l) {
    const size_t n = (size_t)L.ln[l] * L.lm[l] * 4;
    A.GX[l] = take(n);
    A.GT[l] = take(n);
    A.GB[l] = take(n);
  }
  A.nblk = cdiv(p.ny, kAdjBX) * cdiv(p.nx, kAdjBY);
  A.part = take((size_t)A.nblk * 3 * 8);
  A.total = off;
  return true;
}

// ------------------------------------------------------------------ helpers
__device__ __forceinline__ bool live_at(const float* __restrict__ mask, long k) {
  return ldg(mask + k) > 0.5f;
}
__device__ __forceinline__ bool interior(int i, int j, int nx, int ny) {
  return i >= 1 && i <= nx - 2 && j >= 1 && j <= ny - 2;
}

// one-sided mask gradients of the interface projection (operators.py:17-56)
__device__ __forceinline__ float gx_nonper(const float* __restrict__ f, int a, int b, int nx,
                                           int ny, float idx, float h2x) {
  if (a == 0) return (ldg(f + (long)ny + b) - ldg(f + b)) * idx;
  if (a == nx - 1) return (ldg(f + (long)(nx - 1) * ny + b) - ldg(f + (long)(nx - 2) * ny + b)) * idx;
  return (ldg(f + (long)(a + 1) * ny + b) - ldg(f + (long)(a - 1) * ny + b)) * h2x;
}
__device__ __forceinline__ float gy_nonper(const float* __restrict__ f, int a, int b, int ny,
                                           float idy, float h2y) {
  const float* r = f + (long)a * ny;
  if (b == 0) return (ldg(r + 1) - ldg(r)) * idy;
  if (b == ny - 1) return (ldg(r + ny - 1) - ldg(r + ny - 2)) * idy;
  return (ldg(r + b + 1) - ldg(r + b - 1)) * h2y;
}

// transpose of the non-periodic gradient along one axis at index i of n
// (stride between neighbours s): central rows 1..n-2, one-sided rows 0, n-1
__device__ __forceinline__ float grad_T(const float* __restrict__ g, long s, int i, int n,
                                        float ih, float h2) {
  float r = 0.f;
  if (i - 1 >= 1 && i - 1 <= n - 2) r += h2 * ldg(g + (long)(i - 1) * s);
  if (i + 1 >= 1 && i + 1 <= n - 2) r -= h2 * ldg(g + (long)(i + 1) * s);
  if (i == 1) r += ih * ldg(g);
  if (i == 0) r -= ih * ldg(g);
  if (i == n - 1) r += ih * ldg(g + (long)(n - 1) * s);
  if (i == n - 2) r -= ih * ldg(g + (long)(n - 1) * s);
  return r;
}

// Transpose of the von Karman slip-wall boundary gather at source (a, b):
// output u(i, j) copies u(ci(i), cj(j)) (i > 0; ci(nx-1) = nx-2, cj(0) = 1,
// cj(ny-1) = ny-2) and v(i, j) copies v(ci(i), j) (0 < j < ny-1); the inlet
// row and the wall columns of v are constants.  Each output may be weighted
// by its hard mask (the correction's last mask, step.py:396-397).
// With walls = false the wall columns of u are constants too (no-slip: the
// GUI step's correction, step_handlers.py:143-161, and the predictor with
// slip_walls off).
template <bool MASKED>
__device__ __forceinline__ void bc_gather_T(const float* __restrict__ gu_o,
                                            const float* __restrict__ gv_o,
                                            const float* __restrict__ mask, int a, int b, int nx,
                                            int ny, bool walls, float& gu, float& gv) {
  gu = 0.f;
  gv = 0.f;
  if (!interior(a, b, nx, ny)) return;
  const int nrow = a == nx - 2 ? 2 : 1;
  for (int r = 0; r < nrow; ++r) {
    const long base = (long)(r == 0 ? a : nx - 1) * ny;
    auto take = [&](const float* g, long q) {
      return MASKED ? (live_at(mask, q) ? ldg(g + q) : 0.f) : ldg(g + q);
    };
    gu += take(gu_o, base + b);
    if (walls && b == 1) gu += take(gu_o, base);
    if (walls && b == ny - 2) gu += take(gu_o, base + ny - 1);
    gv += take(gv_o, base + b);
  }
}

// ------------------------------------------------------------------ correction
struct AdjCorr {
  const float *gu_o, *gv_o, *gp_o, *mask;
  float *gus, *gvs, *gdpx, *gdpy, *pbar;
  const DevScalars* sc;
  int nx, ny, gui;
  float idx, idy, h2x, h2y, thresh;
};

// cotangents of u*, v* and of the (projected) gradient at source (a, b):
// step_pure, step.py:341-397 reversed (slip-wall copies, a hard mask before
// and after the boundary rows, the interface projection); the GUI step,
// step_handlers.py:128-183 reversed (no-slip walls, the inlet corners
// excluded, one hard mask at the end, no projection)
__global__ void __launch_bounds__(256) k_adj_correct(AdjCorr c) {
  pdl_wait();
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  const int nx = c.nx, ny = c.ny;
  if (i >= nx || j >= ny) return;
  const long k = (long)i * ny + j;
  float gu, gv;
  bc_gather_T<true>(c.gu_o, c.gv_o, c.mask, i, j, nx, ny, !c.gui, gu, gv);
  if (!c.gui && !live_at(c.mask, k)) gu = gv = 0.f;            // step.py:348-349
  c.gus[k] = gu;
  c.gvs[k] = gv;
  const float dt = c.sc->dt_corr;
  float ax = -dt * gu, ay = -dt * gv;                           // (row 0: gu = 0, :341)
  if (c.gui) {
    c.gdpx[k] = ax;
    c.gdpy[k] = ay;
    return;
  }
  const float dmx = gx_nonper(c.mask, i, j, nx, ny, c.idx, c.h2x);
  const float dmy = gy_nonper(c.mask, i, j, ny, c.idy, c.h2y);
  const float gm = sqrtf(dmx * dmx + dmy * dmy);
  if (gm > c.thresh) {                                          // step.py:313-335 (symmetric)
    const float nxv = dmx / (gm + 1e-8f), nyv = dmy / (gm + 1e-8f);
    const float dn = -(ax * nxv + ay * nyv);
    ax = ax + dn * nxv;
    ay = ay + dn * nyv;
  }
  c.gdpx[k] = ax;
  c.gdpy[k] = ay;
}

// cotangent of p: the output's own cotangent plus the gradient's transpose
__global__ void __launch_bounds__(256) k_adj_grad(AdjCorr c) {
  pdl_wait();
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  const int nx = c.nx, ny = c.ny;
  if (i >= nx || j >= ny) return;
  const long k = (long)i * ny + j;
  float r = c.gp_o ? ldg(c.gp_o + k) : 0.f;
  r += grad_T(c.gdpx + j, ny, i, nx, c.idx, c.h2x);
  r += grad_T(c.gdpy + (long)i * ny, 1, j, ny, c.idy, c.h2y);
  c.pbar[k] = r;
}

// ------------------------------------------------------------------ multigrid
// reversed Jacobi sweep: h = (gin with the outlet row zeroed when the forward
// sweep reset it)/d; gb -= h (or = -h); gout = N h
__global__ void __launch_bounds__(256) k_adj_jac(const float* __restrict__ gin,
                                                 float* __restrict__ gout, float* __restrict__ gb,
                                                 int n, int m, float ax, float ay, float d,
                                                 int zero_last, int assign, const int* ncyc,
                                                 int cyc) {
  pdl_wait();
  if (ncyc && cyc >= *ncyc) return;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= n || j >= m) return;
  auto h = [&](int ii, int jj) -> float {
    return (zero_last && ii == n - 1) ? 0.f : ldg(gin + (long)ii * m + jj) / d;
  };
  const long k = (long)i * m + j;
  const float hc = h(i, j);
  gb[k] = assign ? -hc : gb[k] - hc;
  if (gout) {
    const int ip = i + 1 < n ? i + 1 : n - 1, im = i > 0 ? i - 1 : 0;
    const int jp = j + 1 < m ? j + 1 : m - 1, jm = j > 0 ? j - 1 : 0;
    gout[k] = ax * (h(ip, j) + h(im, j)) + ay * (h(i, jp) + h(i, jm));
  }
}

// Two consecutive reversed sweeps of one level in one kernel (the forward's
// two pre- or two post-smoothing sweeps, multigrid_solver.py:182-201):
//   [down side only] x = gin - A s, gb += s, s = R^T(coarse b cotangent)
//   h1 = (x with the outlet row zeroed)/d,  gb -= h1,  t = N h1
//   h2 = t/d,                               gb -= h2,  gout = N h2
// on an 8 x 32 output tile: h1 is staged on the tile and a halo of 2, h2 on a
// halo of 1.  gb is read and written only at the block's own cells; gout
// must not alias gin (neighbouring blocks read gin's halo).
constexpr int kPairBX = 32, kPairBY = 8, kPairH = 2;
constexpr int kPairRI = kPairBY + 2 * kPairH, kPairRJ = kPairBX + 2 * kPairH;
__global__ void __launch_bounds__(kPairBX * kPairBY) k_adj_pair(
    const float* __restrict__ gin, float* __restrict__ gout, float* __restrict__ gb,
    const float* __restrict__ gbc, int n, int m, float ax, float ay, float d, int assign,
    const int* ncyc, int cyc) {
  pdl_wait();
  if (ncyc && cyc >= *ncyc) return;
  __shared__ float H1[kPairRI][kPairRJ];
  __shared__ float H2[kPairRI][kPairRJ];
  const int i0 = blockIdx.y * kPairBY - kPairH, j0 = blockIdx.x * kPairBX - kPairH;
  const int tid = threadIdx.y * kPairBX + threadIdx.x;
  const int mc = m / 2;
  auto sres = [&](int gi, int gj) { return 0.25f * ldg(gbc + (long)(gi >> 1) * mc + (gj >> 1)); };
  for (int q = tid; q < kPairRI * kPairRJ; q += kPairBX * kPairBY) {
    const int r = q / kPairRJ, c = q - r * kPairRJ;
    const int gi = i0 + r, gj = j0 + c;
    float h = 0.f;
    if (gi >= 0 && gi < n && gj >= 0 && gj < m) {
      float x = ldg(gin + (long)gi * m + gj);
      if (gbc) {
        const int ip = gi + 1 < n ? gi + 1 : n - 1, im = gi > 0 ? gi - 1 : 0;
        const int jp = gj + 1 < m ? gj + 1 : m - 1, jm = gj > 0 ? gj - 1 : 0;
        const float sc = sres(gi, gj);
        x -= ax * (sres(ip, gj) + sres(im, gj) - 2.f * sc) + ay * (sres(gi, jp) + sres(gi, jm) - 2.f * sc);
      }
      h = gi == n - 1 ? 0.f : x / d;
    }
    H1[r][c] = h;
  }
  __syncthreads();
  // neighbours with edge ghosts, in tile coordinates (a domain edge maps to the cell itself)
  auto nsum = [&](float (*S)[kPairRJ], int r, int c, int gi, int gj) {
    const int rp = gi + 1 < n ? r + 1 : r, rm = gi > 0 ? r - 1 : r;
    const int cp = gj + 1 < m ? c + 1 : c, cm = gj > 0 ? c - 1 : c;
    return ax * (S[rp][c] + S[rm][c]) + ay * (S[r][cp] + S[r][cm]);
  };
  for (int q = tid; q < (kPairRI - 2) * (kPairRJ - 2); q += kPairBX * kPairBY) {
    const int r = q / (kPairRJ - 2) + 1, c = q % (kPairRJ - 2) + 1;
    const int gi = i0 + r, gj = j0 + c;
    float h = 0.f;
    if (gi >= 0 && gi < n && gj >= 0 && gj < m) h = nsum(H1, r, c, gi, gj) / d;
    H2[r][c] = h;
  }
  __syncthreads();
  const int r = threadIdx.y + kPairH, c = threadIdx.x + kPairH;
  const int gi = i0 + r, gj = j0 + c;
  if (gi >= n || gj >= m) return;
  const long k = (long)gi * m + gj;
  float acc = assign ? 0.f : gb[k];
  if (gbc) acc += sres(gi, gj);
  gb[k] = acc - H1[r][c] - H2[r][c];
  if (gout) gout[k] = nsum(H2, r, c, gi, gj);
}

// the ten reversed coarsest-grid sweeps (the forward smooths 10 times from a
// zero guess, multigrid_solver.py:186-187) on a cluster of kCoarseCtas
// blocks, each holding a band of rows: h = cotangent/d ping-pongs in shared
// memory (the rows next to the band read from the neighbours' shared memory),
// b's cotangent accumulates in a third array.  One cluster barrier per sweep
// (see k_par_coarsest); used when the three band arrays fit a block.
__global__ void __cluster_dims__(kCoarseCtas, 1, 1) __launch_bounds__(kCoarseThreads)
    k_adj_coarsest(const float* __restrict__ gin, float* __restrict__ gb, int n, int m, float ax,
                   float ay, float d, const int* ncyc, int cyc) {
  pdl_wait();
  if (ncyc && cyc >= *ncyc) return;
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const int R = coarse_band_rows(n);
  const int r0 = rank * R, nr = max(0, min(n, r0 + R) - r0);
  extern __shared__ float csm[];
  float* A = csm;            // h = cotangent/d of the band (ping-pong with B)
  float* B = csm + R * m;
  float* G = csm + 2 * R * m;
  for (int q = threadIdx.x; q < nr * m; q += blockDim.x) {
    const float hc = gin[(long)r0 * m + q] / d;
    A[q] = hc;
    G[q] = -hc;
  }
  cl.sync();                 // the neighbours' first values are in place
  for (int s = 9; s >= 1; --s) {
    for (int q = threadIdx.x; q < nr * m; q += blockDim.x) {
      const int li = q / m, j = q - li * m, i = r0 + li;
      const int ip = i + 1 < n ? i + 1 : n - 1, im = i > 0 ? i - 1 : 0;
      const int jp = j + 1 < m ? j + 1 : m - 1, jm = j > 0 ? j - 1 : 0;
      auto hv = [&](int ii, int jj) -> float {
        const int owner = ii / R;
        const float* base = owner == rank ? A : cl.map_shared_rank(A, owner);
        return base[(ii - owner * R) * m + jj];
      };
      const float hn = (ax * (hv(ip, j) + hv(im, j)) + ay * (hv(i, jp) + hv(i, jm))) / d;
      B[q] = hn;
      G[q] = G[q] - hn;
    }
    cl.sync();
    float* t = A;
    A = B;
    B = t;
  }
  for (int q = threadIdx.x; q < nr * m; q += blockDim.x) gb[(long)r0 * m + q] = G[q];
}

// transpose of the reference prolongation (multigrid_solver.py:134-156) onto
// the coarse cell (I, J): even fine cells inject, odd interior ones average
__global__ void __launch_bounds__(256) k_adj_prolong(const float* __restrict__ gf,
                                                     float* __restrict__ gc, int nc, int mc,
                                                     const int* ncyc, int cyc) {
  pdl_wait();
  if (ncyc && cyc >= *ncyc) return;
  const int J = blockIdx.x * blockDim.x + threadIdx.x;
  const int I = blockIdx.y * blockDim.y + threadIdx.y;
  if (I >= nc || J >= mc) return;
  const int mf = 2 * mc;
  auto F = [&](int a, int b) { return ldg(gf + (long)a * mf + b); };
  const bool iu = I <= nc - 2, id = I >= 1, ju = J <= mc - 2, jd = J >= 1;
  float r = F(2 * I, 2 * J);
  float s = 0.f;
  if (iu) s += F(2 * I + 1, 2 * J);
  if (id) s += F(2 * I - 1, 2 * J);
  if (ju) s += F(2 * I, 2 * J + 1);
  if (jd) s += F(2 * I, 2 * J - 1);
  float q = 0.f;
  if (iu && ju) q += F(2 * I + 1, 2 * J + 1);
  if (id && ju) q += F(2 * I - 1, 2 * J + 1);
  if (iu && jd) q += F(2 * I + 1, 2 * J - 1);
  if (id && jd) q += F(2 * I - 1, 2 * J - 1);
  gc[(long)I * mc + J] = r + 0.5f * s + 0.25f * q;
}

// ------------------------------------------------------------------ rhs
// rhs = (div * mask)/dt (step.py:199; the GUI step: div/dt,
// step_handlers.py:98) with b[-1] = 0 (multigrid_solver.py:75-77);
// div = central differences on the interior (operators.py:81-96): adds the
// transpose to the predictor-output cotangent
__global__ void __launch_bounds__(256) k_adj_div(const float* __restrict__ gb0,
                                                 const float* __restrict__ mask,
                                                 float* __restrict__ gus, float* __restrict__ gvs,
                                                 const DevScalars* sc, int nx, int ny, float h2x,
                                                 float h2y, int rhs_mask) {
  pdl_wait();
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  const float dt = sc->dt;
  auto dv = [&](int a, int b) -> float {
    if (!interior(a, b, nx, ny)) return 0.f;                  // (a <= nx-2: never the zeroed row)
    const long q = (long)a * ny + b;
    return rhs_mask ? (ldg(gb0 + q) * ldg(mask + q)) / dt : ldg(gb0 + q) / dt;   // GUI: div/dt
  };
  const long k = (long)i * ny + j;
  gus[k] += h2x * (dv(i - 1, j) - dv(i + 1, j));
  gvs[k] += h2y * (dv(i, j - 1) - dv(i, j + 1));
}

// ------------------------------------------------------------------ predictor
struct AdjRk {
  const float *gus, *gvs;          // k_adj_rk_out: cotangent of the predictor output
  const float *kin_u, *kin_v;      // stages: cotangent of this stage's slope
  const float *wu, *wv;            // stages: the stage state; k_adj_rk_out: predictor output
  const float *chi;
  float *w1u, *w1v, *dbar;
  float *kout_u, *kout_v;          // cotangent of the previous stage's slope
  float *kext_u, *kext_v;          // RK2: 0.5 dt x_n (part of k1's cotangent)
  float *gu, *gv;                  // last stage: cotangents of the step's u, v
  float *gsdf;                     // accumulated (nullable)
  double* part;                    // per-block d/d nu
  const float* mask;
  const DevScalars* sc;
  int nx, ny, last, slip;
  float idx, idy, idx2, idy2, nu, inv_eta, cn, sdf_fac;
  float nuh;                       // nu * nu_hyper_ratio * dx * dy (hyperviscosity)
  float nuh_fac;                   // nu_hyper_ratio * dx * dy
};

// cotangent of the final combination x_n / den, through the predictor's hard
// mask and boundary rows (rk3_simple_new.py:332-337, 262-275, slip or
// no-slip walls; step_pure's second pass, step.py:182-191, composes to the
// first)
__global__ void __launch_bounds__(256) k_adj_rk_out(AdjRk a) {
  pdl_wait();
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  const int nx = a.nx, ny = a.ny;
  if (i >= nx || j >= ny) return;
  const long k = (long)i * ny + j;
  float gu, gv;
  bc_gather_T<false>(a.gus, a.gvs, nullptr, i, j, nx, ny, a.slip, gu, gv);
  if (!live_at(a.mask, k)) gu = gv = 0.f;
  const float dt = a.sc->dt;
  const float rden = 1.f / (1.f + dt * ldg(a.chi + k) * a.inv_eta);
  const float xu = gu * rden, xv = gv * rden;
  // where x != 0 the output cell is interior and live: it holds x_n/den itself
  a.dbar[k] = -(xu * ldg(a.wu + k) + xv * ldg(a.wv + k));
  a.w1u[k] = xu;                                                // 1/3 + 2/3 (RK2: 1)
  a.w1v[k] = xv;
  a.kout_u[k] = a.cn * dt * xu;
  a.kout_v[k] = a.cn * dt * xv;
  if (a.kext_u) {
    a.kext_u[k] = 0.5f * dt * xu;
    a.kext_v[k] = 0.5f * dt * xv;
  }
}

// One reversed stage: the transpose of the explicit right-hand side
// (rk3_simple_new.py:284-313; first-order upwind, edge ghosts) at the stage
// state w, applied to the slope cotangent kbar, then the stage's
// combination.  For target cell c the upwind difference of cell q reads
// +f(q) - f(W(q)) when its velocity is positive, else -f(q) + f(E(q)): the
// gather visits q = c and its four neighbours.
template <bool HYPER>
__global__ void __launch_bounds__(256) k_adj_rk_stage(AdjRk a) {
  pdl_wait();
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  const int nx = a.nx, ny = a.ny;
  const bool valid = i < nx && j < ny;
  df nub{0.f, 0.f};
  if (valid) {
    const long k = (long)i * ny + j;
    const int im = i > 0 ? i - 1 : 0, ip = i < nx - 1 ? i + 1 : nx - 1;
    const int jm = j > 0 ? j - 1 : 0, jp = j < ny - 1 ? j + 1 : ny - 1;
    const long kxm = (long)im * ny + j, kxp = (long)ip * ny + j;
    const long kym = (long)i * ny + jm, kyp = (long)i * ny + jp;
    const float U = ldg(a.wu + k), V = ldg(a.wv + k);
    const float uxm = ldg(a.wu + kxm), uxp = ldg(a.wu + kxp), uym = ldg(a.wu + kym), uyp = ldg(a.wu + kyp);
    const float vxm = ldg(a.wv + kxm), vxp = ldg(a.wv + kxp), vym = ldg(a.wv + kym), vyp = ldg(a.wv + kyp);
    const float ku = ldg(a.kin_u + k), kv = ldg(a.kin_v + k);
    const float kuxm = ldg(a.kin_u + kxm), kuxp = ldg(a.kin_u + kxp);
    const float kuym = ldg(a.kin_u + kym), kuyp = ldg(a.kin_u + kyp);
    const float kvxm = ldg(a.kin_v + kxm), kvxp = ldg(a.kin_v + kxp);
    const float kvym = ldg(a.kin_v + kym), kvyp = ldg(a.kin_v + kyp);
    const float A = -ku, B = -kv;                  // cotangents of the advection terms
    const bool px = U > 0.f, py = V > 0.f;
    // velocity roles: d(adv)/d(velocity) = the upwind difference itself
    const float fxu = px ? (U - uxm) * a.idx : (uxp - U) * a.idx;
    const float fxv = px ? (V - vxm) * a.idx : (vxp - V) * a.idx;
    const float fyu = py ? (U - uym) * a.idy : (uyp - U) * a.idy;
    const float fyv = py ? (V - vym) * a.idy : (vyp - V) * a.idy;
    float gu = A * fxu + B * fxv;
    float gv = A * fyu + B * fyv;
    // diffusion (the edge Laplacian is symmetric)
    gu += a.nu * ((kuxp + kuxm - 2.f * ku) * a.idx2 + (kuyp + kuym - 2.f * ku) * a.idy2);
    gv += a.nu * ((kvxp + kvxm - 2.f * kv) * a.idx2 + (kvyp + kvym - 2.f * kv) * a.idy2);
    // field roles, centre cell (its own ghost at the edges)
    {
      const float al = A * U * a.idx, be = B * U * a.idx;
      float cu = px ? al : -al, cv = px ? be : -be;
      if (i == 0 && px) { cu -= al; cv -= be; }
      if (i == nx - 1 && !px) { cu += al; cv += be; }
      const float ay_ = A * V * a.idy, by_ = B * V * a.idy;
      float du = py ? ay_ : -ay_, dv = py ? by_ : -by_;
      if (j == 0 && py) { du -= ay_; dv -= by_; }
      if (j == ny - 1 && !py) { du += ay_; dv += by_; }
      gu += cu + du;
      gv += cv + dv;
    }
    // field roles, neighbours: q = c + x reads f(c) as its W when U(q) > 0,
    // q = c - x reads f(c) as its E when U(q) <= 0 (likewise in y with V)
    if (i + 1 <= nx - 1 && uxp > 0.f) { gu += kuxp * uxp * a.idx; gv += kvxp * uxp * a.idx; }
    if (i - 1 >= 0 && !(uxm > 0.f)) { gu -= kuxm * uxm * a.idx; gv -= kvxm * uxm * a.idx; }
    if (j + 1 <= ny - 1 && vyp > 0.f) { gu += kuyp * vyp * a.idy; gv += kvyp * vyp * a.idy; }
    if (j - 1 >= 0 && !(vym > 0.f)) { gu -= kuym * vym * a.idy; gv -= kvym * vym * a.idy; }
    // d/d nu: kbar . lap(w)
    const float lu = (uxp + uxm - 2.f * U) * a.idx2 + (uyp + uym - 2.f * U) * a.idy2;
    const float lv = (vxp + vxm - 2.f * V) * a.idx2 + (vyp + vym - 2.f * V) * a.idy2;
    // exact products, summed in double-FP32 (the sum cancels heavily)
    nub = df_add(two_prod(ku, lu), two_prod(kv, lv));
    if (HYPER) {
      // - nu nuh_fac lap(lap(w)) (rk3_simple_new.py:307-312, the edge
      // Laplacian of the edge Laplacian, as the forward evaluates it): its
      // own transpose; lap at the clamped neighbours of (i, j)
      auto lap = [&](const float* __restrict__ f, int ii, int jj) {
        const int p1 = ii < nx - 1 ? ii + 1 : nx - 1, m1 = ii > 0 ? ii - 1 : 0;
        const int q1 = jj < ny - 1 ? jj + 1 : ny - 1, n1 = jj > 0 ? jj - 1 : 0;
        const float c0 = ldg(f + (long)ii * ny + jj);
        return (ldg(f + (long)p1 * ny + jj) + ldg(f + (long)m1 * ny + jj) - 2.f * c0) * a.idx2 +
               (ldg(f + (long)ii * ny + q1) + ldg(f + (long)ii * ny + n1) - 2.f * c0) * a.idy2;
      };
      auto bih = [&](const float* __restrict__ f) {
        const float l0 = lap(f, i, j);
        return (lap(f, ip, j) + lap(f, im, j) - 2.f * l0) * a.idx2 +
               (lap(f, i, jp) + lap(f, i, jm) - 2.f * l0) * a.idy2;
      };
      gu -= a.nuh * bih(a.kin_u);
      gv -= a.nuh * bih(a.kin_v);
      nub = df_add(nub, df_add(two_prod(ku, -a.nuh_fac * bih(a.wu)),
                               two_prod(kv, -a.nuh_fac * bih(a.wv))));
    }
    const float dt = a.sc->dt;
    if (!a.last) {
      const float rden = 1.f / (1.f + dt * ldg(a.chi + k) * a.inv_eta);
      const float xu = gu * rden, xv = gv * rden;
      a.dbar[k] -= xu * U + xv * V;
      a.w1u[k] += xu;
      a.w1v[k] += xv;
      float nku = a.cn * dt * xu, nkv = a.cn * dt * xv;
      if (a.kext_u) {
        nku += a.kext_u[k];
        nkv += a.kext_v[k];
      }
      a.kout_u[k] = nku;
      a.kout_v[k] = nkv;
    } else {
      a.gu[k] = a.w1u[k] + gu;
      a.gv[k] = a.w1v[k] + gv;
      if (a.gsdf) {
        // den = 1 + dt chi/eta, chi = sigmoid(-sdf/(0.1 dx)) (rk3_simple_new.py:194-198)
        const float c = ldg(a.chi + k);
        a.gsdf[k] += a.dbar[k] * dt * a.inv_eta * c * (1.f - c) * a.sdf_fac;
      }
    }
  }
  const double t = block_sum_df(nub);
  if (threadIdx.x == 0 && threadIdx.y == 0) a.part[blockIdx.y * gridDim.x + blockIdx.x] = t;
}

// d/d nu from the stage partials and d/d U_inf from the inlet rows (the
// correction's final row 0 where live, and the predictor output's row 0),
// summed in a fixed order and added to gscal[0], gscal[1]
// (four independent accumulators per thread keep four loads in flight: one
// accumulator left the block waiting on one partial at a time, 28 us)
// The inlet rows: the correction's final row 0 where live (the GUI step
// leaves the two corners on the walls: corr_walls = 0) and the predictor
// output's row 0 (with no-slip walls its two corners are 0: pred_walls = 0).
__global__ void __launch_bounds__(1024) k_adj_scalars(const double* __restrict__ part, int nparts,
                                                      const float* __restrict__ gu_o,
                                                      const float* __restrict__ gus,
                                                      const float* __restrict__ mask, int ny,
                                                      int corr_walls, int pred_walls,
                                                      double* gscal) {
  pdl_wait();
  const int bd = blockDim.x;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0, u = 0.0;
  int q = threadIdx.x;
  for (; q + 3 * bd < nparts; q += 4 * bd) {
    const double a = part[q], b = part[q + bd], c = part[q + 2 * bd], d = part[q + 3 * bd];
    s0 += a;
    s1 += b;
    s2 += c;
    s3 += d;
  }
  for (; q < nparts; q += bd) s0 += part[q];
  double s = (s0 + s1) + (s2 + s3);
  for (int q = threadIdx.x; q < ny; q += blockDim.x) {
    const bool wall = q == 0 || q == ny - 1;
    if (pred_walls || !wall) u += (double)ldg(gus + q);
    if ((corr_walls || !wall) && live_at(mask, q)) u += (double)ldg(gu_o + q);
  }
  s = block_sum(s);
  u = block_sum(u);
  if (threadIdx.x == 0) {
    gscal[0] += s;
    gscal[1] += u;
  }
}

// ------------------------------------------------------------------ driver
size_t step_vjp_workspace(const AjStepParams& p, const Layout& L) {
  AdjLayout A;
  make_adj_layout(p, L, A);
  return A.total;
}

// The side branch that recomputes the forward predictor beside the reverse
// pass of the correction and the multigrid (created once; its use is
// serialised: a capture into a caller's graph does not hold the library's
// graph-cache lock).
namespace {
std::mutex g_vjp_mu;
struct VjpFork {
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
};
const VjpFork* vjp_fork() {
  static VjpFork f;
  static bool ok = false;
  if (!ok) {
    if (cudaStreamCreateWithFlags(&f.side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&f.fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&f.join, cudaEventDisableTiming) != cudaSuccess)
      return nullptr;
    ok = true;
  }
  return &f;
}
}  // namespace

int launch_step_vjp(const AjStepParams& p, const Layout& L, void* ws, void* aws, const float* u,
                    const float* v, const float* mask, const float* gu_o, const float* gv_o,
                    const float* gp_o, float* gu, float* gv, float* gsdf, double* gscal,
                    cudaStream_t st) {
  AdjLayout A;
  make_adj_layout(p, L, A);
  DevScalars* sc = at<DevScalars>(ws, 0);
  const int nx = p.nx, ny = p.ny;
  const long N = (long)nx * ny;
  auto F = [&](size_t off) { return at<float>(aws, off); };
  const dim3 blk(kAdjBX, kAdjBY), grd(cdiv(ny, kAdjBX), cdiv(nx, kAdjBY));
  int rc;
  std::lock_guard<std::mutex> lk(g_vjp_mu);
  const VjpFork* fk = vjp_fork();
  if (!fk) return AJ_ERR_CUDA;
  // ---- forward: dt, then the predictor's stage states.  With one V-cycle
  // nothing before the predictor's reverse pass reads them: the predictor
  // runs on a side branch joined before k_adj_rk_out.  With more cycles the
  // forward solve counts the cycles the reverse pass replays, in line.
  if ((rc = launch_set_dt(p, ws, st)) != AJ_OK) return rc;
  const bool branch = p.v_cycles == 1;
  if (branch) {
    if (cudaEventRecord(fk->fork, st) != cudaSuccess ||
        cudaStreamWaitEvent(fk->side, fk->fork, 0) != cudaSuccess)
      return AJ_ERR_CUDA;
  }
  rc = launch_predictor(p, L, ws, u, v, mask, nullptr, 0, F(A.wnu), F(A.wnv),
                        branch ? fk->side : st);
  if (rc != AJ_OK) return rc;
  if (branch && cudaEventRecord(fk->join, fk->side) != cudaSuccess) return AJ_ERR_CUDA;
  const int* ncyc = nullptr;
  if (p.v_cycles > 1) {
    // the V-cycles the forward ran (the reference skips cycles once converged)
    if ((rc = launch_rhs(p, L, ws, F(A.wnu), F(A.wnv), mask, at<float>(ws, L.b0), st)) != AJ_OK)
      return rc;
    if ((rc = launch_pressure(p, L, ws, mask, nullptr, F(A.pscr), nullptr, st)) != AJ_OK) return rc;
    ncyc = &sc->mg_cycles;
  }
  // ---- correction, reversed
  AdjCorr c{};
  c.gu_o = gu_o;
  c.gv_o = gv_o;
  c.gp_o = gp_o;
  c.mask = mask;
  c.gus = F(A.gus);
  c.gvs = F(A.gvs);
  c.gdpx = F(A.gdpx);
  c.gdpy = F(A.gdpy);
  c.pbar = F(A.GX[0]);
  c.sc = sc;
  c.nx = nx;
  c.ny = ny;
  c.idx = (float)(1.0 / p.dx);
  c.idy = (float)(1.0 / p.dy);
  c.h2x = (float)(1.0 / (2.0 * p.dx));
  c.h2y = (float)(1.0 / (2.0 * p.dy));
  c.thresh = (float)(0.1 / p.dx);
  c.gui = p.variant == AJ_VARIANT_GUI;
  launch_pdl(true, k_adj_correct, grd, blk, 0, st, c);
  launch_pdl(true, k_adj_grad, grd, blk, 0, st, c);
  // ---- multigrid, reversed (cycles from the last to the first)
  if (cudaMemsetAsync(F(A.GB[0]), 0, (size_t)N * 4, st) != cudaSuccess) return AJ_ERR_CUDA;
  const float ax = (float)(1.0 / (p.dx * p.dx)), ay = (float)(1.0 / (p.dy * p.dy));
  const float den = (float)(2.0 * (1.0 / (p.dx * p.dx) + 1.0 / (p.dy * p.dy)));
  const int nl = L.nlev;
  auto lg = [&](int l) { return dim3(cdiv(L.lm[l], kAdjBX), cdiv(L.ln[l], kAdjBY)); };
  // one reversed sweep at level l (b's cotangent: level l's GB)
  auto jac = [&](int l, const float* gin, float* gout, int zero_last, int assign, const int* nc,
                 int cyc) {
    launch_pdl(true, k_adj_jac, lg(l), blk, 0, st, gin, gout, F(A.GB[l]), L.ln[l], L.lm[l], ax,
               ay, den, zero_last, assign, nc, cyc);
  };
  auto pair = [&](int l, const float* gin, float* gout, const float* gbc, int assign,
                  const int* nc, int cyc) {
    launch_pdl(true, k_adj_pair, dim3(cdiv(L.lm[l], kPairBX), cdiv(L.ln[l], kPairBY)),
               dim3(kPairBX, kPairBY), 0, st, gin, gout, F(A.GB[l]), gbc, L.ln[l], L.lm[l], ax, ay,
               den, assign, nc, cyc);
  };
  for (int cyc = p.v_cycles - 1; cyc >= 0; --cyc) {
    const int* nc = cyc == 0 ? nullptr : ncyc;                 // cycle 0 always ran
    // up-sweep, reversed: the two post-sweeps (GX -> GT), then the
    // prolongation's transpose onto the coarser level's GX
    for (int l = 0; l < nl; ++l) {
      pair(l, F(A.GX[l]), F(A.GT[l]), nullptr, l > 0, nc, cyc);
      launch_pdl(true, k_adj_prolong, lg(l + 1), blk, 0, st, F(A.GT[l]), F(A.GX[l + 1]),
                 L.ln[l + 1], L.lm[l + 1], nc, cyc);
    }
    if (parity_coarsest_fused(L)) {                            // coarsest: 10 sweeps from zero
      const int n = L.ln[nl], m = L.lm[nl];
      cudaFuncSetAttribute(k_adj_coarsest, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)kBlockSmemMax);
      launch_pdl(true, k_adj_coarsest, dim3(kCoarseCtas), dim3(kCoarseThreads),
                 (size_t)coarse_band_rows(n) * m * 12, st, F(A.GX[nl]), F(A.GB[nl]), n, m, ax, ay,
                 den, nc, cyc);
    } else {
      for (int s = 9; s >= 0; --s) {
        const float* gin = (s % 2 == 1) ? F(A.GX[nl]) : F(A.GT[nl]);
        float* gout = s == 0 ? nullptr : ((s % 2 == 1) ? F(A.GT[nl]) : F(A.GX[nl]));
        jac(nl, gin, gout, 0, s == 9, nc, cyc);
      }
    }
    // down-sweep, reversed: the restriction's transpose and the two
    // pre-sweeps on GT; the first pre-sweep's input is zero below level 0
    // and in the first cycle, else its cotangent goes to GX[0]
    for (int l = nl - 1; l >= 0; --l)
      pair(l, F(A.GT[l]), (l == 0 && cyc > 0) ? F(A.GX[0]) : nullptr, F(A.GB[l + 1]), 0, nc, cyc);
  }
  // ---- rhs and divergence, reversed
  launch_pdl(true, k_adj_div, grd, blk, 0, st, F(A.GB[0]), mask, F(A.gus), F(A.gvs), sc, nx, ny,
             (float)(1.0 / (2.0 * p.dx)), (float)(1.0 / (2.0 * p.dy)),
             (int)(p.variant == AJ_VARIANT_PURE));
  // ---- predictor, reversed
  const bool rk2 = p.fast_mode != 0;
  AdjRk r{};
  r.gus = F(A.gus);
  r.gvs = F(A.gvs);
  r.wu = F(A.wnu);
  r.wv = F(A.wnv);
  r.chi = at<float>(ws, L.chi);
  r.w1u = F(A.w1u);
  r.w1v = F(A.w1v);
  r.dbar = F(A.dbar);
  r.kout_u = F(A.kAu);
  r.kout_v = F(A.kAv);
  r.kext_u = rk2 ? F(A.kEu) : nullptr;
  r.kext_v = rk2 ? F(A.kEv) : nullptr;
  r.part = at<double>(aws, A.part);
  r.mask = mask;
  r.sc = sc;
  r.nx = nx;
  r.ny = ny;
  r.idx = (float)(1.0 / p.dx);
  r.idy = (float)(1.0 / p.dy);
  r.idx2 = (float)(1.0 / (p.dx * p.dx));
  r.idy2 = (float)(1.0 / (p.dy * p.dy));
  r.nu = (float)p.nu;
  r.inv_eta = (float)(1.0 / p.brinkman_eta);
  r.sdf_fac = (float)(-1.0 / (0.1 * p.dx));
  r.cn = rk2 ? 0.5f : (float)(2.0 / 3.0);
  r.slip = p.slip_walls;
  r.nuh_fac = (float)(p.nu_hyper_ratio * p.dx * p.dy);
  r.nuh = (float)p.nu * r.nuh_fac;
  const bool hyper = p.nu_hyper_ratio > 0.0;
  if (branch && cudaStreamWaitEvent(st, fk->join, 0) != cudaSuccess) return AJ_ERR_CUDA;
  launch_pdl(true, k_adj_rk_out, grd, blk, 0, st, r);
  // stage states: RK3 w3 = sB, w2 = sA; RK2 w2 = sA; stage 1 is the input
  const float* Wu[3] = {u, at<float>(ws, L.sA_u), at<float>(ws, L.sB_u)};
  const float* Wv[3] = {v, at<float>(ws, L.sA_v), at<float>(ws, L.sB_v)};
  const float cn3[3] = {0.f, 1.f, 0.25f};     // RK3: slope of stage s-1 from x_s
  float* KU[2] = {F(A.kAu), F(A.kBu)};
  float* KV[2] = {F(A.kAv), F(A.kBv)};
  const int nst = rk2 ? 2 : 3;
  int cur = 0;
  for (int s = nst; s >= 1; --s) {
    r.kin_u = KU[cur];
    r.kin_v = KV[cur];
    r.kout_u = KU[1 - cur];
    r.kout_v = KV[1 - cur];
    r.wu = Wu[s - 1];
    r.wv = Wv[s - 1];
    r.last = s == 1;
    r.cn = rk2 ? 1.f : cn3[s - 1];
    r.kext_u = (rk2 && s == 2) ? F(A.kEu) : nullptr;
    r.kext_v = (rk2 && s == 2) ? F(A.kEv) : nullptr;
    r.gu = gu;
    r.gv = gv;
    r.gsdf = (s == 1 && p.has_sdf) ? gsdf : nullptr;
    r.part = at<double>(aws, A.part) + (size_t)(nst - s) * A.nblk;
    if (hyper) launch_pdl(true, k_adj_rk_stage<true>, grd, blk, 0, st, r);
    else launch_pdl(true, k_adj_rk_stage<false>, grd, blk, 0, st, r);
    cur = 1 - cur;
  }
  if (gscal)
    launch_pdl(true, k_adj_scalars, dim3(1), dim3(1024), 0, st, at<double>(aws, A.part),
               nst * A.nblk, gu_o, F(A.gus), mask, ny, (int)(p.variant == AJ_VARIANT_PURE),
               (int)(p.slip_walls != 0), gscal);
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

int step_vjp_kernel_count(const AjStepParams& p, const Layout& L) {
  const int nst = p.fast_mode ? 2 : 3;
  int n = 1 + nst;                                  // dt + forward predictor stages
  const bool fused = parity_coarsest_fused(L);
  if (p.v_cycles > 1)                               // rhs, forward solve
    n += 1 + 1 + p.v_cycles * (2 * L.nlev + (fused ? 1 : 10));
  n += 2;                                           // correction, gradient
  n += p.v_cycles * (3 * L.nlev + (fused ? 1 : 10));  // reversed V-cycles
  n += 1 + 1 + nst + 1;                             // divergence, output, stages, scalars
  return n;
}

}  // namespace aj
