// Pressure Poisson solve.
//
// Parity mode reproduces poisson_multigrid (pressure_solvers/multigrid_solver.py:55-241)
// and poisson_multigrid_mac (pressure_solvers/multigrid_solver_mac.py:59-246):
// undamped Jacobi with edge ghosts, coarse levels that keep the fine dx/dy,
// unscaled 2x2-average restriction, a prolongation that leaves the last fine
// row and column zero, 10 coarsest sweeps, outlet row reset after each smoothing
// phase, and the absolute early exit sum(r^2) dx dy < tol^2 after each cycle.
// The second post-smoothing sweep and the prolongation are fused (the sweep
// evaluates p + P(e) on the fly), so each level costs five kernels.
//
// Converging mode (new) solves the same discrete operator to a relative
// residual: FP64 iterative refinement (r = b - A p in FP64, one FP32 V-cycle on
// A e = r, p += e) with red-black Gauss-Seidel smoothing in shared-memory tiles,
// rediscretised coarse operators, cell-centred bilinear prolongation, an FP64
// dense solve on the coarsest grid and FP64 norms.  The refinement loop is a
// CUDA-graph while node whose condition the check kernel sets on the device.
#include "aj_internal.cuh"
#include <math.h>
#include <vector>
#include <string.h>

namespace aj {

// ====================================================================== common
__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// block-wide sum of one double into *dst (atomic); blockDim multiple of 32
__device__ __forceinline__ void block_sum_atomic(double v, double* dst) {
  __shared__ double ws_[32];
  v = warp_sum(v);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int nthreads = blockDim.x * blockDim.y;
  int tid = threadIdx.y * blockDim.x + threadIdx.x;
  lane = tid & 31;
  w = tid >> 5;
  if (lane == 0) ws_[w] = v;
  __syncthreads();
  if (w == 0) {
    v = lane < (nthreads >> 5) ? ws_[lane] : 0.0;
    v = warp_sum(v);
    if (lane == 0) atomicAdd(dst, v);
  }
}

// b = rhs (* mask for MAC), b[-1, :] = 0 (multigrid_solver.py:75-77,
// multigrid_solver_mac.py:78-83)
__global__ void k_mg_rhs(const float* __restrict__ rhs, const float* __restrict__ mask,
                         float* __restrict__ b, int nx, int ny, int mac) {
  long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= (long)nx * ny) return;
  int i = (int)(k / ny);
  float v = mac ? rhs[k] * mask[k] : rhs[k];
  b[k] = (i == nx - 1) ? 0.f : v;
}

int launch_mg_rhs(const AjStepParams& p, const Layout& L, void* ws, const float* rhs,
                  const float* mask, cudaStream_t st) {
  long n = (long)p.nx * p.ny;
  k_mg_rhs<<<cdiv(n, 256), 256, 0, st>>>(rhs, mask, at<float>(ws, L.b0), p.nx, p.ny,
                                         p.grid_type == AJ_GRID_MAC);
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

// ====================================================================== parity
// restriction of a mask level followed by the > 0.5 threshold
// (multigrid_solver_mac.py:213-214)
__global__ void k_mask_restrict(const float* __restrict__ mf, float* __restrict__ mc, int n,
                                int m) {
  int J = blockIdx.x * blockDim.x + threadIdx.x;
  int I = blockIdx.y * blockDim.y + threadIdx.y;
  int nc = n / 2, mc_ = m / 2;
  if (I >= nc || J >= mc_) return;
  const float* f = mf + (long)(2 * I) * m + 2 * J;
  float r = 0.25f * (f[0] + f[m] + f[1] + f[m + 1]);
  mc[(long)I * mc_ + J] = r > 0.5f ? 1.f : 0.f;
}

// value of the reference prolongation at fine (a, b) from coarse c (nc x mc)
__device__ __forceinline__ float prolong_ref(const float* __restrict__ c, int nc, int mc, int a,
                                             int b) {
  int I = a >> 1, J = b >> 1, ao = a & 1, bo = b & 1;
  if (!ao && !bo) return ldg(c + (long)I * mc + J);
  if (ao && !bo) return I <= nc - 2 ? 0.5f * (ldg(c + (long)I * mc + J) + ldg(c + (long)(I + 1) * mc + J)) : 0.f;
  if (!ao && bo) return J <= mc - 2 ? 0.5f * (ldg(c + (long)I * mc + J) + ldg(c + (long)I * mc + J + 1)) : 0.f;
  if (I <= nc - 2 && J <= mc - 2)
    return 0.25f * (ldg(c + (long)I * mc + J) + ldg(c + (long)(I + 1) * mc + J) +
                    ldg(c + (long)I * mc + J + 1) + ldg(c + (long)(I + 1) * mc + J + 1));
  return 0.f;
}

struct ParJac {
  const float* pin;    // null = zero guess
  const float* ec;     // coarse correction to add on the fly (null = none)
  const float* b;
  const float* mask;   // MAC: p_new *= mask
  float* pout;
  const int* skip;
  int n, m, nc, mc, zero_last;
  float ax, ay, den;
};

// one undamped Jacobi sweep with edge ghosts (multigrid_solver.py:158-171)
__global__ void __launch_bounds__(256) k_par_jacobi(ParJac a) {
  if (a.skip && *a.skip) return;
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= a.n || j >= a.m) return;
  auto pv = [&](int ii, int jj) -> float {
    float v = a.pin ? ldg(a.pin + (long)ii * a.m + jj) : 0.f;
    if (a.ec) v = v + prolong_ref(a.ec, a.nc, a.mc, ii, jj);
    return v;
  };
  int ip = i + 1 < a.n ? i + 1 : a.n - 1, im = i > 0 ? i - 1 : 0;
  int jp = j + 1 < a.m ? j + 1 : a.m - 1, jm = j > 0 ? j - 1 : 0;
  long k = (long)i * a.m + j;
  float pn = (a.ax * (pv(ip, j) + pv(im, j)) + a.ay * (pv(i, jp) + pv(i, jm)) - ldg(a.b + k)) / a.den;
  if (a.mask) pn = pn * ldg(a.mask + k);
  if (a.zero_last && i == a.n - 1) pn = 0.f;
  a.pout[k] = pn;
}

// residual r = b - A p (edge ghosts; MAC zeroes the outlet row of A p) and its
// unscaled 2x2 average onto the coarse grid (multigrid_solver.py:108-132, 173-201)
__global__ void __launch_bounds__(256) k_par_resid_restrict(const float* __restrict__ p,
                                                            const float* __restrict__ b,
                                                            float* __restrict__ rc, int n, int m,
                                                            float ax, float ay, int mac_outlet,
                                                            const int* skip) {
  if (skip && *skip) return;
  int J = blockIdx.x * blockDim.x + threadIdx.x;
  int I = blockIdx.y * blockDim.y + threadIdx.y;
  int nc = n / 2, mc = m / 2;
  if (I >= nc || J >= mc) return;
  float r[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    int i = 2 * I + (q & 1), j = 2 * J + (q >> 1);   // order: (0,0),(1,0),(0,1),(1,1)
    long k = (long)i * m + j;
    float c = ldg(p + k);
    float xp = ldg(p + (long)(i + 1 < n ? i + 1 : n - 1) * m + j);
    float xm = ldg(p + (long)(i > 0 ? i - 1 : 0) * m + j);
    float yp = ldg(p + (long)i * m + (j + 1 < m ? j + 1 : m - 1));
    float ym = ldg(p + (long)i * m + (j > 0 ? j - 1 : 0));
    float lap = ax * (xp + xm - 2.f * c) + ay * (yp + ym - 2.f * c);
    if (mac_outlet && i == n - 1) lap = 0.f;
    r[q] = ldg(b + k) - lap;
  }
  rc[(long)I * mc + J] = 0.25f * (r[0] + r[1] + r[2] + r[3]);
}

// sum over the fine grid of (b - A p)^2 in FP64 (multigrid_solver.py:229-231)
__global__ void __launch_bounds__(256) k_par_norm(const float* __restrict__ p,
                                                  const float* __restrict__ b, int n, int m,
                                                  float ax, float ay, int mac_outlet,
                                                  DevScalars* sc, int also_b) {
  if (sc->mg_skip) return;
  double acc = 0.0, accb = 0.0;
  long N = (long)n * m;
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < N; k += (long)gridDim.x * blockDim.x) {
    int i = (int)(k / m), j = (int)(k - (long)i * m);
    float c = ldg(p + k);
    float xp = ldg(p + (long)(i + 1 < n ? i + 1 : n - 1) * m + j);
    float xm = ldg(p + (long)(i > 0 ? i - 1 : 0) * m + j);
    float yp = ldg(p + (long)i * m + (j + 1 < m ? j + 1 : m - 1));
    float ym = ldg(p + (long)i * m + (j > 0 ? j - 1 : 0));
    float lap = ax * (xp + xm - 2.f * c) + ay * (yp + ym - 2.f * c);
    if (mac_outlet && i == n - 1) lap = 0.f;
    float bb = ldg(b + k);
    double r = (double)bb - (double)lap;
    acc += r * r;
    accb += (double)bb * (double)bb;
  }
  block_sum_atomic(acc, &sc->acc[0]);
  if (also_b) {
    __syncthreads();
    block_sum_atomic(accb, &sc->acc[1]);
  }
}

__global__ void k_par_begin(DevScalars* sc) {
  sc->mg_skip = 0;
  sc->mg_cycles = 0;
  sc->acc[0] = 0.0;
  sc->acc[1] = 0.0;
  sc->err = AJ_OK;
}

// converged = sum r^2 dx dy < tol^2 (multigrid_solver.py:222-232)
__global__ void k_par_check(DevScalars* sc, double dxdy, double tol2, int first) {
  if (sc->mg_skip) return;
  if (first) sc->bnorm = sqrt(sc->acc[1]);
  double s = sc->acc[0];
  sc->mg_cycles += 1;
  sc->abs_sq = s * dxdy;
  sc->rel = sc->bnorm > 0.0 ? sqrt(s) / sc->bnorm : sqrt(s);
  if (!isfinite(s)) sc->err = AJ_ERR_NONFINITE;
  sc->mg_skip = (s * dxdy < tol2) ? 1 : 0;
  sc->acc[0] = 0.0;
  sc->acc[1] = 0.0;
}

__global__ void k_copy(const float* __restrict__ s, float* __restrict__ d, long n) {
  long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k < n) d[k] = s[k];
}

__global__ void k_stats(const DevScalars* sc, AjStats* st, int converge_mode) {
  st->cycles = sc->mg_cycles;
  st->converged = converge_mode ? sc->mg_done : sc->mg_skip;
  st->err = sc->err;
  st->pad = 0;
  st->rel_residual = sc->rel;
  st->rhs_norm = sc->bnorm;
  st->dt = sc->dt;
  st->abs_residual_sq = sc->abs_sq;
}

static int parity_solve(const AjStepParams& p, const Layout& L, void* ws, const float* mask,
                        const float* p0, float* pout, cudaStream_t st) {
  DevScalars* sc = at<DevScalars>(ws, 0);
  const int mac = p.grid_type == AJ_GRID_MAC;
  const float ax = (float)(1.0 / (p.dx * p.dx)), ay = (float)(1.0 / (p.dy * p.dy));
  const float den = (float)(2.0 * (1.0 / (p.dx * p.dx) + 1.0 / (p.dy * p.dy)));
  const double tol = p.mg_tolerance > 0 ? p.mg_tolerance : AJ_PARITY_TOL_DEFAULT;
  const int nl = L.nlev;
  float* b0 = at<float>(ws, L.b0);
  float* T0 = at<float>(ws, L.T0);
  const int* skip = &sc->mg_skip;
  dim3 blk(32, 8);
  k_par_begin<<<1, 1, 0, st>>>(sc);
  if (p0) k_copy<<<cdiv((long)p.nx * p.ny, 256), 256, 0, st>>>(p0, pout, (long)p.nx * p.ny);

  auto X = [&](int l) { return l == 0 ? pout : at<float>(ws, L.X[l]); };
  auto T = [&](int l) { return l == 0 ? T0 : at<float>(ws, L.T[l]); };
  auto B = [&](int l) { return l == 0 ? b0 : at<float>(ws, L.B[l]); };
  auto M = [&](int l) -> const float* {
    if (!mac) return nullptr;
    return l == 0 ? mask : at<float>(ws, L.M[l]);
  };
  for (int cyc = 0; cyc < p.v_cycles; ++cyc) {
    const int* sk = cyc == 0 ? nullptr : skip;   // the first cycle always runs
    // down sweep of the V: levels 0..nl-1
    for (int l = 0; l < nl; ++l) {
      int n = L.ln[l], m = L.lm[l];
      dim3 g(cdiv(m, 32), cdiv(n, 8));
      bool zero_in = (l > 0) || (cyc == 0 && !p0);
      ParJac a{};
      a.b = B(l);
      a.mask = M(l);
      a.skip = sk;
      a.n = n;
      a.m = m;
      a.ax = ax;
      a.ay = ay;
      a.den = den;
      // sweep 1: X -> T (or zero -> T)
      a.pin = zero_in ? nullptr : X(l);
      a.pout = T(l);
      a.zero_last = 0;
      k_par_jacobi<<<g, blk, 0, st>>>(a);
      // sweep 2: T -> X, outlet row reset
      a.pin = T(l);
      a.pout = X(l);
      a.zero_last = p.flow_type == AJ_FLOW_VON_KARMAN;
      k_par_jacobi<<<g, blk, 0, st>>>(a);
      dim3 gc(cdiv(m / 2, 32), cdiv(n / 2, 8));
      k_par_resid_restrict<<<gc, blk, 0, st>>>(X(l), B(l), B(l + 1), n, m, ax, ay,
                                               mac && p.flow_type == AJ_FLOW_VON_KARMAN, sk);
    }
    // coarsest: 10 sweeps from zero, ending in X
    {
      int n = L.ln[nl], m = L.lm[nl];
      dim3 g(cdiv(m, 32), cdiv(n, 8));
      ParJac a{};
      a.b = B(nl);
      a.mask = M(nl);
      a.skip = sk;
      a.n = n;
      a.m = m;
      a.ax = ax;
      a.ay = ay;
      a.den = den;
      for (int s = 0; s < 10; ++s) {
        a.pin = s == 0 ? nullptr : (s % 2 == 1 ? T(nl) : X(nl));
        a.pout = s % 2 == 0 ? T(nl) : X(nl);
        k_par_jacobi<<<g, blk, 0, st>>>(a);
      }
    }
    // up sweep: p + P(e) fused into post-sweep 1, then post-sweep 2
    for (int l = nl - 1; l >= 0; --l) {
      int n = L.ln[l], m = L.lm[l];
      dim3 g(cdiv(m, 32), cdiv(n, 8));
      ParJac a{};
      a.b = B(l);
      a.mask = M(l);
      a.skip = sk;
      a.n = n;
      a.m = m;
      a.nc = L.ln[l + 1];
      a.mc = L.lm[l + 1];
      a.ax = ax;
      a.ay = ay;
      a.den = den;
      a.pin = X(l);
      a.ec = X(l + 1);
      a.pout = T(l);
      a.zero_last = 0;
      k_par_jacobi<<<g, blk, 0, st>>>(a);
      a.pin = T(l);
      a.ec = nullptr;
      a.pout = X(l);
      a.zero_last = p.flow_type == AJ_FLOW_VON_KARMAN;
      k_par_jacobi<<<g, blk, 0, st>>>(a);
    }
    k_par_norm<<<cdiv((long)p.nx * p.ny, 256 * 4) < 1216 ? cdiv((long)p.nx * p.ny, 256 * 4) : 1216,
                 256, 0, st>>>(pout, b0, p.nx, p.ny, ax, ay, mac && p.flow_type == AJ_FLOW_VON_KARMAN,
                               sc, cyc == 0);
    k_par_check<<<1, 1, 0, st>>>(sc, p.dx * p.dy, tol * tol, cyc == 0);
  }
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

// ==================================================================== converge
// Tiles: 32 rows (x) by 64 columns (y); two red-black sweeps per smoothing phase.
constexpr int CV_TI = 32, CV_TJ = 64, CV_NS = 2;
constexpr int CV_HD = 2 * CV_NS + 1;   // down kernel halo (sweeps + residual)
constexpr int CV_HU = 2 * CV_NS;       // up kernel halo
constexpr int CV_SID = CV_TI + 2 * CV_HD, CV_SJD = CV_TJ + 2 * CV_HD;
constexpr int CV_SIU = CV_TI + 2 * CV_HU, CV_SJU = CV_TJ + 2 * CV_HU;

struct CvLvl {
  int n, m, level;
  float ax, ay, g;   // g: outlet ghost factor of this level (level >= 1)
};

__device__ __forceinline__ float cv_diag(const CvLvl& L, int gi, int gj) {
  float d = -2.f * (L.ax + L.ay);
  if (gi == 0) d += L.ax;
  if (gj == 0) d += L.ay;
  if (gj == L.m - 1) d += L.ay;
  if (gi == L.n - 1) d += (L.level == 0) ? L.ax : L.ax * L.g;
  return d;
}

// red-black half-sweeps over a shared-memory tile; cells outside the domain
// hold zero and never change (the diagonal carries the ghost rule).  Every
// half-sweep covers the whole tile: after half-sweep h the cells at distance
// >= h+1 from the tile border hold exact red-black values, and the cells
// nearer the border (stale neighbours) lie outside every value that is stored.
template <int SI, int SJ>
__device__ __forceinline__ void cv_sweeps(float* E, const float* R, const CvLvl& L, int gi0,
                                          int gj0, int nhalf) {
  constexpr int ROWS = SI - 2, HW = (SJ - 1) / 2;   // cells of one colour per row (upper bound)
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int nth = blockDim.x * blockDim.y;
  const float inv_int = 1.f / (-2.f * (L.ax + L.ay));
  for (int h = 0; h < nhalf; ++h) {
    const int color = h & 1;
    for (int t = tid; t < ROWS * HW; t += nth) {
      const int r = t / HW, kk = t - r * HW;
      const int ti = 1 + r;
      const int tj = 1 + ((color - ti - 1) & 1) + 2 * kk;
      if (tj >= SJ - 1) continue;
      const int gi = gi0 + ti, gj = gj0 + tj;
      if ((unsigned)gi >= (unsigned)L.n || (unsigned)gj >= (unsigned)L.m) continue;
      if (L.level == 0 && gi == L.n - 1) continue;          // pinned outlet row
      const int c = ti * SJ + tj;
      const float nb = L.ax * (E[c + SJ] + E[c - SJ]) + L.ay * (E[c + 1] + E[c - 1]);
      const bool inner = gi > 0 && gi < L.n - 1 && gj > 0 && gj < L.m - 1;
      E[c] = (R[c] - nb) * (inner ? inv_int : 1.f / cv_diag(L, gi, gj));
    }
    __syncthreads();
  }
}

// pre-smoothing from e = 0, residual, 2x2 average onto the coarse rhs
__global__ void __launch_bounds__(256) k_cv_down(CvLvl L, const float* __restrict__ r,
                                                 float* __restrict__ e_out,
                                                 float* __restrict__ rc, const int* done) {
  if (*done) return;
  __shared__ float E[CV_SID * CV_SJD];
  __shared__ float R[CV_SID * CV_SJD];
  const int i0 = blockIdx.y * CV_TI, j0 = blockIdx.x * CV_TJ;
  const int gi0 = i0 - CV_HD, gj0 = j0 - CV_HD;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, nth = blockDim.x * blockDim.y;
  for (int t = tid; t < CV_SID * CV_SJD; t += nth) {
    int ti = t / CV_SJD, tj = t - ti * CV_SJD;
    int gi = gi0 + ti, gj = gj0 + tj;
    bool in = gi >= 0 && gi < L.n && gj >= 0 && gj < L.m;
    E[t] = 0.f;
    R[t] = in ? ldg(r + (long)gi * L.m + gj) : 0.f;
  }
  __syncthreads();
  cv_sweeps<CV_SID, CV_SJD>(E, R, L, gi0, gj0, 2 * CV_NS);
  // store e and compute the residual on the tile interior (in place in R)
  for (int t = tid; t < CV_TI * CV_TJ; t += nth) {
    int ti = CV_HD + t / CV_TJ, tj = CV_HD + t % CV_TJ;
    int gi = gi0 + ti, gj = gj0 + tj;
    if (gi >= L.n || gj >= L.m) continue;
    const int c = ti * CV_SJD + tj;
    e_out[(long)gi * L.m + gj] = E[c];
    float res = 0.f;
    if (!(L.level == 0 && gi == L.n - 1)) {
      float nb = L.ax * (E[c + CV_SJD] + E[c - CV_SJD]) + L.ay * (E[c + 1] + E[c - 1]);
      res = R[c] - (nb + cv_diag(L, gi, gj) * E[c]);
    }
    R[c] = res;
  }
  __syncthreads();
  const int mc = L.m >> 1, nc = L.n >> 1;
  for (int t = tid; t < (CV_TI / 2) * (CV_TJ / 2); t += nth) {
    int ci = t / (CV_TJ / 2), cj = t % (CV_TJ / 2);
    int I = (i0 >> 1) + ci, J = (j0 >> 1) + cj;
    if (I >= nc || J >= mc) continue;
    int c = (CV_HD + 2 * ci) * CV_SJD + CV_HD + 2 * cj;
    rc[(long)I * mc + J] = 0.25f * (R[c] + R[c + CV_SJD] + R[c + 1] + R[c + CV_SJD + 1]);
  }
}

// cell-centred bilinear prolongation of the coarse correction (ghosts:
// Neumann copies at inlet and walls, outlet ghost g * value)
__device__ __forceinline__ float cv_prolong(const float* __restrict__ ec, int nc, int mc, float g,
                                            int gi, int gj) {
  int I = gi >> 1, J = gj >> 1;
  int Ii = (gi & 1) ? I + 1 : I - 1;
  int Jj = (gj & 1) ? J + 1 : J - 1;
  Jj = Jj < 0 ? 0 : (Jj >= mc ? mc - 1 : Jj);
  auto cval = [&](int a, int b) -> float {
    if (a < 0) a = 0;
    if (a >= nc) return g * ldg(ec + (long)(nc - 1) * mc + b);
    return ldg(ec + (long)a * mc + b);
  };
  float c0 = ldg(ec + (long)I * mc + J);
  return (9.f * c0 + 3.f * cval(Ii, J) + 3.f * cval(I, Jj) + cval(Ii, Jj)) * (1.f / 16.f);
}

// e + P(e_coarse), post-smoothing, store (level 0: p64 += e instead)
__global__ void __launch_bounds__(256) k_cv_up(CvLvl L, const float* __restrict__ r,
                                               const float* __restrict__ e_in,
                                               const float* __restrict__ ec, int nc, int mc,
                                               float gc, float* __restrict__ e_out,
                                               double* __restrict__ p64, const int* done) {
  if (*done) return;
  __shared__ float E[CV_SIU * CV_SJU];
  __shared__ float R[CV_SIU * CV_SJU];
  const int i0 = blockIdx.y * CV_TI, j0 = blockIdx.x * CV_TJ;
  const int gi0 = i0 - CV_HU, gj0 = j0 - CV_HU;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, nth = blockDim.x * blockDim.y;
  for (int t = tid; t < CV_SIU * CV_SJU; t += nth) {
    int ti = t / CV_SJU, tj = t - ti * CV_SJU;
    int gi = gi0 + ti, gj = gj0 + tj;
    bool in = gi >= 0 && gi < L.n && gj >= 0 && gj < L.m;
    float e = 0.f, rr = 0.f;
    if (in) {
      long k = (long)gi * L.m + gj;
      rr = ldg(r + k);
      if (!(L.level == 0 && gi == L.n - 1)) e = ldg(e_in + k) + cv_prolong(ec, nc, mc, gc, gi, gj);
    }
    E[t] = e;
    R[t] = rr;
  }
  __syncthreads();
  cv_sweeps<CV_SIU, CV_SJU>(E, R, L, gi0, gj0, 2 * CV_NS);
  for (int t = tid; t < CV_TI * CV_TJ; t += nth) {
    int ti = CV_HU + t / CV_TJ, tj = CV_HU + t % CV_TJ;
    int gi = gi0 + ti, gj = gj0 + tj;
    if (gi >= L.n || gj >= L.m) continue;
    long k = (long)gi * L.m + gj;
    float e = E[ti * CV_SJU + tj];
    if (p64) p64[k] += (double)e;
    else e_out[k] = e;
  }
}

// coarsest grid: e = A^-1 r with the FP64 inverse (one warp per row)
__global__ void k_cv_coarse(const double* __restrict__ Ainv, const float* __restrict__ rc,
                            float* __restrict__ ec, int N, const int* done) {
  if (*done) return;
  extern __shared__ double rs[];
  for (int t = threadIdx.x; t < N; t += blockDim.x) rs[t] = (double)rc[t];
  __syncthreads();
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int row = blockIdx.x * (blockDim.x >> 5) + warp;
  if (row >= N) return;
  const double* a = Ainv + (long)row * N;
  double s = 0.0;
  for (int c = lane; c < N; c += 32) s += a[c] * rs[c];
  s = warp_sum(s);
  if (lane == 0) ec[row] = (float)s;
}

// p64 = p0 (or 0), outlet row pinned
__global__ void k_cv_init(const float* __restrict__ p0, double* __restrict__ p64, int n, int m) {
  long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= (long)n * m) return;
  int i = (int)(k / m);
  p64[k] = (p0 && i != n - 1) ? (double)p0[k] : 0.0;
}

// FP64 residual of the reference operator: r = b - A p (edge ghosts, outlet
// row pinned at 0 and excluded), stored as FP32 for the V-cycle; FP64 sums
__global__ void __launch_bounds__(256) k_cv_resid(const double* __restrict__ p64,
                                                  const float* __restrict__ b,
                                                  float* __restrict__ r, int n, int m, double ax,
                                                  double ay, DevScalars* sc, int first) {
  if (!first && sc->mg_done) return;
  double acc = 0.0, accb = 0.0;
  long N = (long)n * m;
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < N; k += (long)gridDim.x * blockDim.x) {
    int i = (int)(k / m), j = (int)(k - (long)i * m);
    double rr = 0.0;
    if (i != n - 1) {
      double c = p64[k];
      double xp = p64[(long)(i + 1) * m + j];
      double xm = p64[(long)(i > 0 ? i - 1 : 0) * m + j];
      double yp = p64[(long)i * m + (j + 1 < m ? j + 1 : m - 1)];
      double ym = p64[(long)i * m + (j > 0 ? j - 1 : 0)];
      double bb = (double)b[k];
      rr = bb - (ax * (xp + xm - 2.0 * c) + ay * (yp + ym - 2.0 * c));
      accb += bb * bb;
    }
    r[k] = (float)rr;
    acc += rr * rr;
  }
  block_sum_atomic(acc, &sc->acc[0]);
  if (first) {
    __syncthreads();
    block_sum_atomic(accb, &sc->acc[1]);
  }
}

__global__ void k_cv_begin(DevScalars* sc) {
  sc->mg_done = 0;
  sc->loops = 0;
  sc->mg_cycles = 0;
  sc->acc[0] = 0.0;
  sc->acc[1] = 0.0;
  sc->err = AJ_OK;
}

// relative residual test; drives the graph's while node when h != 0
__global__ void k_cv_check(DevScalars* sc, double rtol, int max_cycles, int first,
                           cudaGraphConditionalHandle h, int use_handle) {
  if (first) {
    sc->bnorm = sqrt(sc->acc[1]);
  } else if (!sc->mg_done) {
    sc->mg_cycles += 1;
  }
  if (first || !sc->mg_done) {
    double nb = sc->bnorm > 0.0 ? sc->bnorm : 1.0;
    double rel = sqrt(sc->acc[0]) / nb;
    sc->rel = rel;
    sc->abs_sq = sc->acc[0];
    if (!isfinite(rel)) {
      sc->err = AJ_ERR_NONFINITE;
      sc->mg_done = 1;
    } else if (rel <= rtol) {
      sc->mg_done = 1;
    } else if (sc->mg_cycles >= max_cycles) {
      sc->err = AJ_ERR_NOT_CONVERGED;
      sc->mg_done = 1;
    }
  }
  sc->acc[0] = 0.0;
  sc->acc[1] = 0.0;
  if (use_handle) {
    // independent bound on the while node: never more bodies than max_cycles + 1
    sc->loops += 1;
    if (sc->loops > max_cycles + 1 && !sc->mg_done) {
      sc->err = AJ_ERR_NOT_CONVERGED;
      sc->mg_done = 1;
    }
    cudaGraphSetConditional(h, sc->mg_done ? 0u : 1u);
  }
}

__global__ void k_cv_out(const double* __restrict__ p64, float* __restrict__ p, long N) {
  long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k < N) p[k] = (float)p64[k];
}

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

// the body of one refinement iteration: V-cycle, then residual + check
static void cv_body(const AjStepParams& p, const Layout& L, void* ws,
                    cudaGraphConditionalHandle h, int use_handle, cudaStream_t st) {
  DevScalars* sc = at<DevScalars>(ws, 0);
  const int* done = &sc->mg_done;
  const int D = L.nlev;
  dim3 blk(32, 8);
  double* p64 = at<double>(ws, L.p64);
  for (int l = 0; l < D; ++l) {
    CvLvl c = cv_level(p, L, l);
    dim3 g(cdiv(c.m, CV_TJ), cdiv(c.n, CV_TI));
    k_cv_down<<<g, blk, 0, st>>>(c, at<float>(ws, L.B[l]), at<float>(ws, L.X[l]),
                                 at<float>(ws, L.B[l + 1]), done);
  }
  {
    int N = L.ncoarse;
    int rows_per_block = 8;
    k_cv_coarse<<<cdiv(N, rows_per_block), 256, N * sizeof(double), st>>>(
        at<double>(ws, L.cinv), at<float>(ws, L.B[D]), at<float>(ws, L.T[D]), N, done);
  }
  for (int l = D - 1; l >= 0; --l) {
    CvLvl c = cv_level(p, L, l);
    dim3 g(cdiv(c.m, CV_TJ), cdiv(c.n, CV_TI));
    float gc = (float)ghost_factor(l + 1);
    k_cv_up<<<g, blk, 0, st>>>(c, at<float>(ws, L.B[l]), at<float>(ws, L.X[l]),
                               at<float>(ws, L.T[l + 1]), L.ln[l + 1], L.lm[l + 1], gc,
                               l == 0 ? nullptr : at<float>(ws, L.T[l]), l == 0 ? p64 : nullptr,
                               done);
  }
  long N = (long)p.nx * p.ny;
  unsigned nb = cdiv(N, 256 * 4);
  if (nb > 1216) nb = 1216;
  k_cv_resid<<<nb, 256, 0, st>>>(p64, at<float>(ws, L.b0), at<float>(ws, L.B[0]), p.nx, p.ny,
                                 1.0 / (p.dx * p.dx), 1.0 / (p.dy * p.dy), sc, 0);
  k_cv_check<<<1, 1, 0, st>>>(sc, p.mg_rtol, p.max_cycles, 0, h, use_handle);
}

static cudaStream_t side_stream() {
  static cudaStream_t s = nullptr;
  if (!s) cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  return s;
}

static int converge_solve(const AjStepParams& p, const Layout& L, void* ws, const float* p0,
                          float* pout, cudaStream_t st) {
  DevScalars* sc = at<DevScalars>(ws, 0);
  long N = (long)p.nx * p.ny;
  double* p64 = at<double>(ws, L.p64);
  k_cv_begin<<<1, 1, 0, st>>>(sc);
  k_cv_init<<<cdiv(N, 256), 256, 0, st>>>(p.warm_start ? p0 : nullptr, p64, p.nx, p.ny);
  unsigned nb = cdiv(N, 256 * 4);
  if (nb > 1216) nb = 1216;
  k_cv_resid<<<nb, 256, 0, st>>>(p64, at<float>(ws, L.b0), at<float>(ws, L.B[0]), p.nx, p.ny,
                                 1.0 / (p.dx * p.dx), 1.0 / (p.dy * p.dy), sc, 1);
  k_cv_check<<<1, 1, 0, st>>>(sc, p.mg_rtol, p.max_cycles, 1, 0, 0);

  // the refinement loop: a while node appended to the graph being captured
  cudaStreamCaptureStatus cs;
  unsigned long long id;
  cudaGraph_t g;
  const cudaGraphNode_t* deps;
  const cudaGraphEdgeData* ed;
  size_t nd;
  if (cudaStreamGetCaptureInfo(st, &cs, &id, &g, &deps, &ed, &nd) != cudaSuccess)
    return AJ_ERR_CUDA;
  if (cs != cudaStreamCaptureStatusActive) {
    // eager launches (profiling mode, see aj_api.cu): a fixed number of loop
    // bodies, each skipping its work once the target is met
    int unroll = eager_unroll(p.max_cycles);
    for (int k = 0; k < unroll; ++k) cv_body(p, L, ws, 0, 0, st);
    k_cv_out<<<cdiv(N, 256), 256, 0, st>>>(p64, pout, N);
    return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
  }
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
  if (cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies) !=
      cudaSuccess)
    return AJ_ERR_CUDA;
  cudaGraph_t body = np.conditional.phGraph_out[0];
  cudaStream_t side = side_stream();
  if (cudaStreamBeginCaptureToGraph(side, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) !=
      cudaSuccess)
    return AJ_ERR_CUDA;
  cv_body(p, L, ws, h, 1, side);
  cudaGraph_t out;
  if (cudaStreamEndCapture(side, &out) != cudaSuccess) return AJ_ERR_CUDA;

  k_cv_out<<<cdiv(N, 256), 256, 0, st>>>(p64, pout, N);
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

// ===================================================================== set-up
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
  // Gauss-Jordan with partial pivoting
  for (int c = 0; c < N; ++c) {
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

int prepare_pressure(const AjStepParams& p, const Layout& L, void* ws, const float* mask,
                     cudaStream_t st) {
  if (p.mg_mode == AJ_MG_PARITY) {
    if (p.grid_type == AJ_GRID_MAC) {
      dim3 blk(32, 8);
      for (int l = 0; l < L.nlev; ++l) {
        const float* mf = l == 0 ? mask : at<float>(ws, L.M[l]);
        int n = L.ln[l], m = L.lm[l];
        dim3 g(cdiv(m / 2, 32), cdiv(n / 2, 8));
        k_mask_restrict<<<g, blk, 0, st>>>(mf, at<float>(ws, L.M[l + 1]), n, m);
      }
    }
  } else {
    std::vector<double> inv;
    if (!coarse_inverse(p, L, inv)) return AJ_ERR_PARAM;
    if (cudaMemcpyAsync(at<double>(ws, L.cinv), inv.data(), inv.size() * sizeof(double),
                        cudaMemcpyHostToDevice, st) != cudaSuccess)
      return AJ_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return AJ_ERR_CUDA;
  }
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

// One launch of a converging-mode level-0 kernel on the workspace's current
// contents (instrumentation: lets a caller time the kernel on its own).
// which: 0 = smoothing + residual + restriction, 1 = prolongation + smoothing +
// FP64 update, 2 = FP64 residual and norms.
int profile_pressure_kernel(const AjStepParams& p, const Layout& L, void* ws, int which,
                            cudaStream_t st) {
  if (p.mg_mode != AJ_MG_CONVERGE) return AJ_ERR_PARAM;
  DevScalars* sc = at<DevScalars>(ws, 0);
  const int* never = reinterpret_cast<const int*>(&sc->pad_[0]);   // always 0
  dim3 blk(32, 8);
  CvLvl c = cv_level(p, L, 0);
  dim3 g(cdiv(c.m, CV_TJ), cdiv(c.n, CV_TI));
  if (which == 0) {
    k_cv_down<<<g, blk, 0, st>>>(c, at<float>(ws, L.B[0]), at<float>(ws, L.X[0]),
                                 at<float>(ws, L.B[1]), never);
  } else if (which == 1) {
    k_cv_up<<<g, blk, 0, st>>>(c, at<float>(ws, L.B[0]), at<float>(ws, L.X[0]),
                               at<float>(ws, L.T[1]), L.ln[1], L.lm[1], (float)ghost_factor(1),
                               nullptr, at<double>(ws, L.p64), never);
  } else if (which == 2) {
    long N = (long)p.nx * p.ny;
    unsigned nb = cdiv(N, 256 * 4);
    if (nb > 1216) nb = 1216;
    k_cv_resid<<<nb, 256, 0, st>>>(at<double>(ws, L.p64), at<float>(ws, L.b0),
                                   at<float>(ws, L.B[0]), p.nx, p.ny, 1.0 / (p.dx * p.dx),
                                   1.0 / (p.dy * p.dy), sc, 1);
  } else {
    return AJ_ERR_PARAM;
  }
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

int launch_pressure(const AjStepParams& p, const Layout& L, void* ws, const float* mask,
                    const float* p0, float* pout, AjStats* stats, cudaStream_t st) {
  int rc;
  if (p.mg_mode == AJ_MG_PARITY) rc = parity_solve(p, L, ws, mask, p0, pout, st);
  else rc = converge_solve(p, L, ws, p0, pout, st);
  if (rc != AJ_OK) return rc;
  if (stats) k_stats<<<1, 1, 0, st>>>(at<DevScalars>(ws, 0), stats, p.mg_mode == AJ_MG_CONVERGE);
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

}  // namespace aj
