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
// The converging mode lives in aj_converge.cu; this file dispatches to it.
#include "aj_internal.cuh"
#include <math.h>

namespace aj {

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

// the coarsest level's 10 Jacobi sweeps from a zero guess
// (multigrid_solver.py:186-187) in one block: the iterate ping-pongs in
// shared memory, b is staged once.  Same arithmetic as k_par_jacobi; used
// when three arrays of the level fit the block's shared memory.
constexpr int kParCoarsestThreads = 1024;
__global__ void __launch_bounds__(kParCoarsestThreads) k_par_coarsest(
    const float* __restrict__ b, const float* __restrict__ mask, float* __restrict__ x, int n,
    int m, float ax, float ay, float den, const int* skip) {
  if (skip && *skip) return;
  extern __shared__ float psm[];
  const int nm = n * m;
  float* P = psm;
  float* Q = psm + nm;
  float* Bs = psm + 2 * nm;
  for (int c = threadIdx.x; c < nm; c += blockDim.x) Bs[c] = b[c];
  __syncthreads();
  for (int s = 0; s < 10; ++s) {
    for (int c = threadIdx.x; c < nm; c += blockDim.x) {
      const int i = c / m, j = c - i * m;
      const int ip = i + 1 < n ? i + 1 : n - 1, im = i > 0 ? i - 1 : 0;
      const int jp = j + 1 < m ? j + 1 : m - 1, jm = j > 0 ? j - 1 : 0;
      auto pv = [&](int ii, int jj) -> float { return s == 0 ? 0.f : P[ii * m + jj]; };
      float pn = (ax * (pv(ip, j) + pv(im, j)) + ay * (pv(i, jp) + pv(i, jm)) - Bs[c]) / den;
      if (mask) pn = pn * mask[c];
      Q[c] = pn;
    }
    __syncthreads();
    float* t = P;
    P = Q;
    Q = t;
  }
  for (int c = threadIdx.x; c < nm; c += blockDim.x) x[c] = P[c];
}

// whether the coarsest level's sweeps run as one k_par_coarsest block
bool parity_coarsest_fused(const Layout& L) {
  return (size_t)L.ln[L.nlev] * L.lm[L.nlev] * 12 <= kBlockSmemMax;
}

__global__ void k_copy(const float* __restrict__ s, float* __restrict__ d, long n) {
  long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k < n) d[k] = s[k];
}

__global__ void k_stats(const DevScalars* sc, AjStats* st, int converge_mode) {
  pdl_wait();
  // all loads before the stores (interleaved, each load waits for a store)
  const int cycles = sc->mg_cycles, conv = converge_mode ? sc->mg_done : sc->mg_skip;
  const int err = sc->err;
  const double rel = sc->rel, bnorm = sc->bnorm, abs_sq = sc->abs_sq;
  const float dt = sc->dt;
  st->cycles = cycles;
  st->converged = conv;
  st->err = err;
  st->pad = 0;
  st->rel_residual = rel;
  st->rhs_norm = bnorm;
  st->dt = dt;
  st->abs_residual_sq = abs_sq;
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
    if (parity_coarsest_fused(L)) {
      const int n = L.ln[nl], m = L.lm[nl];
      const size_t csm = (size_t)n * m * 12;
      cudaFuncSetAttribute(k_par_coarsest, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)kBlockSmemMax);
      k_par_coarsest<<<1, kParCoarsestThreads, csm, st>>>(B(nl), M(nl), X(nl), n, m, ax, ay, den,
                                                           sk);
    } else {
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
    int rc = converge_prepare(p, L, ws, st);
    if (rc != AJ_OK) return rc;
  }
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

int launch_pressure(const AjStepParams& p, const Layout& L, void* ws, const float* mask,
                    const float* p0, float* pout, AjStats* stats, cudaStream_t st,
                    const NnWarm* nn, bool init_done) {
  int rc;
  if (p.mg_mode == AJ_MG_PARITY) {
    rc = parity_solve(p, L, ws, mask, p0, pout, st);
    if (rc != AJ_OK) return rc;
    if (stats) k_stats<<<1, 1, 0, st>>>(at<DevScalars>(ws, 0), stats, 0);
  } else {
    rc = converge_solve(p, L, ws, p0, pout, st, nn, stats, init_done);   // k_cv_out: stats
    if (rc != AJ_OK) return rc;
  }
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

}  // namespace aj
