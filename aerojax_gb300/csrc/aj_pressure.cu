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

#include <cooperative_groups.h>
#include <math.h>

namespace aj {

// b = rhs (* mask for MAC), b[-1, :] = 0 for the von Karman outlet
// (multigrid_solver.py:75-77, multigrid_solver_mac.py:78-83)
__global__ void k_mg_rhs(const float* __restrict__ rhs, const float* __restrict__ mask,
                         float* __restrict__ b, int nx, int ny, int mac, int outlet) {
  long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= (long)nx * ny) return;
  int i = (int)(k / ny);
  float v = mac ? rhs[k] * mask[k] : rhs[k];
  b[k] = (outlet && i == nx - 1) ? 0.f : v;
}

int launch_mg_rhs(const AjStepParams& p, const Layout& L, void* ws, const float* rhs,
                  const float* mask, cudaStream_t st) {
  long n = (long)p.nx * p.ny;
  k_mg_rhs<<<cdiv(n, 256), 256, 0, st>>>(rhs, mask, at<float>(ws, L.b0), p.nx, p.ny,
                                         p.grid_type == AJ_GRID_MAC,
                                         p.flow_type == AJ_FLOW_VON_KARMAN);
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

// ---------------------------------------------------------- other flow types
// Lid-driven cavity: b -= mean(b) before the cycles (multigrid_solver.py:78-80)
// and p -= p[nx/2, ny/2] after them.  The mean: FP64 block partials, summed
// in block order by the last block (reproducible), kept in sc->acc[2].
constexpr int kMeanBlocks = 256;
__global__ void __launch_bounds__(256) k_mean_partials(const float* __restrict__ b, long n,
                                                       DevScalars* sc, double* part) {
  double s = 0.0;
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n;
       k += (long)gridDim.x * blockDim.x)
    s += (double)b[k];
  const double bs = block_sum(s);
  __shared__ int am_last;
  if (threadIdx.x == 0) {
    part[blockIdx.x] = bs;
    __threadfence();
    am_last = atomicAdd(&sc->red_count, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!am_last || threadIdx.x != 0) return;
  __threadfence();
  double t = 0.0;
  for (unsigned q = 0; q < gridDim.x; ++q) t += __ldcg(part + q);
  sc->acc[2] = t / (double)n;
  sc->red_count = 0u;
}
__global__ void k_sub_mean(float* __restrict__ b, long n, const DevScalars* sc) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k < n) b[k] = b[k] - (float)sc->acc[2];
}
__global__ void k_store_center(const float* __restrict__ p, long c, DevScalars* sc) {
  sc->acc[3] = (double)p[c];
}
__global__ void k_sub_center(float* __restrict__ p, long n, const DevScalars* sc) {
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k < n) p[k] = p[k] - (float)sc->acc[3];
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
  const float* b;
  const float* mask;   // MAC: p_new *= mask
  float* pout;
  const int* skip;
  int n, m, zero_last;
  float ax, ay, den;
};

// one undamped Jacobi sweep with edge ghosts (multigrid_solver.py:158-171):
// the coarsest level's sweeps when its bands do not fit the cluster's blocks
__global__ void __launch_bounds__(256) k_par_jacobi(ParJac a) {
  if (a.skip && *a.skip) return;
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= a.n || j >= a.m) return;
  auto pv = [&](int ii, int jj) -> float {
    return a.pin ? ldg(a.pin + (long)ii * a.m + jj) : 0.f;
  };
  int ip = i + 1 < a.n ? i + 1 : a.n - 1, im = i > 0 ? i - 1 : 0;
  int jp = j + 1 < a.m ? j + 1 : a.m - 1, jm = j > 0 ? j - 1 : 0;
  long k = (long)i * a.m + j;
  float pn = (a.ax * (pv(ip, j) + pv(im, j)) + a.ay * (pv(i, jp) + pv(i, jm)) - ldg(a.b + k)) / a.den;
  if (a.mask) pn = pn * ldg(a.mask + k);
  if (a.zero_last && i == a.n - 1) pn = 0.f;
  a.pout[k] = pn;
}

__global__ void k_par_begin(DevScalars* sc) {
  sc->red_count = 0u;
  sc->mg_skip = 0;
  sc->mg_cycles = 0;
  sc->acc[0] = 0.0;
  sc->acc[1] = 0.0;
  sc->err = AJ_OK;
}

// converged = sum r^2 dx dy < tol^2 (multigrid_solver.py:222-232)
// converged = sum r^2 dx dy < tol^2 (multigrid_solver.py:222-232), run by the
// last block of the level-0 up kernel once every block's norm is in
__device__ void par_check_body(DevScalars* sc, double dxdy, double tol2, int first) {
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
// (multigrid_solver.py:186-187) on a cluster of kCoarseCtas blocks: block k
// holds rows [k R, k R + R) of the iterate (ping-pong) and of b in shared
// memory and reads the rows next to its band from its neighbours' shared
// memory.  One cluster barrier per sweep: a sweep reads one buffer and writes
// the other, so after the barrier nobody still reads what the next sweep
// overwrites.  The skip test comes before any barrier and is the same for
// every block; after the last barrier a block reads only its own memory.
// Same arithmetic as k_par_jacobi.
__global__ void __cluster_dims__(kCoarseCtas, 1, 1) __launch_bounds__(kCoarseThreads)
    k_par_coarsest(const float* __restrict__ b, const float* __restrict__ mask,
                   float* __restrict__ x, int n, int m, float ax, float ay, float den,
                   const int* skip) {
  if (skip && *skip) return;
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const int R = coarse_band_rows(n);
  const int r0 = rank * R, nr = max(0, min(n, r0 + R) - r0);
  extern __shared__ float psm[];
  float* P = psm;
  float* Q = psm + R * m;
  float* Bs = psm + 2 * R * m;
  for (int q = threadIdx.x; q < nr * m; q += blockDim.x) Bs[q] = b[(long)r0 * m + q];
  __syncthreads();
  for (int s = 0; s < 10; ++s) {
    for (int q = threadIdx.x; q < nr * m; q += blockDim.x) {
      const int li = q / m, j = q - li * m, i = r0 + li;
      const int ip = i + 1 < n ? i + 1 : n - 1, im = i > 0 ? i - 1 : 0;
      const int jp = j + 1 < m ? j + 1 : m - 1, jm = j > 0 ? j - 1 : 0;
      auto pv = [&](int ii, int jj) -> float {
        if (s == 0) return 0.f;
        const int owner = ii / R;
        const float* base = owner == rank ? P : cl.map_shared_rank(P, owner);
        return base[(ii - owner * R) * m + jj];
      };
      float pn = (ax * (pv(ip, j) + pv(im, j)) + ay * (pv(i, jp) + pv(i, jm)) - Bs[q]) / den;
      if (mask) pn = pn * mask[(long)i * m + j];
      Q[q] = pn;
    }
    cl.sync();
    float* t = P;
    P = Q;
    Q = t;
  }
  for (int q = threadIdx.x; q < nr * m; q += blockDim.x) x[(long)r0 * m + q] = P[q];
}

// whether the coarsest level's sweeps run as one k_par_coarsest block
bool parity_coarsest_fused(const Layout& L) {
  return (size_t)coarse_band_rows(L.ln[L.nlev]) * L.lm[L.nlev] * 12 <= kBlockSmemMax;
}

// ---- one level of the V-cycle per launch, on tiles
// (multigrid_solver.py:173-211).  A tile stages what its output needs with
// halos in shared memory; edge ghosts map to the cell itself; cells outside
// the domain are never read by cells inside it.  Each block writes only its
// own cells, and no output aliases an input another block reads.
struct ParTile {
  const float* xin;   // down: the cycle's input state (null: zero); up: the level's down result
  const float* xc;    // up: the coarser level's result (prolonged on the fly)
  const float* b;
  const float* mask;  // MAC level mask (null: collocated)
  float* xout;        // down: the state after the two pre-sweeps; up: after the post-sweeps
  float* bc;          // down: the restricted residual (the coarser level's b)
  DevScalars* sc;     // up on level 0: the residual norm (multigrid_solver.py:229-231)
  const int* skip;
  int n, m, nc, mc, zero_last, mac_outlet, also_b;
  float ax, ay, den;
  double dxdy, tol2;  // up on level 0: the early-exit test
};
// Output tiles: 16 x 64 on the finest level (4 cells per thread: fewer halo
// cells per output, more loads in flight), 8 x 32 on the coarser ones (their
// grids have few blocks, and a block's dependent phases set the time).
constexpr int kPtThreads = 256;

// Jacobi value at tile cell (r, c) from the staged iterate S (same arithmetic
// as k_par_jacobi); (gi, gj) its global index
template <int RJ>
__device__ __forceinline__ float tile_jacobi(float (*S)[RJ], int r, int c, int gi, int gj,
                                             const ParTile& a) {
  const int rp = gi + 1 < a.n ? r + 1 : r, rm = gi > 0 ? r - 1 : r;
  const int cp = gj + 1 < a.m ? c + 1 : c, cm = gj > 0 ? c - 1 : c;
  const long k = (long)gi * a.m + gj;
  float pn = (a.ax * (S[rp][c] + S[rm][c]) + a.ay * (S[r][cp] + S[r][cm]) - ldg(a.b + k)) / a.den;
  if (a.mask) pn = pn * ldg(a.mask + k);
  return pn;
}

// b - A x at tile cell (r, c) of the staged x (the MAC variant zeroes A x on
// the outlet row)
template <int RJ>
__device__ __forceinline__ float tile_resid(float (*S)[RJ], int r, int c, int gi, int gj,
                                            const ParTile& a) {
  const int rp = gi + 1 < a.n ? r + 1 : r, rm = gi > 0 ? r - 1 : r;
  const int cp = gj + 1 < a.m ? c + 1 : c, cm = gj > 0 ? c - 1 : c;
  const float x = S[r][c];
  float lap = a.ax * (S[rp][c] + S[rm][c] - 2.f * x) + a.ay * (S[r][cp] + S[r][cm] - 2.f * x);
  if (a.mac_outlet && gi == a.n - 1) lap = 0.f;
  return ldg(a.b + (long)gi * a.m + gj) - lap;
}

// down: two pre-sweeps (the second resets the outlet row), the residual and
// its 2x2 average onto the coarser level (multigrid_solver.py:182-201)
template <int kPtBY, int kPtBX>
__global__ void __launch_bounds__(kPtThreads) k_par_down(ParTile a) {
  if (a.skip && *a.skip) return;
  __shared__ float X0[kPtBY + 6][kPtBX + 6];   // input, halo 3
  __shared__ float X1[kPtBY + 4][kPtBX + 4];   // first sweep, halo 2
  __shared__ float X2[kPtBY + 2][kPtBX + 2];   // second sweep, halo 1
  __shared__ float R[kPtBY][kPtBX];            // residual
  const int ti0 = blockIdx.y * kPtBY, tj0 = blockIdx.x * kPtBX;
  const int tid = threadIdx.x, nt = kPtThreads;
  auto inside = [&](int gi, int gj) { return gi >= 0 && gi < a.n && gj >= 0 && gj < a.m; };
  for (int q = tid; q < (kPtBY + 6) * (kPtBX + 6); q += nt) {
    const int r = q / (kPtBX + 6), c = q - r * (kPtBX + 6);
    const int gi = ti0 - 3 + r, gj = tj0 - 3 + c;
    X0[r][c] = (a.xin && inside(gi, gj)) ? ldg(a.xin + (long)gi * a.m + gj) : 0.f;
  }
  __syncthreads();
  for (int q = tid; q < (kPtBY + 4) * (kPtBX + 4); q += nt) {
    const int r = q / (kPtBX + 4), c = q - r * (kPtBX + 4);
    const int gi = ti0 - 2 + r, gj = tj0 - 2 + c;
    X1[r][c] = inside(gi, gj) ? tile_jacobi<kPtBX + 6>(X0, r + 1, c + 1, gi, gj, a) : 0.f;
  }
  __syncthreads();
  for (int q = tid; q < (kPtBY + 2) * (kPtBX + 2); q += nt) {
    const int r = q / (kPtBX + 2), c = q - r * (kPtBX + 2);
    const int gi = ti0 - 1 + r, gj = tj0 - 1 + c;
    float x = 0.f;
    if (inside(gi, gj))
      x = (a.zero_last && gi == a.n - 1) ? 0.f : tile_jacobi<kPtBX + 4>(X1, r + 1, c + 1, gi, gj, a);
    X2[r][c] = x;
  }
  __syncthreads();
  for (int q = tid; q < kPtBY * kPtBX; q += nt) {
    const int r = q / kPtBX, c = q - r * kPtBX;
    const int gi = ti0 + r, gj = tj0 + c;
    float res = 0.f;
    if (inside(gi, gj)) {
      a.xout[(long)gi * a.m + gj] = X2[r + 1][c + 1];
      res = tile_resid<kPtBX + 2>(X2, r + 1, c + 1, gi, gj, a);
    }
    R[r][c] = res;
  }
  __syncthreads();
  for (int q = tid; q < (kPtBY / 2) * (kPtBX / 2); q += nt) {
    const int I = q / (kPtBX / 2), J = q - I * (kPtBX / 2);
    const int gI = ti0 / 2 + I, gJ = tj0 / 2 + J;
    if (gI < a.nc && gJ < a.mc)   // summed in the order (0,0), (1,0), (0,1), (1,1)
      a.bc[(long)gI * a.mc + gJ] =
          0.25f * (R[2 * I][2 * J] + R[2 * I + 1][2 * J] + R[2 * I][2 * J + 1] + R[2 * I + 1][2 * J + 1]);
  }
}

// up: p + P(e) and two post-sweeps (the second resets the outlet row,
// multigrid_solver.py:203-211); with NORM (level 0) also sum (b - A p)^2 and,
// on the first cycle, b^2 (double-FP32 per block, FP64 across blocks)
template <int kPtBY, int kPtBX, bool NORM>
__global__ void __launch_bounds__(kPtThreads) k_par_up(ParTile a) {
  if (a.skip && *a.skip) return;
  constexpr int H = NORM ? 3 : 2;                       // halo of the corrected iterate
  __shared__ float Y[kPtBY + 2 * H][kPtBX + 2 * H];
  __shared__ float X1[kPtBY + 2 * H - 2][kPtBX + 2 * H - 2];
  __shared__ float X2[NORM ? kPtBY + 2 : 1][NORM ? kPtBX + 2 : 1];
  const int ti0 = blockIdx.y * kPtBY, tj0 = blockIdx.x * kPtBX;
  const int tid = threadIdx.x, nt = kPtThreads;
  auto inside = [&](int gi, int gj) { return gi >= 0 && gi < a.n && gj >= 0 && gj < a.m; };
  for (int q = tid; q < (kPtBY + 2 * H) * (kPtBX + 2 * H); q += nt) {
    const int r = q / (kPtBX + 2 * H), c = q - r * (kPtBX + 2 * H);
    const int gi = ti0 - H + r, gj = tj0 - H + c;
    float y = 0.f;
    if (inside(gi, gj)) {
      y = ldg(a.xin + (long)gi * a.m + gj);
      y = y + prolong_ref(a.xc, a.nc, a.mc, gi, gj);
    }
    Y[r][c] = y;
  }
  __syncthreads();
  for (int q = tid; q < (kPtBY + 2 * H - 2) * (kPtBX + 2 * H - 2); q += nt) {
    const int r = q / (kPtBX + 2 * H - 2), c = q - r * (kPtBX + 2 * H - 2);
    const int gi = ti0 - H + 1 + r, gj = tj0 - H + 1 + c;
    X1[r][c] = inside(gi, gj) ? tile_jacobi<kPtBX + 2 * H>(Y, r + 1, c + 1, gi, gj, a) : 0.f;
  }
  __syncthreads();
  auto second = [&](int r, int c, int gi, int gj) {   // (r, c) in X1 coordinates
    return (a.zero_last && gi == a.n - 1) ? 0.f : tile_jacobi<kPtBX + 2 * H - 2>(X1, r, c, gi, gj, a);
  };
  if constexpr (!NORM) {
    for (int q = tid; q < kPtBY * kPtBX; q += nt) {
      const int r = q / kPtBX, c = q - r * kPtBX;
      const int gi = ti0 + r, gj = tj0 + c;
      if (inside(gi, gj)) a.xout[(long)gi * a.m + gj] = second(r + 1, c + 1, gi, gj);
    }
  } else {
  for (int q = tid; q < (kPtBY + 2) * (kPtBX + 2); q += nt) {
    const int r = q / (kPtBX + 2), c = q - r * (kPtBX + 2);
    const int gi = ti0 - 1 + r, gj = tj0 - 1 + c;
    X2[r][c] = inside(gi, gj) ? second(r + 1, c + 1, gi, gj) : 0.f;
  }
  __syncthreads();
  df rr{0.f, 0.f}, bb{0.f, 0.f};
  for (int q = tid; q < kPtBY * kPtBX; q += nt) {
    const int r = q / kPtBX, c = q - r * kPtBX;
    const int gi = ti0 + r, gj = tj0 + c;
    if (inside(gi, gj)) {
      a.xout[(long)gi * a.m + gj] = X2[r + 1][c + 1];
      const float bv = ldg(a.b + (long)gi * a.m + gj);
      const float res = tile_resid<kPtBX + 2>(X2, r + 1, c + 1, gi, gj, a);
      // (b - A p) in FP32 as the reference evaluates it; its square exactly
      rr = df_add(rr, two_prod(res, res));
      bb = df_add(bb, two_prod(bv, bv));
    }
  }
  const double s = block_sum_df(rr);
  const double sb = a.also_b ? block_sum_df(bb) : 0.0;
  __shared__ int am_last;
  if (tid == 0) {
    atomicAdd(&a.sc->acc[0], s);
    if (a.also_b) atomicAdd(&a.sc->acc[1], sb);
    __threadfence();
    am_last = atomicAdd(&a.sc->red_count, 1u) == gridDim.x * gridDim.y - 1;
  }
  __syncthreads();
  if (am_last && tid == 0) {   // every block's sums are in: the early-exit test
    __threadfence();
    a.sc->red_count = 0u;
    par_check_body(a.sc, a.dxdy, a.tol2, a.also_b);
  }
  }
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

// Taylor-Green: the reference's residual wraps periodically while its
// smoother keeps edge ghosts (multigrid_solver.py:158-183), so the residual
// at a boundary cell needs the smoothed iterate on the far side of the
// domain.  Its V-cycle therefore runs unfused: Jacobi sweeps (k_par_jacobi),
// then these kernels.
// r = b - A x with wrapped neighbours, 2x2 average onto the coarser b
__global__ void __launch_bounds__(256) k_tg_resid_restrict(const float* __restrict__ x,
                                                           const float* __restrict__ b,
                                                           float* __restrict__ bc, int n, int m,
                                                           float ax, float ay, const int* skip) {
  if (skip && *skip) return;
  const int J = blockIdx.x * blockDim.x + threadIdx.x;
  const int I = blockIdx.y * blockDim.y + threadIdx.y;
  const int nc = n / 2, mc = m / 2;
  if (I >= nc || J >= mc) return;
  float r[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int i = 2 * I + (q & 1), j = 2 * J + (q >> 1);
    const int ip = i + 1 < n ? i + 1 : 0, im = i > 0 ? i - 1 : n - 1;
    const int jp = j + 1 < m ? j + 1 : 0, jm = j > 0 ? j - 1 : m - 1;
    const float c = ldg(x + (long)i * m + j);
    const float lap = ax * (ldg(x + (long)ip * m + j) + ldg(x + (long)im * m + j) - 2.f * c) +
                      ay * (ldg(x + (long)i * m + jp) + ldg(x + (long)i * m + jm) - 2.f * c);
    r[q] = ldg(b + (long)i * m + j) - lap;
  }
  // summed in the order (0,0), (1,0), (0,1), (1,1) like the tiled kernels
  bc[(long)I * mc + J] = 0.25f * (r[0] + r[1] + r[2] + r[3]);
}
// x += P(xc) in place (the reference prolongation, last row and column 0)
__global__ void __launch_bounds__(256) k_tg_prolong_add(float* __restrict__ x,
                                                        const float* __restrict__ xc, int n,
                                                        int m, const int* skip) {
  if (skip && *skip) return;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= n || j >= m) return;
  const long k = (long)i * m + j;
  x[k] = x[k] + prolong_ref(xc, n / 2, m / 2, i, j);
}
// level 0 after the cycle: sum (b - A x)^2 with wrapped neighbours (and, on
// the first cycle, b^2) in double-FP32 per block, FP64 across blocks; the
// last block runs the early-exit test
__global__ void __launch_bounds__(256) k_tg_norm(const float* __restrict__ x,
                                                 const float* __restrict__ b, int n, int m,
                                                 float ax, float ay, DevScalars* sc, double dxdy,
                                                 double tol2, int also_b, const int* skip) {
  if (skip && *skip) return;
  df rr{0.f, 0.f}, bb{0.f, 0.f};
  const long N = (long)n * m;
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < N;
       k += (long)gridDim.x * blockDim.x) {
    const int i = (int)(k / m), j = (int)(k - (long)i * m);
    const int ip = i + 1 < n ? i + 1 : 0, im = i > 0 ? i - 1 : n - 1;
    const int jp = j + 1 < m ? j + 1 : 0, jm = j > 0 ? j - 1 : m - 1;
    const float c = ldg(x + k);
    const float lap = ax * (ldg(x + (long)ip * m + j) + ldg(x + (long)im * m + j) - 2.f * c) +
                      ay * (ldg(x + (long)i * m + jp) + ldg(x + (long)i * m + jm) - 2.f * c);
    const float bv = ldg(b + k);
    const float res = bv - lap;
    rr = df_add(rr, two_prod(res, res));
    bb = df_add(bb, two_prod(bv, bv));
  }
  const double s = block_sum_df(rr);
  const double sb = also_b ? block_sum_df(bb) : 0.0;
  __shared__ int am_last;
  if (threadIdx.x == 0) {
    atomicAdd(&sc->acc[0], s);
    if (also_b) atomicAdd(&sc->acc[1], sb);
    __threadfence();
    am_last = atomicAdd(&sc->red_count, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (am_last && threadIdx.x == 0) {
    __threadfence();
    sc->red_count = 0u;
    par_check_body(sc, dxdy, tol2, also_b);
  }
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
  const long N0 = (long)p.nx * p.ny;
  k_par_begin<<<1, 1, 0, st>>>(sc);
  if (p0) k_copy<<<cdiv(N0, 256), 256, 0, st>>>(p0, pout, N0);
  if (p.flow_type == AJ_FLOW_LID_DRIVEN_CAVITY) {   // b -= mean(b) (multigrid_solver.py:78-80)
    k_mean_partials<<<kMeanBlocks, 256, 0, st>>>(b0, N0, sc, at<double>(ws, L.part));
    k_sub_mean<<<cdiv(N0, 256), 256, 0, st>>>(b0, N0, sc);
  }

  auto X = [&](int l) { return l == 0 ? pout : at<float>(ws, L.X[l]); };
  auto T = [&](int l) { return l == 0 ? T0 : at<float>(ws, L.T[l]); };
  auto B = [&](int l) { return l == 0 ? b0 : at<float>(ws, L.B[l]); };
  auto M = [&](int l) -> const float* {
    if (!mac) return nullptr;
    return l == 0 ? mask : at<float>(ws, L.M[l]);
  };
  const int vk = p.flow_type == AJ_FLOW_VON_KARMAN;
  // the coarsest level's 10 sweeps from zero, ending in X(nl)
  auto coarsest = [&](const int* sk) {
    if (parity_coarsest_fused(L)) {
      const int n = L.ln[nl], m = L.lm[nl];
      const size_t csm = (size_t)coarse_band_rows(n) * m * 12;
      cudaFuncSetAttribute(k_par_coarsest, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)kBlockSmemMax);
      k_par_coarsest<<<kCoarseCtas, kCoarseThreads, csm, st>>>(B(nl), M(nl), X(nl), n, m, ax, ay,
                                                               den, sk);
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
  };
  if (p.flow_type == AJ_FLOW_TAYLOR_GREEN) {
    // unfused V-cycle (the wrapped residual needs the other side of the domain):
    // every level's iterate lives in X(l), T(l) is the sweeps' other buffer
    for (int cyc = 0; cyc < p.v_cycles; ++cyc) {
      const int* sk = cyc == 0 ? nullptr : skip;
      auto sweeps = [&](int l, const float* first_in) {
        ParJac a{};
        a.b = B(l);
        a.mask = M(l);
        a.skip = sk;
        a.n = L.ln[l];
        a.m = L.lm[l];
        a.ax = ax;
        a.ay = ay;
        a.den = den;
        dim3 g(cdiv(a.m, 32), cdiv(a.n, 8));
        a.pin = first_in;
        a.pout = T(l);
        k_par_jacobi<<<g, blk, 0, st>>>(a);
        a.pin = T(l);
        a.pout = X(l);
        k_par_jacobi<<<g, blk, 0, st>>>(a);
      };
      for (int l = 0; l < nl; ++l) {
        sweeps(l, (l == 0 && !(cyc == 0 && !p0)) ? X(0) : nullptr);
        dim3 g(cdiv(L.lm[l + 1], 32), cdiv(L.ln[l + 1], 8));
        k_tg_resid_restrict<<<g, blk, 0, st>>>(X(l), B(l), B(l + 1), L.ln[l], L.lm[l], ax, ay, sk);
      }
      coarsest(sk);
      for (int l = nl - 1; l >= 0; --l) {
        dim3 g(cdiv(L.lm[l], 32), cdiv(L.ln[l], 8));
        k_tg_prolong_add<<<g, blk, 0, st>>>(X(l), X(l + 1), L.ln[l], L.lm[l], sk);
        sweeps(l, X(l));
      }
      k_tg_norm<<<kMeanBlocks, 256, 0, st>>>(X(0), B(0), p.nx, p.ny, ax, ay, sc, p.dx * p.dy,
                                             tol * tol, cyc == 0, sk);
    }
    return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
  }
  auto tile_grid = [&](int l) {
    return l == 0 ? dim3(cdiv(L.lm[l], 64), cdiv(L.ln[l], 16)) : dim3(cdiv(L.lm[l], 32), cdiv(L.ln[l], 8));
  };
  for (int cyc = 0; cyc < p.v_cycles; ++cyc) {
    const int* sk = cyc == 0 ? nullptr : skip;   // the first cycle always runs
    // down the V: levels 0..nl-1; each level's pre-smoothed state goes to T,
    // its restricted residual to the next level's b
    for (int l = 0; l < nl; ++l) {
      ParTile a{};
      a.xin = (l == 0 && !(cyc == 0 && !p0)) ? X(0) : nullptr;
      a.b = B(l);
      a.mask = M(l);
      a.xout = T(l);
      a.bc = B(l + 1);
      a.skip = sk;
      a.n = L.ln[l];
      a.m = L.lm[l];
      a.nc = L.ln[l + 1];
      a.mc = L.lm[l + 1];
      a.zero_last = vk;
      a.mac_outlet = mac && vk;
      a.ax = ax;
      a.ay = ay;
      a.den = den;
      if (l == 0) k_par_down<16, 64><<<tile_grid(l), kPtThreads, 0, st>>>(a);
      else k_par_down<8, 32><<<tile_grid(l), kPtThreads, 0, st>>>(a);
    }
    // coarsest: 10 sweeps from zero, ending in X
    coarsest(sk);
    // up the V: T + P(coarser X), two post-sweeps, into X; level 0 also
    // forms the residual norm and its last block runs the early-exit test
    // (multigrid_solver.py:222-232)
    for (int l = nl - 1; l >= 0; --l) {
      ParTile a{};
      a.xin = T(l);
      a.xc = X(l + 1);
      a.b = B(l);
      a.mask = M(l);
      a.xout = X(l);
      a.sc = sc;
      a.skip = sk;
      a.n = L.ln[l];
      a.m = L.lm[l];
      a.nc = L.ln[l + 1];
      a.mc = L.lm[l + 1];
      a.zero_last = vk;
      a.mac_outlet = mac && vk;
      a.also_b = cyc == 0;
      a.ax = ax;
      a.ay = ay;
      a.den = den;
      a.dxdy = p.dx * p.dy;
      a.tol2 = tol * tol;
      if (l == 0) k_par_up<16, 64, true><<<tile_grid(l), kPtThreads, 0, st>>>(a);
      else k_par_up<8, 32, false><<<tile_grid(l), kPtThreads, 0, st>>>(a);
    }
  }
  if (p.flow_type == AJ_FLOW_LID_DRIVEN_CAVITY) {   // p -= p[nx/2, ny/2]
    k_store_center<<<1, 1, 0, st>>>(pout, (long)(p.nx / 2) * p.ny + p.ny / 2, sc);
    k_sub_center<<<cdiv(N0, 256), 256, 0, st>>>(pout, N0, sc);
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
  } else if (p.mg_mode == AJ_MG_CONVERGE) {
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
