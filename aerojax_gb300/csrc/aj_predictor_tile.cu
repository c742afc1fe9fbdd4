// Fused MAC predictor: the three SSP-RK3 stages of rk_step_unified_mac
// (advection_schemes/rk3_mac.py:220-504, blended upwind advection, Laplacian
// diffusion with the face eddy viscosity, implicit Brinkman), the hard mask and
// the boundary rows of the last stage, and the pressure right-hand side
// b = mask * div(u*)/dt (solver/operators_mac.py:73-80,
// pressure_solvers/multigrid_solver_mac.py:78; outlet row 0,
// multigrid_solver.py:75-77) in ONE kernel.
//
// Each block owns a 32 x 32-cell tile.  Its inputs (u, v, the mask, the
// eddy viscosity) are staged once into shared memory with a halo of three
// faces - one per stage - u, the mask and the viscosity by TMA tensor copies
// (cp.async.bulk.tensor, a 40 x 39 box whose first column is rounded down to
// the 16-byte boundary), v (its rows of ny+1 floats are not 16-byte strided)
// by coalesced loads.  Stage 1 is evaluated on the tile plus two faces, stage
// 2 plus one, stage 3 on the tile plus the +x/+y faces the divergence needs;
// every stage reads the previous one from shared memory.  Against three stage
// launches and the divergence kernel, u and v are read once and u*, v* and b
// written once; the price is ~1.2x stage evaluations on the halo.
//
// The stencil formulas and their operation order are those of k_rk_mac
// (aj_predictor.cu), so every path gives the same values (bit for bit on the
// GPU).  They cover the MAC grid, RK3, upwind advection, no hyperviscosity,
// the von Karman flow, and are opt-in: AEROJAX_TILE_PREDICTOR=1 selects the
// fused kernel, =2 the per-stage tile kernels below.  Both measured slower
// than the k_rk_mac stage kernels on the 2048x512 step (+23 and +37 us): the
// stencils are issue-bound, the global-memory kernels get their neighbour
// re-reads from L1, and the tiles add a staging phase, a barrier per stage
// and (fused) 1.2x halo evaluations and 1.7 waves of large blocks.
#include "aj_internal.cuh"
#include <cuda.h>
#include <cudaTypedefs.h>
#include <stdlib.h>
#include <mutex>

namespace aj {

namespace {

constexpr int FTI = 32, FTJ = 32;        // tile cells
constexpr int FH = 3;                    // halo faces (one per stage)
constexpr int FJ0 = 4;                   // column halo rounded up to 16 bytes
constexpr int FSI = FTI + 2 * FH + 1;    // 39 rows: faces i0-3 .. i0+35
constexpr int FSJ = 40;                  // 40 columns: j0-4 .. j0+35
constexpr int FNP = 1568;                // floats per array (FSI*FSJ = 1560, padded to 128 B)
constexpr int F_THREADS = 256;
constexpr int F_ARRAYS = 6;
constexpr size_t F_SMEM = (size_t)F_ARRAYS * FNP * sizeof(float);
static_assert(FSI * FSJ <= FNP && (FNP * 4) % 128 == 0, "shared-memory arrays must stay 128-byte aligned");
static_assert(FJ0 >= FH && FSJ >= FJ0 + FTJ + FH + 1, "the box must cover the halo");
constexpr unsigned F_TMA_BOX_BYTES = FSI * FSJ * 4;
// measured on the 2048x512 NACA step (GB300, graph-launched): the k_rk_mac
// stage kernels 0.323 ms per extrapolated step, the fused tile kernel 0.346,
// the per-stage tile kernels 0.360 - both tiled paths are opt-in
constexpr int kTileDefault = 0;

struct FArgs {
  const float* u;      // u (nx+1, ny): the RK combinations' x0 (read from L1/L2)
  const float* v;      // v (nx, ny+1), loaded with plain loads; also x0
  const float* vin;    // per-stage kernels: the stage input's v
  float *uo, *vo, *b;  // u*, v*, pressure rhs (nullable)
  DevScalars* sc;
  int nx, ny, slip, has_nsg, outlet;
  float idx, idy, idx2, idy2, nu, inv_eta, U;
};

struct FCtx {
  int nx, ny, bi, bj, slip;
  float idx, idy, idx2, idy2, nu, inv_eta, U;
  const float* M;
  const float* S;      // null: no eddy viscosity
  const float* gu;     // step input u, v in global memory (the stages' x0)
  const float* gv;
  __device__ __forceinline__ int at(int i, int j) const { return (i - bi) * FSJ + (j - bj); }
  __device__ __forceinline__ float u0(int i, int j) const { return ldg(gu + (long)i * ny + j); }
  __device__ __forceinline__ float v0(int i, int j) const {
    return ldg(gv + (long)i * (ny + 1) + j);
  }
};

// ------------------------------------------------------------ TMA / mbarrier
__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait on phase 0 of the barrier: true when the copies landed
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar) {
  for (int it = 0; it < (1 << 20); ++it)
    if (mbar_try_wait(bar, 0)) return true;
  return false;
}
// 2-D tensor copy of one box into shared memory, completing on `bar`;
// x = column (innermost, a multiple of 4 floats), y = row
__device__ __forceinline__ void tma_load_2d(float* dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];\n" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// ------------------------------------------------------------ stencils
// working copies of the stage input (rk3_mac.py:292-330, von Karman)
__device__ __forceinline__ float f_uw(const FCtx& c, const float* Us, int i, int j) {
  const int nx = c.nx, ny = c.ny;
  if (!c.slip && (j == 0 || j == ny - 1)) return 0.f;
  if (i == 0) return c.U;
  const int ii = i == nx ? nx - 1 : i;
  const int jj = c.slip ? (j == 0 ? 1 : (j == ny - 1 ? ny - 2 : j)) : j;
  return Us[c.at(ii, jj)];
}
__device__ __forceinline__ float f_vw(const FCtx& c, const float* Vs, int i, int j) {
  if (i == 0 || j == 0 || j == c.ny) return 0.f;
  const int ii = i == c.nx - 1 ? c.nx - 2 : i;
  return Vs[c.at(ii, j)];
}
// face Laplacian, slip (edge) or no-slip (antisymmetric wall) ghosts
template <int COMP>
__device__ __forceinline__ float f_lap(const FCtx& c, const float* F, int i, int j) {
  const int n = COMP == 0 ? c.nx + 1 : c.nx;
  const int m = COMP == 0 ? c.ny : c.ny + 1;
  const float cc = F[c.at(i, j)];
  float xp, xm, yp, ym;
  if (c.slip) {
    xp = F[c.at(clampi(i + 1, n), j)];
    xm = F[c.at(clampi(i - 1, n), j)];
    yp = F[c.at(i, clampi(j + 1, m))];
    ym = F[c.at(i, clampi(j - 1, m))];
  } else if (COMP == 0) {
    xp = F[c.at(clampi(i + 1, n), j)];
    xm = F[c.at(clampi(i - 1, n), j)];
    yp = j + 1 < m ? F[c.at(i, j + 1)] : -cc;
    ym = j - 1 >= 0 ? F[c.at(i, j - 1)] : -cc;
  } else {
    xp = i + 1 < n ? F[c.at(i + 1, j)] : -cc;
    xm = i - 1 >= 0 ? F[c.at(i - 1, j)] : -cc;
    yp = F[c.at(i, clampi(j + 1, m))];
    ym = F[c.at(i, clampi(j - 1, m))];
  }
  return (xp + xm - 2.f * cc) * c.idx2 + (yp + ym - 2.f * cc) * c.idy2;
}
__device__ __forceinline__ float f_xface(const FCtx& c, const float* C, int i, int j) {
  return 0.5f * (C[c.at(clampi(i, c.nx), j)] + C[c.at(clampi(i - 1, c.nx), j)]);
}
__device__ __forceinline__ float f_yface(const FCtx& c, const float* C, int i, int j) {
  return 0.5f * (C[c.at(i, clampi(j, c.ny))] + C[c.at(i, clampi(j - 1, c.ny))]);
}

// RK3 stage update (rk3_mac.py:465-486) with the hard mask on the last stage
template <int STAGE>
__device__ __forceinline__ float f_finish(const FCtx& c, float x0, float r, float chi, float dt) {
  const float den = 1.f + dt * chi * c.inv_eta;
  if (STAGE == 1) return brinkman_div(x0 + dt * r, den);
  const float xs = x0 + dt * r;
  if (STAGE == 2) return brinkman_div(0.75f * x0 + 0.25f * xs, den);
  const float out = brinkman_div((1.f / 3.f) * x0 + (2.f / 3.f) * xs, den);
  return chi < 0.5f ? out : 0.f;
}

// general u face (any position of the domain)
template <int STAGE>
__device__ float f_stage_u(const FCtx& c, const float* Us, const float* Vs, int i, int j,
                           float dt) {
  const int nx = c.nx, ny = c.ny;
  const float uw = f_uw(c, Us, i, j);
  auto vcen = [&](int ci) {
    ci = clampi(ci, nx);
    return 0.5f * (f_vw(c, Vs, ci, j + 1) + f_vw(c, Vs, ci, j));
  };
  const float v_at_u = 0.5f * (vcen(i) + vcen(i - 1));
  const float uxm = f_uw(c, Us, i > 0 ? i - 1 : 0, j);
  const float uxp = f_uw(c, Us, i < nx ? i + 1 : nx, j);
  const float back = (uw - uxm) * c.idx, fwd = (uxp - uw) * c.idx;
  const float al = upwind_weight(uw);
  const float adv_x = uw * (al * back + (1.f - al) * fwd);
  float du_dy;
  if (j == 0) du_dy = (f_uw(c, Us, i, 1) - uw) * c.idy;
  else if (j == ny - 1) du_dy = (uw - f_uw(c, Us, i, ny - 2)) * c.idy;
  else du_dy = (f_uw(c, Us, i, j + 1) - f_uw(c, Us, i, j - 1)) * (0.5f * c.idy);
  const float adv = (adv_x + v_at_u * du_dy) * f_xface(c, c.M, i, j);
  const float lap = f_lap<0>(c, Us, i, j);
  const float nut = c.S ? c.nu + f_xface(c, c.S, i, j) : c.nu;
  const float r = -adv + nut * lap;
  const float chi = 0.5f * ((1.f - c.M[c.at(clampi(i, nx), j)]) +
                            (1.f - c.M[c.at(clampi(i - 1, nx), j)]));
  return f_finish<STAGE>(c, c.u0(i, j), r, chi, dt);
}

// general v face
template <int STAGE>
__device__ float f_stage_v(const FCtx& c, const float* Us, const float* Vs, int i, int j,
                           float dt) {
  const int nx = c.nx, ny = c.ny;
  const float vw = f_vw(c, Vs, i, j);
  auto ucen = [&](int cj) {
    cj = clampi(cj, ny);
    return 0.5f * (f_uw(c, Us, i + 1, cj) + f_uw(c, Us, i, cj));
  };
  const float u_at_v = 0.5f * (ucen(j) + ucen(j - 1));
  const float vym = f_vw(c, Vs, i, j > 0 ? j - 1 : 0);
  const float vyp = f_vw(c, Vs, i, j < ny ? j + 1 : ny);
  const float back = (vw - vym) * c.idy, fwd = (vyp - vw) * c.idy;
  const float al = upwind_weight(vw);
  const float adv_y = vw * (al * back + (1.f - al) * fwd);
  float dv_dx;
  if (i == 0) dv_dx = (f_vw(c, Vs, 1, j) - vw) * c.idx;
  else if (i == nx - 1) dv_dx = (vw - f_vw(c, Vs, nx - 2, j)) * c.idx;
  else dv_dx = (f_vw(c, Vs, i + 1, j) - f_vw(c, Vs, i - 1, j)) * (0.5f * c.idx);
  const float adv = (u_at_v * dv_dx + adv_y) * f_yface(c, c.M, i, j);
  const float lap = f_lap<1>(c, Vs, i, j);
  const float nut = c.S ? c.nu + f_yface(c, c.S, i, j) : c.nu;
  const float r = -adv + nut * lap;
  const float chi = 0.5f * ((1.f - c.M[c.at(i, clampi(j, ny))]) +
                            (1.f - c.M[c.at(i, clampi(j - 1, ny))]));
  return f_finish<STAGE>(c, c.v0(i, j), r, chi, dt);
}

// interior u face of the slip-wall channel: every neighbour is a plain value
template <int STAGE>
__device__ __forceinline__ float f_stage_u_int(const FCtx& c, const float* Us, const float* Vs,
                                               int i, int j, int k, float dt) {
  const float* u = Us + k;
  const float uw = u[0], uxm = u[-FSJ], uxp = u[FSJ], uym = u[-1], uyp = u[1];
  const float* v = Vs + k;
  const float vc_i = 0.5f * (v[1] + v[0]);
  const float vc_m = 0.5f * (v[1 - FSJ] + v[-FSJ]);
  const float v_at_u = 0.5f * (vc_i + vc_m);
  const float back = (uw - uxm) * c.idx, fwd = (uxp - uw) * c.idx;
  const float al = upwind_weight(uw);
  const float adv_x = uw * (al * back + (1.f - al) * fwd);
  const float du_dy = (uyp - uym) * (0.5f * c.idy);
  const float m_i = c.M[k], m_im = c.M[k - FSJ];
  const float adv = (adv_x + v_at_u * du_dy) * (0.5f * (m_i + m_im));
  const float lap = (uxp + uxm - 2.f * uw) * c.idx2 + (uyp + uym - 2.f * uw) * c.idy2;
  const float nut = c.S ? c.nu + 0.5f * (c.S[k] + c.S[k - FSJ]) : c.nu;
  const float r = -adv + nut * lap;
  const float chi = 0.5f * ((1.f - m_i) + (1.f - m_im));
  return f_finish<STAGE>(c, c.u0(i, j), r, chi, dt);
}

template <int STAGE>
__device__ __forceinline__ float f_stage_v_int(const FCtx& c, const float* Us, const float* Vs,
                                               int i, int j, int k, float dt) {
  const float* v = Vs + k;
  const float vw = v[0], vym = v[-1], vyp = v[1], vxm = v[-FSJ], vxp = v[FSJ];
  const float* u = Us + k;
  const float uc_j = 0.5f * (u[FSJ] + u[0]);
  const float uc_m = 0.5f * (u[FSJ - 1] + u[-1]);
  const float u_at_v = 0.5f * (uc_j + uc_m);
  const float back = (vw - vym) * c.idy, fwd = (vyp - vw) * c.idy;
  const float al = upwind_weight(vw);
  const float adv_y = vw * (al * back + (1.f - al) * fwd);
  const float dv_dx = (vxp - vxm) * (0.5f * c.idx);
  const float m_j = c.M[k], m_jm = c.M[k - 1];
  const float adv = (u_at_v * dv_dx + adv_y) * (0.5f * (m_j + m_jm));
  const float lap = (vxp + vxm - 2.f * vw) * c.idx2 + (vyp + vym - 2.f * vw) * c.idy2;
  const float nut = c.S ? c.nu + 0.5f * (c.S[k] + c.S[k - 1]) : c.nu;
  const float r = -adv + nut * lap;
  const float chi = 0.5f * ((1.f - m_j) + (1.f - m_jm));
  return f_finish<STAGE>(c, c.v0(i, j), r, chi, dt);
}

// One stage over the box of faces [ib, ib+BH) x [jb, jb+BW): reads the stage
// input (Us, Vs), writes Ou, Ov.  INTERIOR: the whole box lies in the
// slip-wall channel's interior (no boundary logic).
template <int STAGE, int BH, int BW, bool INTERIOR>
__device__ __forceinline__ void f_stage(const FCtx& c, bool fast_flow, const float* Us,
                                        const float* Vs, float* Ou, float* Ov, int ib, int jb,
                                        float dt) {
  const int nx = c.nx, ny = c.ny;
  for (int t = threadIdx.x; t < BH * BW; t += F_THREADS) {
    const int a = t / BW;
    const int i = ib + a, j = jb + (t - a * BW);
    const int k = c.at(i, j);
    if (INTERIOR || (fast_flow && i >= 2 && i <= nx - 3 && j >= 2 && j <= ny - 3)) {
      const float uo = f_stage_u_int<STAGE>(c, Us, Vs, i, j, k, dt);
      const float vo = f_stage_v_int<STAGE>(c, Us, Vs, i, j, k, dt);
      Ou[k] = uo;
      Ov[k] = vo;
      continue;
    }
    if (i >= 0 && i <= nx && j >= 0 && j < ny) {
      Ou[k] = (fast_flow && i >= 2 && i <= nx - 2 && j >= 2 && j <= ny - 3)
                  ? f_stage_u_int<STAGE>(c, Us, Vs, i, j, k, dt)
                  : f_stage_u<STAGE>(c, Us, Vs, i, j, dt);
    }
    if (i >= 0 && i < nx && j >= 0 && j <= ny) {
      Ov[k] = (fast_flow && i >= 2 && i <= nx - 3 && j >= 2 && j <= ny - 2)
                  ? f_stage_v_int<STAGE>(c, Us, Vs, i, j, k, dt)
                  : f_stage_v<STAGE>(c, Us, Vs, i, j, dt);
    }
  }
}

// The three stages.  Buffers: U0/V0 hold the step input (stage 1 reads it)
// and then stage 2's values; A holds stage 1's and then stage 3's.  Every
// stage's x0 comes from the input in global memory.
template <bool INTERIOR>
__device__ __forceinline__ void f_stages(const FCtx& c, bool fast_flow, float* sm, int i0, int j0,
                                         float dt) {
  float *U0 = sm, *V0 = sm + FNP, *Au = sm + 4 * FNP, *Av = sm + 5 * FNP;
  f_stage<1, FTI + 5, FTJ + 5, INTERIOR>(c, fast_flow, U0, V0, Au, Av, i0 - 2, j0 - 2, dt);
  __syncthreads();
  f_stage<2, FTI + 3, FTJ + 3, INTERIOR>(c, fast_flow, Au, Av, U0, V0, i0 - 1, j0 - 1, dt);
  __syncthreads();
  f_stage<3, FTI + 1, FTJ + 1, INTERIOR>(c, fast_flow, U0, V0, Au, Av, i0, j0, dt);
  __syncthreads();
}

__global__ void __launch_bounds__(F_THREADS, 5) k_pred_mac_tile(
    FArgs a, const __grid_constant__ CUtensorMap tm_u, const __grid_constant__ CUtensorMap tm_m,
    const __grid_constant__ CUtensorMap tm_s) {
  pdl_wait();
  extern __shared__ __align__(128) float sm[];
  __shared__ uint64_t bar;
  const int tid = threadIdx.x;
  const int nx = a.nx, ny = a.ny;
  const int i0 = blockIdx.y * FTI, j0 = blockIdx.x * FTJ;
  float *U0 = sm, *V0 = sm + FNP, *M = sm + 2 * FNP, *S = sm + 3 * FNP;
  float *Au = sm + 4 * FNP, *Av = sm + 5 * FNP;
  float *Bu = U0, *Bv = V0;   // the final values reuse the input buffers
  // stage the inputs: u, mask (and nu_sgs) by TMA, v by coalesced loads
  if (tid == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  }
  __syncthreads();
  if (tid == 0) {
    mbar_expect_tx(&bar, F_TMA_BOX_BYTES * (a.has_nsg ? 3u : 2u));
    tma_load_2d(U0, &tm_u, j0 - FJ0, i0 - FH, &bar);
    tma_load_2d(M, &tm_m, j0 - FJ0, i0 - FH, &bar);
    if (a.has_nsg) tma_load_2d(S, &tm_s, j0 - FJ0, i0 - FH, &bar);
  }
  for (int t = tid; t < FSI * FSJ; t += F_THREADS) {
    const int r = t / FSJ, q = t - r * FSJ;
    const int gi = i0 - FH + r, gj = j0 - FJ0 + q;
    V0[t] = ((unsigned)gi < (unsigned)nx && (unsigned)gj <= (unsigned)ny)
                ? ldg(a.v + (long)gi * (ny + 1) + gj)
                : 0.f;
  }
  const bool landed = mbar_wait_bounded(&bar);
  if (__syncthreads_or(!landed)) {
    // the copies did not complete in time: flag it, wait (bounded) once more
    // for the copies in flight, and leave the outputs untouched
    if (tid == 0) a.sc->err = AJ_ERR_TIMEOUT;
    mbar_wait_bounded(&bar);
    __syncthreads();
    return;
  }
  FCtx c;
  c.nx = nx;
  c.ny = ny;
  c.bi = i0 - FH;
  c.bj = j0 - FJ0;
  c.slip = a.slip;
  c.idx = a.idx;
  c.idy = a.idy;
  c.idx2 = a.idx2;
  c.idy2 = a.idy2;
  c.nu = a.nu;
  c.inv_eta = a.inv_eta;
  c.U = a.U;
  c.M = M;
  c.S = a.has_nsg ? S : nullptr;
  c.gu = a.u;
  c.gv = a.v;
  const float dt = a.sc->dt;
  const bool fast_flow = a.slip != 0;   // von Karman with slip walls
  // the stage-1 box spans faces i0-2 .. i0+TI+2, j0-2 .. j0+TJ+2
  const bool interior = fast_flow && i0 - 2 >= 2 && i0 + FTI + 2 <= nx - 3 && j0 - 2 >= 2 &&
                        j0 + FTJ + 2 <= ny - 3;
  if (interior) f_stages<true>(c, fast_flow, sm, i0, j0, dt);
  else f_stages<false>(c, fast_flow, sm, i0, j0, dt);
  // stage-3 values are in Au/Av on faces [i0, i0+TI] x [j0, j0+TJ]: the
  // boundary rows of the last stage (rk3_mac.py:292-330 after the hard mask),
  // into Bu/Bv, then the owned faces to global memory
  for (int t = tid; t < (FTI + 1) * (FTJ + 1); t += F_THREADS) {
    const int r = t / (FTJ + 1);
    const int i = i0 + r, j = j0 + (t - r * (FTJ + 1));
    const int k = c.at(i, j);
    if (i <= nx && j < ny) {
      float o;
      if (!a.slip && (j == 0 || j == ny - 1)) o = 0.f;
      else if (i == 0) o = a.U;
      else {
        const int ii = i == nx ? nx - 1 : i;
        const int jj = a.slip ? (j == 0 ? 1 : (j == ny - 1 ? ny - 2 : j)) : j;
        o = Au[c.at(ii, jj)];
      }
      Bu[k] = o;
      if ((i < i0 + FTI || i == nx) && j < j0 + FTJ) a.uo[(long)i * ny + j] = o;
    }
    if (i < nx && j <= ny) {
      float o;
      if (i == 0 || j == 0 || j == ny) o = 0.f;
      else o = Av[c.at(i == nx - 1 ? nx - 2 : i, j)];
      Bv[k] = o;
      if (i < i0 + FTI && (j < j0 + FTJ || j == ny)) a.vo[(long)i * (ny + 1) + j] = o;
    }
  }
  if (!a.b) return;
  __syncthreads();
  // b = mask * div(u*, v*) / dt, 0 on the outlet row (k_rhs, aj_project.cu)
  for (int t = tid; t < FTI * FTJ; t += F_THREADS) {
    const int r = t / FTJ;
    const int i = i0 + r, j = j0 + (t - r * FTJ);
    if (i >= nx || j >= ny) continue;
    const int k = c.at(i, j);
    const float du = (Bu[k + FSJ] - Bu[k]) * a.idx;
    const float dv = (Bv[k + 1] - Bv[k]) * a.idy;
    float out = ((du + dv) / dt) * M[k];
    if (a.outlet && i == nx - 1) out = 0.f;
    a.b[(long)i * ny + j] = out;
  }
}

// ------------------------------------------------------------ per-stage tiles
// One RK3 stage per launch on the same 32 x 32 tiles with a one-face halo:
// the stage input's u, the mask and the viscosity arrive by TMA (a 40 x 35
// box), v by coalesced loads; every stencil then reads shared memory.  The
// tile computes faces [i0, i0+32] x [j0, j0+32] (the +1 row and column only
// serve the last stage's divergence) and stores the faces it owns; the last
// stage also applies the boundary rows and forms the pressure rhs.
constexpr int SSI = FTI + 3;                // 35 rows: faces i0-1 .. i0+33
constexpr int SNP = 1408;                   // floats per array (35*40 = 1400, padded to 128 B)
constexpr size_t S_SMEM = (size_t)6 * SNP * sizeof(float);
constexpr unsigned S_TMA_BOX_BYTES = SSI * FSJ * 4;
static_assert(SSI * FSJ <= SNP && (SNP * 4) % 128 == 0, "per-stage arrays must stay aligned");

template <int STAGE>
__global__ void __launch_bounds__(F_THREADS, 5) k_pred_mac_stage(
    FArgs a, const __grid_constant__ CUtensorMap tm_u, const __grid_constant__ CUtensorMap tm_m,
    const __grid_constant__ CUtensorMap tm_s) {
  pdl_wait();
  extern __shared__ __align__(128) float sm[];
  __shared__ uint64_t bar;
  const int tid = threadIdx.x;
  const int nx = a.nx, ny = a.ny;
  const int i0 = blockIdx.y * FTI, j0 = blockIdx.x * FTJ;
  float *Us = sm, *Vs = sm + SNP, *M = sm + 2 * SNP, *S = sm + 3 * SNP;
  float *Au = sm + 4 * SNP, *Av = sm + 5 * SNP;
  if (tid == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  }
  __syncthreads();
  if (tid == 0) {
    mbar_expect_tx(&bar, S_TMA_BOX_BYTES * (a.has_nsg ? 3u : 2u));
    tma_load_2d(Us, &tm_u, j0 - FJ0, i0 - 1, &bar);
    tma_load_2d(M, &tm_m, j0 - FJ0, i0 - 1, &bar);
    if (a.has_nsg) tma_load_2d(S, &tm_s, j0 - FJ0, i0 - 1, &bar);
  }
  for (int t = tid; t < SSI * FSJ; t += F_THREADS) {
    const int r = t / FSJ, q = t - r * FSJ;
    const int gi = i0 - 1 + r, gj = j0 - FJ0 + q;
    Vs[t] = ((unsigned)gi < (unsigned)nx && (unsigned)gj <= (unsigned)ny)
                ? ldg(a.vin + (long)gi * (ny + 1) + gj)
                : 0.f;
  }
  const bool landed = mbar_wait_bounded(&bar);
  if (__syncthreads_or(!landed)) {
    if (tid == 0) a.sc->err = AJ_ERR_TIMEOUT;
    mbar_wait_bounded(&bar);
    __syncthreads();
    return;
  }
  FCtx c;
  c.nx = nx;
  c.ny = ny;
  c.bi = i0 - 1;
  c.bj = j0 - FJ0;
  c.slip = a.slip;
  c.idx = a.idx;
  c.idy = a.idy;
  c.idx2 = a.idx2;
  c.idy2 = a.idy2;
  c.nu = a.nu;
  c.inv_eta = a.inv_eta;
  c.U = a.U;
  c.M = M;
  c.S = a.has_nsg ? S : nullptr;
  c.gu = a.u;
  c.gv = a.v;
  const float dt = a.sc->dt;
  const bool fast_flow = a.slip != 0;
  const bool interior = fast_flow && i0 >= 2 && i0 + FTI <= nx - 3 && j0 >= 2 && j0 + FTJ <= ny - 3;
  if (interior)
    f_stage<STAGE, FTI + 1, FTJ + 1, true>(c, fast_flow, Us, Vs, Au, Av, i0, j0, dt);
  else
    f_stage<STAGE, FTI + 1, FTJ + 1, false>(c, fast_flow, Us, Vs, Au, Av, i0, j0, dt);
  __syncthreads();
  if (STAGE < 3) {
    // the faces this tile owns, to the stage buffer
    for (int t = tid; t < (FTI + 1) * (FTJ + 1); t += F_THREADS) {
      const int r = t / (FTJ + 1);
      const int i = i0 + r, j = j0 + (t - r * (FTJ + 1));
      const int k = c.at(i, j);
      if (i <= nx && j < ny && (i < i0 + FTI || i == nx) && j < j0 + FTJ)
        a.uo[(long)i * ny + j] = Au[k];
      if (i < nx && j <= ny && i < i0 + FTI && (j < j0 + FTJ || j == ny))
        a.vo[(long)i * (ny + 1) + j] = Av[k];
    }
    return;
  }
  // last stage: boundary rows into Us/Vs (the stage input is consumed) and
  // the owned faces to u*, v*
  float *Bu = Us, *Bv = Vs;
  for (int t = tid; t < (FTI + 1) * (FTJ + 1); t += F_THREADS) {
    const int r = t / (FTJ + 1);
    const int i = i0 + r, j = j0 + (t - r * (FTJ + 1));
    const int k = c.at(i, j);
    if (i <= nx && j < ny) {
      float o;
      if (!a.slip && (j == 0 || j == ny - 1)) o = 0.f;
      else if (i == 0) o = a.U;
      else {
        const int ii = i == nx ? nx - 1 : i;
        const int jj = a.slip ? (j == 0 ? 1 : (j == ny - 1 ? ny - 2 : j)) : j;
        o = Au[c.at(ii, jj)];
      }
      Bu[k] = o;
      if ((i < i0 + FTI || i == nx) && j < j0 + FTJ) a.uo[(long)i * ny + j] = o;
    }
    if (i < nx && j <= ny) {
      float o;
      if (i == 0 || j == 0 || j == ny) o = 0.f;
      else o = Av[c.at(i == nx - 1 ? nx - 2 : i, j)];
      Bv[k] = o;
      if (i < i0 + FTI && (j < j0 + FTJ || j == ny)) a.vo[(long)i * (ny + 1) + j] = o;
    }
  }
  if (!a.b) return;
  __syncthreads();
  for (int t = tid; t < FTI * FTJ; t += F_THREADS) {
    const int r = t / FTJ;
    const int i = i0 + r, j = j0 + (t - r * FTJ);
    if (i >= nx || j >= ny) continue;
    const int k = c.at(i, j);
    const float du = (Bu[k + FSJ] - Bu[k]) * a.idx;
    const float dv = (Bv[k + 1] - Bv[k]) * a.idy;
    float out = ((du + dv) / dt) * M[k];
    if (a.outlet && i == nx - 1) out = 0.f;
    a.b[(long)i * ny + j] = out;
  }
}

// ------------------------------------------------------------ host side
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    cudaGetLastError();
  });
  return fn;
}

// a rows x cols float32 array (row stride cols) as a 2-D tensor with a
// box_rows x FSJ box; out-of-range box elements read as zero
bool encode_box(CUtensorMap* map, const float* base, int rows, int cols, int box_rows = FSI) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)cols * sizeof(float)};
  cuuint32_t box[2] = {FSJ, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides,
            box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// AEROJAX_TILE_PREDICTOR: 0 = the k_rk_mac stage kernels, 1 = the fused
// three-stage tile kernel, 2 = the per-stage tile kernels
int tile_predictor_mode() {
  static int v = -1;
  if (v < 0) {
    const char* e = getenv("AEROJAX_TILE_PREDICTOR");
    v = (e && e[0] >= '0' && e[0] <= '2') ? e[0] - '0' : kTileDefault;
  }
  return v;
}
bool tile_predictor_enabled() { return tile_predictor_mode() != 0; }

bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

}  // namespace

// the options the fused kernel covers; nx even and ny a multiple of 4 keep
// every boundary row's source face inside the last tile's stage-3 box and the
// rows 16-byte strided for the tensor copies
bool tile_predictor_params_ok(const AjStepParams& p) {
  return tile_predictor_enabled() && p.grid_type == AJ_GRID_MAC && p.fast_mode == 0 &&
         p.nu_hyper_ratio <= 0.0 && p.advection == AJ_ADV_UPWIND &&
         p.flow_type == AJ_FLOW_VON_KARMAN && p.nx % 2 == 0 && p.ny % 4 == 0 && p.nx >= 4 &&
         p.ny >= 4;
}

bool tile_predictor_ok(const AjStepParams& p, const float* u, const float* mask,
                       const float* nsg) {
  return tile_predictor_params_ok(p) && aligned16(u) && aligned16(mask) &&
         (!nsg || aligned16(nsg)) && encode_fn() != nullptr;
}

int launch_predictor_tile(const AjStepParams& p, void* ws, const float* u, const float* v,
                          const float* mask, const float* nsg, float* us, float* vs, float* b,
                          const float* const* stage_bufs, cudaStream_t st) {
  const int mode = tile_predictor_mode();
  const double eta = p.brinkman_eta > 1e-10 ? p.brinkman_eta : 1e-10;   // rk3_mac.py:234
  FArgs a{};
  a.u = u;
  a.v = v;
  a.vin = v;
  a.uo = us;
  a.vo = vs;
  a.b = b;
  a.sc = at<DevScalars>(ws, 0);
  a.nx = p.nx;
  a.ny = p.ny;
  a.slip = p.slip_walls;
  a.has_nsg = nsg != nullptr;
  a.outlet = p.flow_type == AJ_FLOW_VON_KARMAN;
  a.idx = (float)(1.0 / p.dx);
  a.idy = (float)(1.0 / p.dy);
  a.idx2 = (float)(1.0 / (p.dx * p.dx));
  a.idy2 = (float)(1.0 / (p.dy * p.dy));
  a.nu = (float)p.nu;
  a.inv_eta = (float)(1.0 / eta);
  a.U = (float)p.U_inf;
  dim3 grd(cdiv(p.ny, FTJ), cdiv(p.nx, FTI));
  if (mode == 1) {
    CUtensorMap tu, tm, ts;
    if (!encode_box(&tu, u, p.nx + 1, p.ny) || !encode_box(&tm, mask, p.nx, p.ny) ||
        !encode_box(&ts, nsg ? nsg : mask, p.nx, p.ny))
      return AJ_ERR_CUDA;
    static std::once_flag once;
    static cudaError_t attr_rc = cudaSuccess;
    std::call_once(once, [] {
      attr_rc = cudaFuncSetAttribute(k_pred_mac_tile, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)F_SMEM);
    });
    if (attr_rc != cudaSuccess) return AJ_ERR_CUDA;
    launch_pdl(true, k_pred_mac_tile, grd, dim3(F_THREADS), F_SMEM, st, a, tu, tm, ts);
    return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
  }
  // per-stage tiles: stage 1 u, v -> buffers A; stage 2 A -> B; stage 3 B -> u*, v*, b
  float* A_u = const_cast<float*>(stage_bufs[0]);
  float* A_v = const_cast<float*>(stage_bufs[1]);
  float* B_u = const_cast<float*>(stage_bufs[2]);
  float* B_v = const_cast<float*>(stage_bufs[3]);
  CUtensorMap tm, ts, t1, t2, t3;
  if (!encode_box(&tm, mask, p.nx, p.ny, SSI) || !encode_box(&ts, nsg ? nsg : mask, p.nx, p.ny, SSI) ||
      !encode_box(&t1, u, p.nx + 1, p.ny, SSI) || !encode_box(&t2, A_u, p.nx + 1, p.ny, SSI) ||
      !encode_box(&t3, B_u, p.nx + 1, p.ny, SSI))
    return AJ_ERR_CUDA;
  static std::once_flag once2;
  static cudaError_t attr2 = cudaSuccess;
  std::call_once(once2, [] {
    cudaError_t e1 = cudaFuncSetAttribute(k_pred_mac_stage<1>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S_SMEM);
    cudaError_t e2 = cudaFuncSetAttribute(k_pred_mac_stage<2>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S_SMEM);
    cudaError_t e3 = cudaFuncSetAttribute(k_pred_mac_stage<3>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S_SMEM);
    attr2 = e1 != cudaSuccess ? e1 : (e2 != cudaSuccess ? e2 : e3);
  });
  if (attr2 != cudaSuccess) return AJ_ERR_CUDA;
  FArgs a1 = a, a2 = a, a3 = a;
  a1.uo = A_u;
  a1.vo = A_v;
  a1.b = nullptr;
  a2.vin = A_v;
  a2.uo = B_u;
  a2.vo = B_v;
  a2.b = nullptr;
  a3.vin = B_v;
  launch_pdl(true, k_pred_mac_stage<1>, grd, dim3(F_THREADS), S_SMEM, st, a1, t1, tm, ts);
  launch_pdl(true, k_pred_mac_stage<2>, grd, dim3(F_THREADS), S_SMEM, st, a2, t2, tm, ts);
  launch_pdl(true, k_pred_mac_stage<3>, grd, dim3(F_THREADS), S_SMEM, st, a3, t3, tm, ts);
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

int tile_predictor_kernels() { return tile_predictor_mode() == 1 ? 1 : 3; }

}  // namespace aj
