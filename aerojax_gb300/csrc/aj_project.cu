// Projection: divergence of the predicted velocity -> pressure right-hand side,
// and the pressure-gradient correction with the interface projection, the
// boundary conditions and the hard mask.  Also the obstacle geometry set-up.
//
// Collocated PURE  : solver/pure_functions/step.py:182-199 and :259-397
// Collocated GUI   : solver/simulation/step_handlers.py:92-98 and :128-185
// MAC GUI          : solver/simulation/step_handlers.py:218-224 and :238-293
// Boundary conditions are fused by evaluating the corrected velocity at the
// cell each boundary copies from, so the kernel writes every cell exactly once.
#include "aj_internal.cuh"
#include <math.h>

namespace aj {

// ------------------------------------------------------------------ rhs
// writes the multigrid right-hand side b directly:
//   collocated: div = central difference on the interior, 0 on the ring
//               (solver/operators.py:81-96); PURE rhs = div*mask/dt, GUI div/dt
//   MAC:        div = face differences (solver/operators_mac.py:73-80),
//               rhs = div/dt, b = rhs*mask (multigrid_solver_mac.py:78)
//   von Karman: b[-1, :] = 0 (multigrid_solver.py:75-77)
//   Taylor-Green (collocated): the periodic central divergence
//               (solver/operators.py:75-78, step.py:192-197)
__global__ void __launch_bounds__(256) k_rhs(const float* __restrict__ us,
                                             const float* __restrict__ vs,
                                             const float* __restrict__ mask,
                                             float* __restrict__ b, int nx, int ny, float h2x,
                                             float h2y, float idx, float idy, int mac, int pure,
                                             int outlet, int periodic, const DevScalars* sc) {
  pdl_wait();
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  const float dt = sc->dt;
  long k = (long)i * ny + j;
  float out;
  if (mac) {
    out = rhs_mac_cell(us, vs, mask, i, j, nx, ny, idx, idy, dt, 0);
  } else {
    float div = 0.f;
    if (periodic) {
      const int ip = wrapi(i + 1, nx), im = wrapi(i - 1, nx);
      const int jp = wrapi(j + 1, ny), jm = wrapi(j - 1, ny);
      div = (ldg(us + (long)ip * ny + j) - ldg(us + (long)im * ny + j)) * h2x +
            (ldg(vs + (long)i * ny + jp) - ldg(vs + (long)i * ny + jm)) * h2y;
    } else if (i > 0 && i < nx - 1 && j > 0 && j < ny - 1) {
      div = (ldg(us + (long)(i + 1) * ny + j) - ldg(us + (long)(i - 1) * ny + j)) * h2x +
            (ldg(vs + (long)i * ny + j + 1) - ldg(vs + (long)i * ny + j - 1)) * h2y;
    }
    out = pure ? (div * ldg(mask + k)) / dt : div / dt;
  }
  if (outlet && i == nx - 1) out = 0.f;
  b[k] = out;
}

int launch_rhs(const AjStepParams& p, const Layout& L, void* ws, const float* us,
               const float* vs, const float* mask, float* b, cudaStream_t st) {
  dim3 blk(32, 8), grd(cdiv(p.ny, 32), cdiv(p.nx, 8));
  launch_pdl(true, k_rhs, dim3(grd), dim3(blk), 0, st, us, vs, mask, b, p.nx, p.ny,
             (float)(1.0 / (2.0 * p.dx)), (float)(1.0 / (2.0 * p.dy)), (float)(1.0 / p.dx),
             (float)(1.0 / p.dy), p.grid_type == AJ_GRID_MAC, p.variant == AJ_VARIANT_PURE,
             p.flow_type == AJ_FLOW_VON_KARMAN, p.flow_type == AJ_FLOW_TAYLOR_GREEN,
             at<DevScalars>(ws, 0));
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

// ------------------------------------------------------------------ correction
struct Corr {
  const float *us, *vs, *p, *mask;
  float *uo, *vo;
  const DevScalars* sc;
  int nx, ny, variant, flow;
  float idx, idy, h2x, h2y, thresh, U;
};

// non-periodic gradient: central interior, one-sided edges (operators.py:17-56)
__device__ __forceinline__ float gnx(const float* __restrict__ f, int a, int b, int nx, int ny,
                                     float idx, float h2x) {
  if (a == 0) return (ldg(f + (long)ny + b) - ldg(f + b)) * idx;
  if (a == nx - 1) return (ldg(f + (long)(nx - 1) * ny + b) - ldg(f + (long)(nx - 2) * ny + b)) * idx;
  return (ldg(f + (long)(a + 1) * ny + b) - ldg(f + (long)(a - 1) * ny + b)) * h2x;
}
__device__ __forceinline__ float gny(const float* __restrict__ f, int a, int b, int nx, int ny,
                                     float idy, float h2y) {
  const float* r = f + (long)a * ny;
  if (b == 0) return (ldg(r + 1) - ldg(r)) * idy;
  if (b == ny - 1) return (ldg(r + ny - 1) - ldg(r + ny - 2)) * idy;
  return (ldg(r + b + 1) - ldg(r + b - 1)) * h2y;
}

// corrected velocity at (a, b) before the boundary conditions (COMP 0 = u)
template <int COMP>
__device__ __forceinline__ float w_pure(const Corr& c, int a, int b, float dt) {
  long k = (long)a * c.ny + b;
  if (!(ldg(c.mask + k) > 0.5f)) return 0.f;                      // step.py:348-349
  float dpx = gnx(c.p, a, b, c.nx, c.ny, c.idx, c.h2x);
  float dpy = gny(c.p, a, b, c.nx, c.ny, c.idy, c.h2y);
  float dmx = gnx(c.mask, a, b, c.nx, c.ny, c.idx, c.h2x);
  float dmy = gny(c.mask, a, b, c.nx, c.ny, c.idy, c.h2y);
  float gm = sqrtf(dmx * dmx + dmy * dmy);
  if (gm > c.thresh) {                                             // step.py:313-335
    float nxv = dmx / (gm + 1e-8f), nyv = dmy / (gm + 1e-8f);
    float dn = dpx * nxv + dpy * nyv;
    dpx = dpx - dn * nxv;
    dpy = dpy - dn * nyv;
  }
  if (a == 0) dpx = 0.f;                                           // step.py:341
  return COMP == 0 ? ldg(c.us + k) - dt * dpx : ldg(c.vs + k) - dt * dpy;
}

template <int COMP>
__device__ __forceinline__ float w_gui(const Corr& c, int a, int b, float dt) {
  long k = (long)a * c.ny + b;
  if (COMP == 0) {
    float dpx = a == 0 ? 0.f : gnx(c.p, a, b, c.nx, c.ny, c.idx, c.h2x);   // :134-135
    return ldg(c.us + k) - dt * dpx;
  }
  return ldg(c.vs + k) - dt * gny(c.p, a, b, c.nx, c.ny, c.idy, c.h2y);
}

// periodic central gradient (solver/operators.py:11-38), the form both steps
// use for every flow but the von Karman channel
__device__ __forceinline__ float gpx(const float* __restrict__ f, int a, int b, int nx, int ny,
                                     float h2x) {
  return (ldg(f + (long)wrapi(a + 1, nx) * ny + b) - ldg(f + (long)wrapi(a - 1, nx) * ny + b)) *
         h2x;
}
__device__ __forceinline__ float gpy(const float* __restrict__ f, int a, int b, int ny,
                                     float h2y) {
  const float* r = f + (long)a * ny;
  return (ldg(r + wrapi(b + 1, ny)) - ldg(r + wrapi(b - 1, ny))) * h2y;
}

// corrected velocity with periodic gradients: step_pure (interface
// projection on the periodic mask gradient, step.py:259-335) or the GUI step
// (step_handlers.py:129-140), before the boundary rows
template <int COMP>
__device__ __forceinline__ float w_periodic(const Corr& c, int a, int b, float dt) {
  const long k = (long)a * c.ny + b;
  float dpx = gpx(c.p, a, b, c.nx, c.ny, c.h2x);
  float dpy = gpy(c.p, a, b, c.ny, c.h2y);
  if (c.variant == AJ_VARIANT_PURE) {
    const float dmx = gpx(c.mask, a, b, c.nx, c.ny, c.h2x);
    const float dmy = gpy(c.mask, a, b, c.ny, c.h2y);
    const float gm = sqrtf(dmx * dmx + dmy * dmy);
    if (gm > c.thresh) {
      const float nxv = dmx / (gm + 1e-8f), nyv = dmy / (gm + 1e-8f);
      const float dn = dpx * nxv + dpy * nyv;
      dpx = dpx - dn * nxv;
      dpy = dpy - dn * nyv;
    }
  }
  return COMP == 0 ? ldg(c.us + k) - dt * dpx : ldg(c.vs + k) - dt * dpy;
}

// collocated correction of the lid-driven cavity and Taylor-Green flows:
// the lid rows of step.py:378-390 (lid velocity 1) / step_handlers.py:162-171
// (lid velocity U_inf), none for Taylor-Green, then the hard mask
__device__ __forceinline__ void correct_col_other(const Corr& c, int i, int j, float dt,
                                                  float* uo, float* vo) {
  const int nx = c.nx, ny = c.ny;
  float u, v;
  if (c.flow == AJ_FLOW_LID_DRIVEN_CAVITY) {
    const bool edge = i == 0 || i == nx - 1 || j == 0;
    const float lid = c.variant == AJ_VARIANT_PURE ? 1.f : c.U;
    u = edge ? 0.f : (j == ny - 1 ? lid : w_periodic<0>(c, i, j, dt));
    v = (edge || j == ny - 1) ? 0.f : w_periodic<1>(c, i, j, dt);
  } else {
    u = w_periodic<0>(c, i, j, dt);
    v = w_periodic<1>(c, i, j, dt);
  }
  const bool m = ldg(c.mask + (long)i * ny + j) > 0.5f;
  *uo = m ? u : 0.f;
  *vo = m ? v : 0.f;
}

__global__ void __launch_bounds__(256) k_correct_col(Corr c) {
  pdl_wait();
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  const int nx = c.nx, ny = c.ny;
  if (i >= nx || j >= ny) return;
  long k = (long)i * ny + j;
  const float dt = c.sc->dt_corr;
  if (c.flow != AJ_FLOW_VON_KARMAN) {
    correct_col_other(c, i, j, dt, c.uo + k, c.vo + k);
    return;
  }
  float uo, vo;
  int ai = (i == nx - 1) ? nx - 2 : i;
  if (c.variant == AJ_VARIANT_PURE) {
    // BC of step.py:365-377, then the hard mask at (i, j) (:396-397)
    int bj = j == 0 ? 1 : (j == ny - 1 ? ny - 2 : j);
    uo = (i == 0) ? c.U : w_pure<0>(c, ai, bj, dt);
    vo = (i == 0 || j == 0 || j == ny - 1) ? 0.f : w_pure<1>(c, ai, j, dt);
  } else {
    // BC of step_handlers.py:143-161 (inlet excludes the corners, no-slip walls)
    if (j == 0 || j == ny - 1) uo = 0.f;
    else uo = (i == 0) ? c.U : w_gui<0>(c, ai, j, dt);
    vo = (i == 0 || j == 0 || j == ny - 1) ? 0.f : w_gui<1>(c, ai, j, dt);
  }
  bool m = ldg(c.mask + k) > 0.5f;                                 // step_handlers.py:182-183
  c.uo[k] = m ? uo : 0.f;
  c.vo[k] = m ? vo : 0.f;
}

// MAC GUI correction: staggered gradients (operators_mac.py:40-55; the face
// gradient on the boundary faces is 0), BC of step_handlers.py:256-274
__global__ void __launch_bounds__(256) k_correct_mac(Corr c) {
  pdl_wait();
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  const int nx = c.nx, ny = c.ny;
  const float dt = c.sc->dt_corr;
  if (c.flow != AJ_FLOW_VON_KARMAN) {
    // the same staggered gradients; the lid-driven cavity's rows
    // (step_handlers.py:265-274), none for Taylor-Green
    const bool ldc = c.flow == AJ_FLOW_LID_DRIVEN_CAVITY;
    if (i <= nx && j < ny) {
      float o;
      if (ldc && (i == 0 || i == nx || j == 0)) o = 0.f;
      else if (ldc && j == ny - 1) o = c.U;
      else {
        const float dpx = (ldg(c.p + (long)clampi(i, nx) * ny + j) -
                           ldg(c.p + (long)clampi(i - 1, nx) * ny + j)) * c.idx;
        o = ldg(c.us + (long)i * ny + j) - dt * dpx;
      }
      c.uo[(long)i * ny + j] = o;
    }
    if (i < nx && j <= ny) {
      float o;
      if (ldc && (i == 0 || i == nx - 1 || j == 0 || j == ny)) o = 0.f;
      else {
        const float dpy = (ldg(c.p + (long)i * ny + clampi(j, ny)) -
                           ldg(c.p + (long)i * ny + clampi(j - 1, ny))) * c.idy;
        o = ldg(c.vs + (long)i * (ny + 1) + j) - dt * dpy;
      }
      c.vo[(long)i * (ny + 1) + j] = o;
    }
    return;
  }
  if (i <= nx && j < ny) {
    float o;
    if (j == 0 || j == ny - 1) o = 0.f;
    else if (i == 0) o = c.U;
    else {
      int a = i == nx ? nx - 1 : i;
      float dpx = (ldg(c.p + (long)clampi(a, nx) * ny + j) - ldg(c.p + (long)clampi(a - 1, nx) * ny + j)) * c.idx;
      o = ldg(c.us + (long)a * ny + j) - dt * dpx;
    }
    c.uo[(long)i * ny + j] = o;
  }
  if (i < nx && j <= ny) {
    float o;
    if (i == 0 || j == 0 || j == ny) o = 0.f;
    else {
      int a = i == nx - 1 ? nx - 2 : i;
      float dpy = (ldg(c.p + (long)a * ny + clampi(j, ny)) - ldg(c.p + (long)a * ny + clampi(j - 1, ny))) * c.idy;
      o = ldg(c.vs + (long)a * (ny + 1) + j) - dt * dpy;
    }
    c.vo[(long)i * (ny + 1) + j] = o;
  }
}

int launch_correct(const AjStepParams& p, const Layout& L, void* ws, const float* us,
                   const float* vs, const float* pr, const float* mask, float* uo, float* vo,
                   cudaStream_t st) {
  Corr c{};
  c.us = us;
  c.vs = vs;
  c.p = pr;
  c.mask = mask;
  c.uo = uo;
  c.vo = vo;
  c.sc = at<DevScalars>(ws, 0);
  c.nx = p.nx;
  c.ny = p.ny;
  c.variant = p.variant;
  c.flow = p.flow_type;
  c.idx = (float)(1.0 / p.dx);
  c.idy = (float)(1.0 / p.dy);
  c.h2x = (float)(1.0 / (2.0 * p.dx));
  c.h2y = (float)(1.0 / (2.0 * p.dy));
  c.thresh = (float)(0.1 / p.dx);
  c.U = (float)p.U_inf;
  dim3 blk(32, 8);
  if (p.grid_type == AJ_GRID_MAC) {
    dim3 grd(cdiv(p.ny + 1, 32), cdiv(p.nx + 1, 8));
    launch_pdl(true, k_correct_mac, dim3(grd), dim3(blk), 0, st, c);
  } else {
    dim3 grd(cdiv(p.ny, 32), cdiv(p.nx, 8));
    launch_pdl(true, k_correct_col, dim3(grd), dim3(blk), 0, st, c);
  }
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

// ------------------------------------------------------------------ geometry
struct Geo {
  int kind;
  double g[8];
};

__device__ double sdf_at(const Geo& G, double X, double Y) {
  switch (G.kind) {
    case AJ_GEOM_CYLINDER:                                   // mask_generator.py:151-153
      return sqrt((X - G.g[0]) * (X - G.g[0]) + (Y - G.g[1]) * (Y - G.g[1])) - G.g[2];
    case AJ_GEOM_CYL3_ROW: {                                 // cylinder_array.py:8-42
      double r = G.g[2] / 2.0, best = 1e300;
      for (int q = 0; q < 3; ++q) {
        double cx = G.g[0] + q * G.g[3];
        double d = sqrt((X - cx) * (X - cx) + (Y - G.g[1]) * (Y - G.g[1])) - r;
        best = q == 0 ? d : fmin(best, d);
      }
      return best;
    }
    case AJ_GEOM_CYL3_TRI: {                                 // equilateral triangle, apex upstream
      double r = G.g[2] / 2.0, s = G.g[3], R = s / sqrt(3.0);
      double px[3] = {G.g[0] - R, G.g[0] + 0.5 * R, G.g[0] + 0.5 * R};
      double py[3] = {G.g[1], G.g[1] + 0.5 * s, G.g[1] - 0.5 * s};
      double best = 1e300;
      for (int q = 0; q < 3; ++q) {
        double d = sqrt((X - px[q]) * (X - px[q]) + (Y - py[q]) * (Y - py[q])) - r;
        best = q == 0 ? d : fmin(best, d);
      }
      return best;
    }
    case AJ_GEOM_NACA4: {                                    // naca_airfoils.py:109-178
      double chord = G.g[0], aoa = G.g[1] * (M_PI / 180.0), x0 = G.g[2], y0 = G.g[3];
      double m = G.g[4], pp = G.g[5], t = G.g[6];
      double Xl = X - x0, Yl = Y - y0;
      double Xr = Xl * cos(aoa) - Yl * sin(aoa);
      double Yr = Xl * sin(aoa) + Yl * cos(aoa);
      double xn = Xr / chord, yn = Yr / chord;
      bool inc = xn >= 0.0 && xn <= 1.0;
      double xs = fmin(fmax(xn, 0.0), 1.0);
      double yt = 5.0 * t * (0.2969 * sqrt(fabs(xs)) - 0.1260 * xs - 0.3516 * xs * xs +
                             0.2843 * xs * xs * xs - 0.1015 * xs * xs * xs * xs);
      double yc, dyc;
      if (xn <= pp) {
        yc = m / (pp * pp) * (2.0 * pp * xn - xn * xn);
        dyc = 2.0 * m / (pp * pp) * (pp - xn);
      } else {
        yc = m / ((1.0 - pp) * (1.0 - pp)) * ((1.0 - 2.0 * pp) + 2.0 * pp * xn - xn * xn);
        dyc = 2.0 * m / ((1.0 - pp) * (1.0 - pp)) * (pp - xn);
      }
      double th = atan(dyc);
      double yu = yc + yt * cos(th), yl = yc - yt * cos(th);
      double ds = fmin(fabs(yn - yu) * chord, fabs(yn - yl) * chord);
      double dle = sqrt(Xr * Xr + Yr * Yr);
      double dte = sqrt((Xr - chord) * (Xr - chord) + Yr * Yr);
      double dist = inc ? ds : fmin(dle, dte);
      bool inside = inc && (yn >= yl - 0.01) && (yn <= yu + 0.01);
      return inside ? -dist : dist;
    }
    default:
      return 1e30;
  }
}

__global__ void k_geometry(Geo G, int nx, int ny, double sx, double sy, double inv_eps,
                           float* __restrict__ mask, float* __restrict__ sdf) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  double X = i * sx, Y = j * sy;                             // linspace(0, l, n)
  double s = sdf_at(G, X, Y);
  double x = -s * inv_eps;                                   // mask = 1 - sigmoid(-sdf/eps)
  double chi = x >= 0.0 ? 1.0 / (1.0 + exp(-x)) : exp(x) / (1.0 + exp(x));
  long k = (long)i * ny + j;
  if (mask) mask[k] = (float)(1.0 - chi);
  if (sdf) sdf[k] = (float)s;
}

}  // namespace aj

extern "C" int32_t aj_geometry(int32_t nx, int32_t ny, double lx, double ly, int32_t kind,
                               const double* geo_host, double eps, float* mask, float* sdf,
                               void* stream) {
  using namespace aj;
  if (nx < 2 || ny < 2 || eps <= 0.0) return AJ_ERR_PARAM;
  Geo G{};
  G.kind = kind;
  int ng = kind == AJ_GEOM_NACA4 ? 7 : (kind == AJ_GEOM_CYLINDER ? 3 : 4);
  if (kind < AJ_GEOM_CYLINDER || kind > AJ_GEOM_CYL3_TRI || !geo_host) return AJ_ERR_PARAM;
  for (int q = 0; q < ng; ++q) G.g[q] = geo_host[q];
  dim3 blk(32, 8), grd(cdiv(ny, 32), cdiv(nx, 8));
  k_geometry<<<grd, blk, 0, (cudaStream_t)stream>>>(G, nx, ny, lx / (nx - 1), ly / (ny - 1),
                                                     1.0 / eps, mask, sdf);
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

// ---------------------------------------------------------------- diagnostics
// The post-step fields of step_for_visualization
// (solver/simulation/visualization_step.py:224-256) into headless device
// buffers: vorticity and divergence (solver/operators.py:75-108,
// solver/operators_mac.py:58-115; non-periodic for the von Karman channel,
// periodic otherwise) and the speed of the cell-centred velocity.  On the MAC
// grid the reference's vorticity differentiates the centred u in x and the
// centred v in y (its names say dv/dx and du/dy); that is reproduced.
namespace aj {

// Dye (passive scalar) step at cell (i, j), the reference's four variants
// (operators.py:111-150, operators_mac.py:161-215): c + dt (-(uc dc/dx +
// vc dc/dy) + kappa lap c), clipped to [0, 1]; (uc, vc) is the cell's velocity.
struct Dye {
  const float* c;
  float* c_out;
  float dt, kappa, dx2, dy2;   // dx2, dy2: dx*dx and dy*dy rounded once to FP32
};
template <bool MAC, bool PER>
__device__ __forceinline__ float dye_at(const Dye& d, int i, int j, int nx, int ny, float h2x,
                                        float h2y, float dx, float uc, float vc) {
  const float* c = d.c;
  const float cc = c[(long)i * ny + j];
  // only the neighbours each variant reads: edge-padded (clamped) x and y for
  // MAC; wrapped for the collocated periodic one; clamped x (which also gives
  // the one-sided inlet/outlet differences) and wrapped y for the collocated
  // non-periodic one; MAC periodic differences wrap but its Laplacian clamps
  const int ipx = PER && !MAC ? wrapi(i + 1, nx) : clampi(i + 1, nx);
  const int imx = PER && !MAC ? wrapi(i - 1, nx) : clampi(i - 1, nx);
  const int jpy = (MAC && !PER) ? clampi(j + 1, ny) : wrapi(j + 1, ny);
  const int jmy = (MAC && !PER) ? clampi(j - 1, ny) : wrapi(j - 1, ny);
  const float xp = c[(long)ipx * ny + j], xm = c[(long)imx * ny + j];
  const float yp = c[(long)i * ny + jpy], ym = c[(long)i * ny + jmy];
  float dcx, dcy, lap;
  if (MAC && PER) {
    // periodic central differences, edge-padded Laplacian (laplacian_staggered)
    const float xwp = c[(long)wrapi(i + 1, nx) * ny + j], xwm = c[(long)wrapi(i - 1, nx) * ny + j];
    const float yep = c[(long)i * ny + clampi(j + 1, ny)], yem = c[(long)i * ny + clampi(j - 1, ny)];
    dcx = (xwp - xwm) / h2x;
    dcy = (yp - ym) / h2y;
    lap = (xp + xm - 2.f * cc) / d.dx2 + (yep + yem - 2.f * cc) / d.dy2;
  } else if (MAC) {
    dcx = (xp - xm) / h2x;
    dcy = (yp - ym) / h2y;
    lap = (xp + xm - 2.f * cc) / d.dx2 + (yp + ym - 2.f * cc) / d.dy2;
  } else if (PER) {
    dcx = (xp - xm) / h2x;
    dcy = (yp - ym) / h2y;
    lap = ((((xm + xp) + ym) + yp) - 4.f * cc) / d.dx2;   // dx^2 for all five points
  } else {
    if (i == 0) dcx = (xp - cc) / dx;   // one-sided at the inlet and outlet rows
    else if (i == nx - 1) dcx = (cc - xm) / dx;
    else dcx = (xp - xm) / h2x;
    dcy = (yp - ym) / h2y;   // periodic in y
    lap = ((xp - 2.f * cc) + xm) / d.dx2 + ((ym + yp) - 2.f * cc) / d.dy2;
  }
  const float adv = uc * dcx + vc * dcy;
  const float cn = cc + d.dt * (-adv + d.kappa * lap);
  return fminf(fmaxf(cn, 0.f), 1.f);
}

// The post-step epilogue, one read of the new velocity: vorticity,
// divergence, speed (step_for_visualization, visualization_step.py:224-256)
// and the dye step, each optional (null output: not computed).
template <bool MAC, bool PER>
__global__ void k_diagnostics(const float* __restrict__ u, const float* __restrict__ v, int nx,
                              int ny, float dx, float dy, float* __restrict__ vort,
                              float* __restrict__ div, float* __restrict__ speed, Dye dye) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  const long k = (long)i * ny + j;
  const float h2x = 2.f * dx, h2y = 2.f * dy;
  if (MAC) {
    const int nyv = ny + 1;
    auto uc = [&](int a, int b) {
      return __fmul_rn(0.5f, __fadd_rn(u[(long)(a + 1) * ny + b], u[(long)a * ny + b]));
    };
    auto vc = [&](int a, int b) {
      return __fmul_rn(0.5f, __fadd_rn(v[(long)a * nyv + b + 1], v[(long)a * nyv + b]));
    };
    int ip, im, jp, jm;
    if (PER) {
      ip = wrapi(i + 1, nx), im = wrapi(i - 1, nx), jp = wrapi(j + 1, ny), jm = wrapi(j - 1, ny);
    } else {
      ip = clampi(i + 1, nx), im = clampi(i - 1, nx), jp = clampi(j + 1, ny), jm = clampi(j - 1, ny);
    }
    if (vort) vort[k] = (uc(ip, j) - uc(im, j)) / h2x - (vc(i, jp) - vc(i, jm)) / h2y;
    if (div)
      div[k] = (u[(long)(i + 1) * ny + j] - u[(long)i * ny + j]) / dx +
               (v[(long)i * nyv + j + 1] - v[(long)i * nyv + j]) / dy;
    if (speed || dye.c) {
      const float a = uc(i, j), b = vc(i, j);
      if (speed) speed[k] = sqrtf(a * a + b * b);
      if (dye.c) dye.c_out[k] = dye_at<true, PER>(dye, i, j, nx, ny, h2x, h2y, dx, a, b);
    }
  } else {
    if (vort) {
      float gx, gy;
      if (PER) {
        gx = (v[(long)wrapi(i + 1, nx) * ny + j] - v[(long)wrapi(i - 1, nx) * ny + j]) / h2x;
        gy = (u[(long)i * ny + wrapi(j + 1, ny)] - u[(long)i * ny + wrapi(j - 1, ny)]) / h2y;
      } else {
        if (i == 0) gx = (v[k + ny] - v[k]) / dx;
        else if (i == nx - 1) gx = (v[k] - v[k - ny]) / dx;
        else gx = (v[k + ny] - v[k - ny]) / h2x;
        if (j == 0) gy = (u[k + 1] - u[k]) / dy;
        else if (j == ny - 1) gy = (u[k] - u[k - 1]) / dy;
        else gy = (u[k + 1] - u[k - 1]) / h2y;
      }
      vort[k] = gx - gy;
    }
    if (div) {
      float d = 0.f;
      if (PER) {
        d = (u[(long)wrapi(i + 1, nx) * ny + j] - u[(long)wrapi(i - 1, nx) * ny + j]) / h2x +
            (v[(long)i * ny + wrapi(j + 1, ny)] - v[(long)i * ny + wrapi(j - 1, ny)]) / h2y;
      } else if (i > 0 && i < nx - 1 && j > 0 && j < ny - 1) {
        d = (u[k + ny] - u[k - ny]) / h2x + (v[k + 1] - v[k - 1]) / h2y;
      }
      div[k] = d;
    }
    if (speed) speed[k] = sqrtf(u[k] * u[k] + v[k] * v[k]);
    if (dye.c) dye.c_out[k] = dye_at<false, PER>(dye, i, j, nx, ny, h2x, h2y, dx, u[k], v[k]);
  }
}

static int post_step(const AjStepParams* prm, const float* u, const float* v, const float* c_in,
                     float* c_out, float dt, float diffusivity, float* vort, float* div,
                     float* speed, void* stream) {
  if (!prm || !u || !v || prm->nx < 2 || prm->ny < 2 || prm->dx <= 0 || prm->dy <= 0)
    return AJ_ERR_PARAM;
  if ((c_in == nullptr) != (c_out == nullptr) || (c_in && c_in == c_out)) return AJ_ERR_PARAM;
  const int nx = prm->nx, ny = prm->ny;
  const bool mac = prm->grid_type == AJ_GRID_MAC;
  const bool per = prm->flow_type != AJ_FLOW_VON_KARMAN;
  const float dx = (float)prm->dx, dy = (float)prm->dy;
  const Dye dye{c_in, c_out, dt, diffusivity, (float)(prm->dx * prm->dx),
                (float)(prm->dy * prm->dy)};
  dim3 blk(32, 8), grd(cdiv(ny, 32), cdiv(nx, 8));
  cudaStream_t st = (cudaStream_t)stream;
  if (mac && per)
    k_diagnostics<true, true><<<grd, blk, 0, st>>>(u, v, nx, ny, dx, dy, vort, div, speed, dye);
  else if (mac)
    k_diagnostics<true, false><<<grd, blk, 0, st>>>(u, v, nx, ny, dx, dy, vort, div, speed, dye);
  else if (per)
    k_diagnostics<false, true><<<grd, blk, 0, st>>>(u, v, nx, ny, dx, dy, vort, div, speed, dye);
  else
    k_diagnostics<false, false><<<grd, blk, 0, st>>>(u, v, nx, ny, dx, dy, vort, div, speed, dye);
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}
}  // namespace aj

extern "C" int32_t aj_diagnostics(const AjStepParams* prm, const float* u, const float* v,
                                  float* vort, float* div, float* speed, void* stream) {
  return aj::post_step(prm, u, v, nullptr, nullptr, 0.f, 0.f, vort, div, speed, stream);
}

extern "C" int32_t aj_post_step(const AjStepParams* prm, const float* u, const float* v,
                                const float* c_in, float* c_out, float dt, float diffusivity,
                                float* vort, float* div, float* speed, void* stream) {
  return aj::post_step(prm, u, v, c_in, c_out, dt, diffusivity, vort, div, speed, stream);
}
