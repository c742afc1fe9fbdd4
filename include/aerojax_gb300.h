/*
 * aerojax_gb300 — C ABI of the GB300 (sm_103a) projection-step library.
 *
 * The library replaces the hot path of AeroJAX's incompressible projection
 * step.  Each entry point below names the reference function it stands in for
 * (paths are relative to the AeroJAX project root).
 *
 * Conventions shared by every entry point
 *  - 2-D fields are float32, C order, indexed [i][j] with x on the first axis
 *    and y contiguous (solver/params.py:56, meshgrid indexing='ij').
 *    Collocated: u, v, p are nx*ny.  MAC: u is (nx+1)*ny, v is nx*(ny+1),
 *    p is nx*ny (solver/params.py:16-18).
 *  - All pointers are device pointers unless stated otherwise.  The caller
 *    owns every buffer; the library never allocates.  Scratch memory comes
 *    from a caller-allocated workspace sized by aj_workspace_size().
 *  - Work is enqueued on the given stream; nothing synchronises the host.
 *    aj_step / aj_poisson_mg issue no host reads and no allocation, so they
 *    can be captured in a CUDA graph after aj_prepare has run.
 *  - Return value: AJ_OK or an AjStatus error code (argument checks happen
 *    on the host before anything is enqueued).  Errors detected on the device
 *    (non-finite values, non-convergence in converging mode) are written to
 *    AjStats::err, read back asynchronously by the caller.
 */
#ifndef AEROJAX_GB300_H
#define AEROJAX_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  AJ_OK = 0,
  AJ_ERR_SHAPE = 1,         /* grid not divisible for multigrid: the reference's ValueError
                               (pressure_solvers/multigrid_solver.py:104-106)            */
  AJ_ERR_PARAM = 2,         /* unsupported option / bad scalar                           */
  AJ_ERR_NONFINITE = 3,     /* NaN/Inf seen in the pressure residual (device-side)       */
  AJ_ERR_NOT_CONVERGED = 4, /* converging mode hit max_cycles above rtol (device-side)   */
  AJ_ERR_TIMEOUT = 5,       /* a bounded device-side wait gave up                        */
  AJ_ERR_CUDA = 6,          /* a CUDA launch failed                                      */
  AJ_ERR_WORKSPACE = 7      /* workspace too small or null                               */
} AjStatus;

enum { AJ_GRID_COLLOCATED = 0, AJ_GRID_MAC = 1 };
enum { AJ_FLOW_VON_KARMAN = 0, AJ_FLOW_LID_DRIVEN_CAVITY = 1, AJ_FLOW_TAYLOR_GREEN = 2 };
/* PURE = step_pure (solver/pure_functions/step.py:49-467);
   GUI  = BaselineSolver._step (solver/simulation/step_handlers.py:62-301). */
enum { AJ_VARIANT_PURE = 0, AJ_VARIANT_GUI = 1 };
enum { AJ_LES_NONE = 0, AJ_LES_SMAGORINSKY = 1, AJ_LES_DYNAMIC = 2 };
enum { AJ_ADV_UPWIND = 0, AJ_ADV_WENO5 = 1 };
/* PARITY   = the reference V-cycle, fixed v_cycles, absolute early exit;
   CONVERGE = FP32 red-black Gauss-Seidel V-cycles (2 pre- and 2
              post-smoothing sweeps per level, 1 post-smoothing sweep on the
              finest) inside double-FP32 iterative refinement, an exact
              separable coarse solve (or an FP64 dense one), FP64 norms,
              relative stop;
   NONE     = no pressure solve: a workspace for aj_prepare, aj_predictor and
              aj_les only, on any grid of at least 4x4 cells and any flow type
              (the reference's rk_step_unified and LES models take any shape);
              the solving entry points reject it with AJ_ERR_PARAM. */
enum { AJ_MG_PARITY = 0, AJ_MG_CONVERGE = 1, AJ_MG_NONE = 2 };
/* Initial guess of the converging solve (no reference counterpart: the
   reference always starts from p = 0, multigrid_solver.py:219).
   ZERO        p = 0
   GUESS       p = p_guess (float, caller-owned)
   EXTRAPOLATE p = p1 + (dt / dt1) (p1 - p2) from the last two solutions of
               this workspace, kept in double-FP32 by the library; p_guess
               (nullable) seeds the first two steps. */
enum { AJ_WARM_ZERO = 0, AJ_WARM_GUESS = 1, AJ_WARM_EXTRAPOLATE = 2 };

/* Every scalar and static option of one step.  Mirrors the keyword arguments
   of step_pure (solver/pure_functions/step.py:50-66) plus the attributes the
   GUI step reads from BaselineSolver (step_handlers.py:64-90). */
typedef struct {
  int32_t nx, ny;                /* cell counts (p shape)                             */
  int32_t grid_type;             /* AJ_GRID_*                                         */
  int32_t flow_type;             /* AJ_FLOW_*  (von_karman is the configs' flow)      */
  int32_t variant;               /* AJ_VARIANT_*                                      */
  int32_t les_model;             /* AJ_LES_*                                          */
  int32_t advection;             /* AJ_ADV_*                                          */
  int32_t mg_mode;               /* AJ_MG_*                                           */
  int32_t fast_mode;             /* 1 = Heun RK2, 0 = RK3 (rk3_simple_new.py:356)     */
  int32_t slip_walls;            /* 1 = slip walls inside the predictor               */
  int32_t v_cycles;              /* parity mode: V-cycles per solve                   */
  int32_t levels;                /* parity mode: multigrid levels (reference: 4)      */
  int32_t max_cycles;            /* converging mode: cap on refinement cycles         */
  int32_t has_sdf;               /* collocated: chi from sdf (rk3_simple_new.py:194)  */
  int32_t cfl_dt;                /* 1 = dt from the CFL rule on the device each step  */
  int32_t warm_start;            /* converging mode initial guess: AJ_WARM_*          */
  int32_t nn_factor;             /* learned warm start: network grid is nx/F x ny/F,
                                    F in {2, 4, 8}, both multiples of 8
                                    (0 = off; aj_step_nn only)                        */
  double dx, dy;
  double dt;                     /* used when cfl_dt == 0                             */
  double dt_correction;          /* GUI: trace-time self.dt (step_handlers.py:139);
                                    <= 0 means "same as dt"                           */
  double nu, U_inf, brinkman_eta;
  double smagorinsky_constant;
  double nu_hyper_ratio;         /* GUI only; step_pure hard-wires 0 (step.py:178)    */
  double mg_tolerance;           /* parity: absolute early-exit tol (default 1e-6)    */
  double mg_rtol;                /* converging: relative residual target (1e-6)       */
  double cfl_target, dt_min, dt_max;  /* timestepping/cfl_adaptive_dt.py:6-71       */
  double les_delta;              /* LES filter width; <= 0 means sqrt(dx*dy)
                                    (step_handlers.py:71)                              */
} AjStepParams;

/* Device-resident per-call statistics (written by the last kernels of a call). */
typedef struct {
  int32_t cycles;        /* V-cycles executed                                      */
  int32_t converged;     /* parity: absolute test met; converging: rtol met        */
  int32_t err;           /* AJ_OK or a device-side AjStatus                        */
  int32_t pad;
  double rel_residual;   /* ||b - A p||_2 / ||b||_2 (FP64) after the solve         */
  double rhs_norm;       /* ||b||_2 (FP64)                                         */
  double dt;             /* dt the step used                                       */
  double abs_residual_sq;/* sum r^2 * dx * dy (the reference's early-exit quantity)*/
} AjStats;

/* Library version, e.g. 100 for 0.1.0. */
int32_t aj_version(void);

/* Bytes of device workspace needed for the given parameters (0 on bad params). */
size_t aj_workspace_size(const AjStepParams* prm);

/* Validates parameters the way the reference would at trace time.
   Returns AJ_OK, AJ_ERR_SHAPE (multigrid_solver.py:96-106) or AJ_ERR_PARAM. */
int32_t aj_check_params(const AjStepParams* prm);

/* Per-geometry set-up: Brinkman chi (rk3_simple_new.py:194-200), face masks,
   multigrid mask pyramid (multigrid_solver_mac.py:213-214), converging-mode
   coarse-grid inverse.  Must run again when the mask, sdf, grid or solver
   options change.  mask: nx*ny; sdf: nx*ny or NULL.  Synchronous. */
int32_t aj_prepare(const AjStepParams* prm, const float* mask, const float* sdf,
                   void* workspace, size_t workspace_bytes, void* stream);

/* One projection step.  Replaces step_pure (solver/pure_functions/step.py:49-467)
   for variant PURE and BaselineSolver._step (step_handlers.py:296-301) for
   variant GUI.  u_out/v_out/p_out must not alias the inputs; p_guess (nx*ny,
   nullable) seeds converging mode when warm_start is set. stats: device ptr or
   NULL. */
int32_t aj_step(const AjStepParams* prm, const float* u, const float* v, const float* mask,
                const float* p_guess, float* u_out, float* v_out, float* p_out,
                void* workspace, size_t workspace_bytes, AjStats* stats, void* stream);

/* Reverse mode of one step_pure: the vector-Jacobian product that jax.grad
   evaluates through the reference's differentiable rollouts
   (solver/solver.py:34-75 differentiable_rollout, :78-114 design_loss /
   grad_design_loss; inverse_design_WIP/optimizer_autodiff.py:113-205).
   Covers the collocated von Karman step with upwind RK3/RK2, a fixed dt
   (cfl_dt = 0) and the parity V-cycle: variant PURE (step_pure) and variant
   GUI without LES (BaselineSolver._step, step_handlers.py:62-185: the step
   the WIP optimizer scans, hyperviscosity and either wall condition);
   AJ_ERR_PARAM otherwise.
   Inputs: the step's inputs u, v (nx*ny) and the mask of aj_prepare on this
   workspace (prepared with the SDF when has_sdf), and the cotangents of the
   step's outputs gu_out, gv_out and gp_out (nullable: zero).  Writes the
   cotangents of the inputs gu, gv; adds the SDF's cotangent into gsdf
   (nullable; nothing is added without an SDF) and (d/d nu, d/d U_inf) into
   gscal[0..1] (nullable, FP64).  adj_workspace: aj_step_vjp_workspace_size
   bytes.  The forward stage states are recomputed inside the call. */
size_t aj_step_vjp_workspace_size(const AjStepParams* prm);
int32_t aj_step_vjp(const AjStepParams* prm, const float* u, const float* v, const float* mask,
                    const float* gu_out, const float* gv_out, const float* gp_out, float* gu,
                    float* gv, float* gsdf, double* gscal, void* workspace,
                    size_t workspace_bytes, void* adj_workspace, size_t adj_bytes, void* stream);
/* Kernels one aj_step_vjp launches (-1 on unsupported parameters). */
int32_t aj_step_vjp_kernel_count(const AjStepParams* prm);

/* The pressure solve alone.  Replaces poisson_multigrid
   (pressure_solvers/multigrid_solver.py:55-241) for grid_type COLLOCATED and
   poisson_multigrid_mac (pressure_solvers/multigrid_solver_mac.py:59-246) for
   grid_type MAC.  rhs, mask, p: nx*ny.  p0 nullable (zero guess). */
int32_t aj_poisson_mg(const AjStepParams* prm, const float* rhs, const float* mask,
                      const float* p0, float* p, void* workspace, size_t workspace_bytes,
                      AjStats* stats, void* stream);

/* Smagorinsky eddy viscosity.  Replaces constant_smagorinsky
   (solver/les_models.py:179-200) and dynamic_smagorinsky (:79-176) on
   collocated inputs (nx*ny).  model: AJ_LES_SMAGORINSKY or AJ_LES_DYNAMIC.
   cd_out nullable.  Dynamic needs a workspace of aj_workspace_size() with
   les_model = AJ_LES_DYNAMIC. */
int32_t aj_les(const AjStepParams* prm, int32_t model, const float* u, const float* v,
               float* nu_sgs, float* cd_out, void* workspace, size_t workspace_bytes,
               void* stream);

/* RK3/RK2 predictor with Brinkman penalisation.  Replaces rk_step_unified
   (advection_schemes/rk3_simple_new.py:175-358) for COLLOCATED and
   rk_step_unified_mac (advection_schemes/rk3_mac.py:220-504) for MAC.
   nu_sgs nullable; `double_count` = 1 reproduces the GUI collocated call that
   passes nu + nu_sgs as nu (step_handlers.py:76,84-85). Needs aj_prepare. */
int32_t aj_predictor(const AjStepParams* prm, const float* u, const float* v,
                     const float* mask, const float* nu_sgs, int32_t double_count,
                     float* u_star, float* v_star, void* workspace, size_t workspace_bytes,
                     void* stream);

/* CFL time step on the device.  Replaces compute_cfl_timestep
   (timestepping/cfl_adaptive_dt.py:6-71).  dt_out: one float (device). */
int32_t aj_cfl_dt(const AjStepParams* prm, const float* u, const float* v, float* dt_out,
                  void* workspace, size_t workspace_bytes, void* stream);

/* Obstacle geometry: SDF and mask = 1 - sigmoid(-sdf/eps)
   (solver/simulation/mask_generator.py:10-160, obstacles/naca_airfoils.py:109-178,
   obstacles/cylinder_array.py:8-42).  Coordinates are linspace(0, lx, nx) x
   linspace(0, ly, ny) (solver/params.py:51-56).  kind: AJ_GEOM_*.  geo[]:
     CYLINDER : cx, cy, r
     NACA4    : chord, aoa_deg, x_le, y_le, m, p, t
     CYL3_ROW : cx, cy, diameter, spacing          (three in a row along x)
     CYL3_TRI : cx, cy, diameter, spacing          (equilateral triangle)       */
enum { AJ_GEOM_NONE = 0, AJ_GEOM_CYLINDER = 1, AJ_GEOM_NACA4 = 2, AJ_GEOM_CYL3_ROW = 3,
       AJ_GEOM_CYL3_TRI = 4 };
int32_t aj_geometry(int32_t nx, int32_t ny, double lx, double ly, int32_t kind,
                    const double* geo_host, double eps, float* mask, float* sdf, void* stream);

/* ---------------------------------------------------------------------------
   Learned pressure warm start.  The reference's learned operators
   (neural_operators/nn_pressure_operator_*.py, trained by
   neural_operators/training_utils.py:84-253) replace the pressure solve
   (step_handlers.py:101-107); here a 4-level convolutional encoder-decoder
   (3x3 convs, base 32 channels, ~0.69 M parameters, BF16 tensor-core
   operands with FP32 accumulation) predicts a correction to the previous
   pressure on a grid nn_factor times coarser, and the converging multigrid
   always finishes the solve to mg_rtol.  Parameters: one flat FP32 master
   vector (per layer W[3][3][Cin][Cout] then b[Cout]) plus a BF16 packed copy
   made by aj_nn_pack.  Activations: NHWC [n][h][w][c], h and w multiples of 8. */
size_t aj_nn_param_count(void);
size_t aj_nn_packed_count(void);
size_t aj_nn_act_bytes(int32_t n, int32_t h, int32_t w);
/* Device pointer of the network input [n][h][w][16] inside an activation buffer. */
float* aj_nn_input(int32_t n, int32_t h, int32_t w, void* act);
int32_t aj_nn_pack(const float* master, uint16_t* packed, void* stream);
/* Forward pass; activations stay in `act` for the backward pass; y_out
   ([n][h][w][16], channel 0 = prediction) may be NULL. */
int32_t aj_nn_forward(int32_t n, int32_t h, int32_t w, const uint16_t* packed, const float* master,
                      void* act, size_t act_bytes, float* y_out, void* stream);
/* Gradient of sum(dy * y) w.r.t. the master parameters (grad is overwritten). */
int32_t aj_nn_backward(int32_t n, int32_t h, int32_t w, const float* dy, const uint16_t* packed,
                       const float* master, void* act, size_t act_bytes, float* grad,
                       void* stream);
/* MSE of channel 0 against target [n][h][w] (loss: one double, device), and dy. */
int32_t aj_nn_loss(int32_t n, int32_t h, int32_t w, const float* y, const float* target, float* dy,
                   double* loss, void* stream);
/* Adam on the master parameters with gradients clipped to [-clip, clip]
   (training_utils.py:162-188); step is 1-based. */
int32_t aj_nn_adam(float* master, const float* grad, float* m, float* v, int32_t step, float lr,
                   float beta1, float beta2, float eps, float clip, void* stream);
/* [n][h][w][3] features -> [n][h][w][16] network input. */
int32_t aj_nn_expand(int32_t n, int32_t h, int32_t w, const float* x3, float* x16, void* stream);
/* Training data for one solve (prm->nn_factor > 0): features x3_out
   [h][w][3] from the pressure rhs b (nx*ny, e.g. aj_workspace_rhs after a
   step), the mask and the previous pressure; with p_true the target
   [h][w] (nullable outputs).  Mirrors the reference's dataset contract
   (training_utils.py:35-51). */
int32_t aj_nn_features(const AjStepParams* prm, const float* b, const float* mask,
                       const float* p_prev, const float* p_true, float* x3_out, float* target_out,
                       void* workspace, size_t workspace_bytes, void* stream);
/* The learned warm start on its own, the reference's learned pressure
   operator call model(rhs, mask) (step_handlers.py:104-107,
   neural_operators/nn_pressure_operator_*.py) recast as a multigrid guess:
   p0 = p_prev + the network's correction from (rhs, mask, p_prev), for
   aj_poisson_mg's p0 in converging mode.  prm as for aj_step_nn (converging
   mode, nn_factor > 0); the workspace is the step's (aj_workspace_size(prm)).
   The outlet row of p0 is 0 (pinned in every solve).  Returns AJ_ERR_PARAM, AJ_ERR_SHAPE (the
   network grid's shape rule) or AJ_ERR_WORKSPACE before enqueueing anything. */
int32_t aj_nn_warmstart(const AjStepParams* prm, const float* rhs, const float* mask,
                        const float* p_prev, const uint16_t* nn_packed, const float* nn_master,
                        float* p0, void* workspace, size_t workspace_bytes, void* stream);
/* The pressure right-hand side of the last aj_step / aj_step_nn on this
   workspace (device pointer, nx*ny). */
const float* aj_workspace_rhs(const AjStepParams* prm, void* workspace);
/* One projection step (as aj_step, converging multigrid) whose pressure solve
   starts from p_prev + the network's correction. */
int32_t aj_step_nn(const AjStepParams* prm, const float* u, const float* v, const float* mask,
                   const float* p_prev, const uint16_t* nn_packed, const float* nn_master,
                   float* u_out, float* v_out, float* p_out, void* workspace,
                   size_t workspace_bytes, AjStats* stats, void* stream);

/* One step with the fields in (pinned) HOST memory - the call a host-driven
   loop makes (the reference's BaselineSolver._step hands back NumPy-visible
   arrays every step, step_handlers.py:296-301).  One graph launch: the
   upload of u, v, the step (aj_step, or aj_step_nn when nn_packed/nn_master
   are given), the download of u, v and p.  The pressure guess h_p is uploaded
   on a side branch that only the pressure solve waits for, and the new
   pressure is downloaded while the velocity correction runs.  d_in and
   d_out are device buffers of (nu + nv + nx*ny) floats each (nu, nv: the u
   and v sizes of the grid) that the call uses for the device copies; h_p
   may be NULL when the step ignores the guess. */
int32_t aj_step_host(const AjStepParams* prm, const float* h_u, const float* h_v,
                     const float* mask, const float* h_p, float* h_u_out, float* h_v_out,
                     float* h_p_out, float* d_in, float* d_out, const uint16_t* nn_packed,
                     const float* nn_master, void* ws, size_t bytes, AjStats* stats,
                     void* stream);

/* Post-step fields of step_for_visualization (visualization_step.py:224-256)
   into caller buffers (each nx*ny, nullable): vorticity
   (operators.py:105-108 / operators_mac.py:101-115; the periodic forms
   operators.py:99-102 / operators_mac.py:83-98 when flow_type is not von
   Karman), divergence (operators.py:75-96 / operators_mac.py:58-80) and the
   speed of the cell-centred velocity.  Reads prm->nx, ny, dx, dy, grid_type,
   flow_type. */
int32_t aj_diagnostics(const AjStepParams* prm, const float* u, const float* v, float* vort,
                       float* div, float* speed, void* stream);

/* The post-step epilogue in one kernel that reads the new velocity once:
   the diagnostics of aj_diagnostics and one explicit step of the passive
   scalar (dye) c (nx*ny, cell-centred): c_out = clip(c_in + dt (-(u, v).grad
   c_in + diffusivity lap c_in), 0, 1) with the reference's four variants
   (scalar_advection_diffusion_periodic / _nonperiodic, operators.py:111-150;
   the _staggered pair for MAC, operators_mac.py:161-215; non-periodic for the
   von Karman flow).  Every output is optional (NULL: not computed); c_in and
   c_out come together and must not alias.  Replaces the dye update and the
   step_for_visualization fields of the GUI loop
   (visualization_step.py:224-256). */
int32_t aj_post_step(const AjStepParams* prm, const float* u, const float* v, const float* c_in,
                     float* c_out, float dt, float diffusivity, float* vort, float* div,
                     float* speed, void* stream);

/* Allocation-free pressure solve, for callers that cannot allocate device
   memory: hosts that own every device byte through their own allocator (a
   framework's caching allocator, an XLA custom call without a scratch
   buffer) and latency-critical loops that cannot afford cudaMalloc's implicit
   synchronisation.  Same result as aj_poisson_mg in parity mode on the
   collocated grid (von Karman), but its scratch is a 14 MiB device array
   inside the library, so the caller passes only rhs, mask (nx*ny) and p
   (nx*ny); stats may be NULL.  The array is reserved on every device where
   the library's module is loaded (at first use under lazy module loading,
   the default; at context creation with CUDA_MODULE_LOADING=EAGER) until the
   process exits.  The call uses the current device's array: the stream and
   the three buffers must belong to the current device (AJ_ERR_PARAM
   otherwise).  Parameters follow aj_poisson_mg's rules; grids above
   AJ_STATIC_MAX_CELLS cells return AJ_ERR_WORKSPACE.  The first call on each
   device looks up the array's device address (cudaGetSymbolAddress); make
   that first call before any stream capture.  Every call shares the array:
   calls that overlap on the GPU race, so order them on one stream.  No
   counterpart in the reference. */
#define AJ_STATIC_MAX_CELLS (1 << 20)
int32_t aj_poisson_mg_static(const AjStepParams* prm, const float* rhs, const float* mask,
                             float* p, AjStats* stats, void* stream);

/* Instrumentation: one launch of a hot kernel on the workspace's current
   contents after an aj_step, so that it can be timed alone.  which:
   0/1/2 = converging multigrid level-0 down / up / FP64-residual kernel;
   3 = the predictor stages from (u, v).  No reference counterpart. */
int32_t aj_profile_kernel(const AjStepParams* prm, int32_t which, const float* u,
                          const float* v, const float* mask, void* workspace,
                          size_t workspace_bytes, void* stream);

/* Number of kernels one aj_step launches for these parameters when the
   converging solver ran `cycles` V-cycles (parity mode ignores `cycles`).
   Instrumentation only; no reference counterpart. */
int32_t aj_kernel_count(const AjStepParams* prm, int32_t cycles);

/* Drops the CUDA graphs aj_step / aj_poisson_mg instantiated for uncaptured
   streams (they are keyed by parameters, workspace and buffer pointers).
   Call only while none of them is executing.  No reference counterpart. */
int32_t aj_release_graphs(void);

/* Autotuner of the converging multigrid's level-0 tile shape for prm's grid
   (converging mode, after aj_prepare on this workspace): times each
   candidate `reps` times (level-0 pre- and post-smoothing kernels on the
   workspace's current contents), keeps the fastest for every later call on
   this grid shape in this process, and returns the per-candidate times (host
   array of AJ_TILE_VARIANTS floats, ms, nullable) and the choice (host,
   nullable).  Synchronises the stream.  No reference counterpart. */
#define AJ_TILE_VARIANTS 3
int32_t aj_autotune(const AjStepParams* prm, void* workspace, size_t workspace_bytes,
                    int32_t reps, float* times_ms, int32_t* chosen, void* stream);

/* Batched ensemble: one step of n independent simulations (each with its own
   parameters - grid sizes may differ -, fields and prepared workspace) as a
   single CUDA graph launch whose n branches run concurrently on the GPU.
   Every array is a host array of n entries; the pointers in them are device
   pointers (p_guess entries may be NULL where warm_start is not
   AJ_WARM_GUESS; stats: device array of n AjStats or NULL).  Instance i gets
   exactly what aj_step would give it.  No reference counterpart (the
   reference steps one simulation at a time). */
#define AJ_ENSEMBLE_MAX 256
int32_t aj_ensemble_step(int32_t n, const AjStepParams* prms, const float* const* u,
                         const float* const* v, const float* const* mask,
                         const float* const* p_guess, float* const* u_out, float* const* v_out,
                         float* const* p_out, void* const* workspaces,
                         const size_t* workspace_bytes, AjStats* stats, void* stream);

/* ---------------------------------------------------------------------------
   XLA FFI handlers: aj_prepare and aj_step as JAX custom calls, the binding
   of the reference's jit boundary (solver/simulation/step_handlers.py:304-315
   jax.jit(self._step); solver/pure_functions/step.py:49 step_pure's jit).
   Each takes XLA's XLA_FFI_CallFrame* (typed FFI, API version 0) and returns
   NULL or an XLA_FFI_Error* made with the call frame's API; register with
   jax.ffi.register_ffi_target(name, jax.ffi.pycapsule(fn), platform="CUDA").
   Both read one attribute "params": a uint8 array holding an AjStepParams.
   aj_ffi_prepare: (mask f32[nx*ny], sdf f32[nx*ny] or f32[0]) -> workspace
                   u8[>= aj_workspace_size]; synchronous, like aj_prepare.
   aj_ffi_step:    (u, v, mask, p_guess f32 (p_guess may be f32[0]),
                   workspace u8) -> (u_out, v_out, p_out f32[, workspace u8
                   aliased with the argument]).
   Argument errors come back as INVALID_ARGUMENT (RESOURCE_EXHAUSTED for a
   short workspace) with the AjStatus name in the message.  Stages other
   than execute return NULL. */
void* aj_ffi_prepare(void* call_frame);
void* aj_ffi_step(void* call_frame);

#ifdef __cplusplus
}
#endif
#endif /* AEROJAX_GB300_H */
