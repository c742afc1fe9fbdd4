// Internal declarations shared by the aerojax_gb300 CUDA translation units.
// Fields are row-major [i][j] with j (y) contiguous; threads map along j.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include "../../include/aerojax_gb300.h"

#define AJ_MAX_LEVELS 12
#define AJ_MAX_COARSE 64           // target cells of the converging-mode coarsest grid
#define AJ_MAX_COARSE_HARD 1024    // largest coarsest grid accepted (odd-sized grids)
#define AJ_PARITY_TOL_DEFAULT 1e-6

namespace aj {

// Device scalars living at the head of the workspace.
struct DevScalars {
  float dt;            // step dt (set on the device each step)
  float dt_corr;       // dt used by the pressure correction
  unsigned int cfl_max_bits;   // max |velocity| as float bits (atomicMax)
  unsigned int cfl_count;      // blocks finished (last-block pattern)
  int mg_skip;         // parity mode: V-cycles after convergence are skipped
  int mg_cycles;       // V-cycles executed in this solve
  int mg_done;         // converging mode: target met (later cycles skip)
  int err;             // device-side AjStatus
  double acc[4];       // reduction accumulators (residual, rhs, spare)
  double rel;          // last relative residual
  double bnorm;        // ||b||
  double abs_sq;       // sum r^2 dx dy
  unsigned int red_count;
  int loops;           // converging mode: executions of the while body
  int pcur;            // converging mode: which FP64 pressure buffer is current
  double nn_rms_r, nn_rms_p, nn_out_scale;   // learned warm start: per-sample scales
  int hist_n;          // converging mode: solutions held in the history (0..2)
  int hist_cur;        // history slot of the latest solution
  int hist_pending;    // a solve finished since the last k_cv_begin
  float dt_last;       // dt of the last finished solve
  float dt_prev;       // dt of the latest solution in the history
  unsigned int pad_[3];
};

struct Layout {
  size_t scalars = 0;
  size_t chi = 0, mask_u = 0, mask_v = 0;               // geometry-derived
  size_t sA_u = 0, sA_v = 0, sB_u = 0, sB_v = 0;        // predictor stage buffers
  size_t sS_u = 0, sS_v = 0;                            // predictor output (u*, v*)
  size_t k1_u = 0, k1_v = 0;                            // RK2 first slope
  size_t nu_sgs = 0;
  size_t dyn = 0;                                       // dynamic LES temporaries
  size_t b0 = 0, T0 = 0;                                // multigrid level-0 rhs, scratch
  size_t X[AJ_MAX_LEVELS + 1] = {0}, T[AJ_MAX_LEVELS + 1] = {0};
  size_t B[AJ_MAX_LEVELS + 1] = {0}, M[AJ_MAX_LEVELS + 1] = {0};
  size_t p64 = 0, p64b = 0;                             // converging mode FP64 pressure (ping-pong)
  size_t hist = 0;                                      // extrapolation history: 2 double-FP32 solutions
  size_t cinv = 0;                                      // coarsest-grid inverse (FP64)
  int lc = 0;                                           // first level of the coarse solve
  int ld = 0;                                           // level of the separable direct solve (0: none)
  size_t dcy = 0, dly = 0, dtmp = 0;                    // its cosine basis, y eigenvalues, scratch
  size_t nn_act = 0;                                    // learned warm start: activations
  size_t part = 0;                                      // per-block partial sums (FP64)
  size_t total = 0;
  // multigrid hierarchy
  int nlev = 0;                 // parity: max_levels (coarsest index); converge: depth
  int ln[AJ_MAX_LEVELS + 1] = {0}, lm[AJ_MAX_LEVELS + 1] = {0};
  int ncoarse = 0;              // converging: coarsest cell count
};

// Number of dynamic-LES temporaries (nx*ny floats each).
constexpr int kDynFields = 12;
constexpr int kPartials = 4096;

bool make_layout(const AjStepParams& p, Layout& L);
int check_params(const AjStepParams& p);
// effective parameters of a call (defaults filled in, step_pure's fixed options)
AjStepParams normalise(const AjStepParams& in);
int parity_levels(int nx, int ny, int levels, int* max_levels);
int converge_depth(int nx, int ny);

template <typename T>
inline T* at(void* ws, size_t off) { return reinterpret_cast<T*>(static_cast<char*>(ws) + off); }

// ------------------------------------------------------------------ helpers
__device__ __forceinline__ int clampi(int i, int n) { return i < 0 ? 0 : (i >= n ? n - 1 : i); }
// The MAC predictor's upwind weight alpha = (1 + tanh(w / 0.05)) / 2 of
// rk3_mac.py:386-391, evaluated as the equal logistic 1 / (1 + e^(-40 w))
// with the hardware exponential and a fast reciprocal: a few instructions
// instead of tanhf's sequence, relative error ~1e-7, exactly 0 and 1 in the
// tails (e^(-40 w) overflowing to infinity gives 0).
__device__ __forceinline__ float upwind_weight(float w) {
  return __fdividef(1.f, 1.f + __expf(-40.f * w));
}
// The implicit Brinkman step's division by 1 + dt chi / eta (>= 1) with the
// fast reciprocal (2 ulp) instead of the IEEE division sequence
__device__ __forceinline__ float brinkman_div(float num, float den) {
  return __fdividef(num, den);
}
// The pressure right-hand side of a MAC cell, mask * div(u*) / dt
// (operators_mac.py:73-80, multigrid_solver_mac.py:78), 0 on the outlet row
// when the flow pins it (multigrid_solver.py:75-77); k_rhs and the learned
// warm start's features kernel both use it.
__device__ __forceinline__ float rhs_mac_cell(const float* __restrict__ us,
                                              const float* __restrict__ vs,
                                              const float* __restrict__ mask, int i, int j, int nx,
                                              int ny, float idx, float idy, float dt, int outlet) {
  const float du = (__ldg(us + (long)(i + 1) * ny + j) - __ldg(us + (long)i * ny + j)) * idx;
  const float dv = (__ldg(vs + (long)i * (ny + 1) + j + 1) - __ldg(vs + (long)i * (ny + 1) + j)) * idy;
  const float out = ((du + dv) / dt) * __ldg(mask + (long)i * ny + j);
  return (outlet && i == nx - 1) ? 0.f : out;
}
__device__ __forceinline__ int wrapi(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }
template <bool PER>
__device__ __forceinline__ int pidx(int i, int n) { return PER ? wrapi(i, n) : clampi(i, n); }

__device__ __forceinline__ float ldg(const float* p) { return __ldg(p); }

// float atomic max for non-negative values (bit pattern order == value order)
__device__ __forceinline__ void atomic_max_nonneg(unsigned int* addr, float v) {
  atomicMax(addr, __float_as_uint(v));
}

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum of one double per thread, added atomically to *dst by one
// thread.  Every thread of the block must call it (it synchronises).
__device__ __forceinline__ void block_sum_atomic(double v, double* dst) {
  __shared__ double ws_[32];
  v = warp_sum(v);
  const int nthreads = blockDim.x * blockDim.y;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int lane = tid & 31, w = tid >> 5;
  if (lane == 0) ws_[w] = v;
  __syncthreads();
  if (w == 0) {
    v = lane < (nthreads >> 5) ? ws_[lane] : 0.0;
    v = warp_sum(v);
    if (lane == 0) atomicAdd(dst, v);
  }
  __syncthreads();
}

// ------------------------------------------------------------------ paired FP32
// Blackwell's paired FP32 instructions: each lane of __fadd2_rn / __fmul2_rn /
// __ffma2_rn rounds as the scalar operation does, and the explicit
// intrinsics are never contracted, so two independent values computed side
// by side cost one instruction per operation
__device__ __forceinline__ float2 f2(float x) { return make_float2(x, x); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// a - b as fma(b, -1, a): the exact difference, rounded once
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, f2(-1.f), a); }

// ------------------------------------------------------------------ double-FP32
// an unevaluated sum hi + lo of two floats (~48-bit significand on the FP32
// pipes; GB300 runs FP64 at 1/64 of the FP32 rate)
struct df {
  float hi, lo;
};
// Knuth's TwoSum: s + e == a + b exactly
__device__ __forceinline__ df two_sum(float a, float b) {
  float s = a + b;
  float bb = s - a;
  float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
// Dekker's FastTwoSum, valid for |a| >= |b|
__device__ __forceinline__ df quick_two_sum(float a, float b) {
  float s = a + b;
  return {s, b - (s - a)};
}
// Dekker's TwoProd with a fused multiply-add: p + e == a * b exactly
__device__ __forceinline__ df two_prod(float a, float b) {
  float p = a * b;
  return {p, fmaf(a, b, -p)};
}
__device__ __forceinline__ df df_add(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  df t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = quick_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return quick_two_sum(s.hi, s.lo);
}

// Block-wide sum of one double-FP32 value per thread, in a fixed order (the
// result is bit-reproducible): a TwoSum butterfly inside each warp, one FP64
// value per warp, the warps summed by thread 0, which gets the total.  Every
// thread of the block must call it (it synchronises).
__device__ __forceinline__ double block_sum_df(df v) {
  __shared__ double wd_[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float h = __shfl_xor_sync(0xffffffffu, v.hi, o);
    const float l = __shfl_xor_sync(0xffffffffu, v.lo, o);
    v = df_add(v, df{h, l});
  }
  const int nthreads = blockDim.x * blockDim.y;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  if ((tid & 31) == 0) wd_[tid >> 5] = (double)v.hi + (double)v.lo;
  __syncthreads();
  double t = 0.0;
  if (tid == 0)
    for (int k = 0; k < (nthreads >> 5); ++k) t += wd_[k];
  __syncthreads();
  return t;
}

// Block-wide sum of one float per thread added atomically to *dst by one
// thread: a double-FP32 TwoSum butterfly in each warp (the FP32 pipes; the
// FP64 butterfly of block_sum_atomic costs ~10 FP64 operations per thread on
// GB300's 1/64-rate FP64 pipe), one FP64 value per warp.  Every thread of the
// block must call it (it synchronises).
__device__ __forceinline__ void block_sum_atomic_f(float v, double* dst) {
  __shared__ double wf_[32];
  df s{v, 0.f};
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float h = __shfl_xor_sync(0xffffffffu, s.hi, o);
    const float l = __shfl_xor_sync(0xffffffffu, s.lo, o);
    s = df_add(s, df{h, l});
  }
  const int nthreads = blockDim.x * blockDim.y;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  if ((tid & 31) == 0) wf_[tid >> 5] = (double)s.hi + (double)s.lo;
  __syncthreads();
  if (tid == 0) {
    double t = 0.0;
    for (int k = 0; k < (nthreads >> 5); ++k) t += wf_[k];
    atomicAdd(dst, t);
  }
  __syncthreads();
}

// Block-wide sum of one double per thread in a fixed order (the result is
// bit-reproducible); the total is returned to thread 0.  Every thread of the
// block must call it (it synchronises).
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double wb_[32];
  v = warp_sum(v);
  const int nthreads = blockDim.x * blockDim.y;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int lane = tid & 31, w = tid >> 5;
  if (lane == 0) wb_[w] = v;
  __syncthreads();
  double t = 0.0;
  if (tid == 0)
    for (int k = 0; k < (nthreads >> 5); ++k) t += wb_[k];
  __syncthreads();
  return t;
}

// ------------------------------------------------------------------ dependent launch
// Programmatic dependent launch: a kernel started with launch_pdl may be
// scheduled as its predecessor on the stream drains (the launch latency
// overlaps the predecessor's tail; ~5 us per 2048x512 step).  It must execute
// pdl_wait() - which returns once the predecessor grid has completed and its
// writes are visible - before it reads or writes anything a predecessor
// touches, on every path (early returns included), so that its own completion
// still implies its predecessors'.  A no-op in a kernel launched normally.
// (Early triggers, griddepcontrol.launch_dependents at the start of the
// network's convolutions so that the next layer stages its weights sooner,
// or after the wait in the multigrid kernels, measured slower - the latter
// by a quarter of the solve: the dependent's blocks sit resident beside the
// running grid - and are not used.)
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
// AEROJAX_PDL=0 turns dependent launches off (read once)
bool pdl_enabled();
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(bool pdl, void (*kernel)(KArgs...), dim3 grid, dim3 block,
                              size_t smem, cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = (pdl && pdl_enabled()) ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// ------------------------------------------------------------------ launchers
// predictor (aj_predictor.cu)
int launch_predictor(const AjStepParams& p, const Layout& L, void* ws, const float* u,
                     const float* v, const float* mask, const float* nsg, int double_count,
                     float* us, float* vs, cudaStream_t st);
// the MAC predictor's three stages, boundary rows and pressure rhs (b,
// nullable) in one shared-memory tile kernel (aj_predictor_tile.cu)
bool tile_predictor_params_ok(const AjStepParams& p);
bool tile_predictor_ok(const AjStepParams& p, const float* u, const float* mask,
                       const float* nsg);
// stage_bufs: the workspace's stage buffers (A_u, A_v, B_u, B_v) the
// per-stage tile kernels pass the intermediate stages through
int launch_predictor_tile(const AjStepParams& p, void* ws, const float* u, const float* v,
                          const float* mask, const float* nsg, float* us, float* vs, float* b,
                          const float* const* stage_bufs, cudaStream_t st);
// kernels one tile predictor launches (1 fused, 3 per stage)
int tile_predictor_kernels();
int launch_les(const AjStepParams& p, const Layout& L, void* ws, int model, const float* u,
               const float* v, int mac_input, float* nu_sgs, float* cd, cudaStream_t st);
int launch_cfl(const AjStepParams& p, void* ws, const float* u, const float* v,
               float* dt_out, cudaStream_t st);
int launch_set_dt(const AjStepParams& p, void* ws, cudaStream_t st);
bool parity_coarsest_fused(const Layout& L);   // coarsest sweeps on one cluster (aj_pressure.cu)
// reverse mode of the collocated step_pure (aj_adjoint.cu)
size_t step_vjp_workspace(const AjStepParams& p, const Layout& L);
int launch_step_vjp(const AjStepParams& p, const Layout& L, void* ws, void* aws, const float* u,
                    const float* v, const float* mask, const float* gu_o, const float* gv_o,
                    const float* gp_o, float* gu, float* gv, float* gsdf, double* gscal,
                    cudaStream_t st);
int step_vjp_kernel_count(const AjStepParams& p, const Layout& L);
int launch_chi(const AjStepParams& p, const Layout& L, void* ws, const float* mask,
               const float* sdf, cudaStream_t st);
// projection (aj_project.cu)
int launch_rhs(const AjStepParams& p, const Layout& L, void* ws, const float* us,
               const float* vs, const float* mask, float* b, cudaStream_t st);
int launch_correct(const AjStepParams& p, const Layout& L, void* ws, const float* us,
                   const float* vs, const float* pr, const float* mask, float* uo, float* vo,
                   cudaStream_t st);
// pressure (aj_pressure.cu)
int prepare_pressure(const AjStepParams& p, const Layout& L, void* ws, const float* mask,
                     cudaStream_t st);
int launch_mg_rhs(const AjStepParams& p, const Layout& L, void* ws, const float* rhs,
                  const float* mask, cudaStream_t st);
// the learned warm start inside a converging solve (null pointers: off)
// the MAC converging step with the learned warm start forms its pressure
// right-hand side in the network's features kernel (no k_rhs launch)
inline bool nn_forms_rhs(const AjStepParams& p, bool learned) {
  return learned && p.grid_type == AJ_GRID_MAC && p.mg_mode == AJ_MG_CONVERGE;
}
// convolution launches of one inference pass (the layer pairs fused or not)
int nn_inference_conv_launches();
struct NnWarm {
  const uint16_t* packed = nullptr;
  const float* master = nullptr;
  const float* mask = nullptr;
  // MAC predictor outputs: when set, the features kernel forms the pressure
  // right-hand side itself (and stores it) instead of reading k_rhs's
  const float* us = nullptr;
  const float* vs = nullptr;
};
// init_done: converge_init already ran (the step launches it beside the
// predictor)
int launch_pressure(const AjStepParams& p, const Layout& L, void* ws, const float* mask,
                    const float* p0, float* pout, AjStats* stats, cudaStream_t st,
                    const NnWarm* nn = nullptr, bool init_done = false);
int profile_pressure_kernel(const AjStepParams& p, const Layout& L, void* ws, int which,
                            cudaStream_t st);
// converging multigrid (aj_converge.cu)
int converge_prepare(const AjStepParams& p, const Layout& L, void* ws, cudaStream_t st);
int converge_solve(const AjStepParams& p, const Layout& L, void* ws, const float* p0,
                   float* pout, cudaStream_t st, const NnWarm* nn = nullptr,
                   AjStats* stats = nullptr, bool init_done = false);
int converge_init(const AjStepParams& p, const Layout& L, void* ws, const float* p0,
                  cudaStream_t st);
size_t converge_block_smem(const Layout& L, int lc);
int converge_first_block_level(const Layout& L);
int converge_direct_level(const Layout& L);
// level-0 tile shape of a grid (0 until converge_autotune has run for it)
int tile_variant(int nx, int ny);
int converge_autotune(const AjStepParams& p, const Layout& L, void* ws, int reps, float* times_ms,
                      int* chosen, cudaStream_t st);
// learned warm start (aj_nn.cu)
size_t nn_step_act_bytes(const AjStepParams& p);
bool nn_step_shape_ok(const AjStepParams& p);
// adds the network's correction to the initial double-FP32 state (hi: N
// floats, lo: N floats) of a converging solve with right-hand side b
int nn_correct_state(const AjStepParams& p, const Layout& L, void* ws, const float* b,
                     const NnWarm& nn, float* state, cudaStream_t st);
constexpr size_t kBlockSmemMax = 220 * 1024;   // coarse-level kernel shared memory budget
// The parity V-cycle's coarsest level (10 Jacobi sweeps) runs on a cluster of
// kCoarseCtas blocks, each holding a band of rows in shared memory.
constexpr int kCoarseCtas = 8;
constexpr int kCoarseThreads = 256;
__host__ __device__ inline int coarse_band_rows(int n) { return (n + kCoarseCtas - 1) / kCoarseCtas; }

inline unsigned cdiv(long a, long b) { return (unsigned)((a + b - 1) / b); }

// Profiling mode: AEROJAX_EAGER=1 makes aj_step / aj_poisson_mg launch their
// kernels straight onto the stream instead of through a CUDA graph (profilers
// cannot attribute kernels inside graphs with conditional nodes); the
// converging loop then runs AEROJAX_UNROLL bodies (default max_cycles).
bool eager_mode();
int eager_unroll(int max_cycles);

}  // namespace aj
