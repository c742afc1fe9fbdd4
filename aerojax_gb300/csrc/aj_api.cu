// C ABI of aerojax_gb300 (declared in include/aerojax_gb300.h).
//
// aj_step and aj_poisson_mg record their kernels into a CUDA graph: when the
// caller's stream is already capturing, straight into the caller's graph;
// otherwise into a graph owned by the library, instantiated once per distinct
// (parameters, workspace, buffers) and launched on the caller's stream.  The
// converging multigrid's refinement loop is a while node inside that graph,
// so a step never waits on the host.
#include "aj_internal.cuh"
#include <deque>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>
#include <string.h>
#include <stdlib.h>

namespace aj {

int parity_levels(int nx, int ny, int levels, int* max_levels) {
  // multigrid_solver.py:96-106, plus the shapes its recursion needs
  int ml = 1, tx = nx, ty = ny;
  while (tx % 2 == 0 && ty % 2 == 0 && ml < levels) {
    tx /= 2;
    ty /= 2;
    ml++;
  }
  if (ml < 2) return AJ_ERR_SHAPE;
  int n = nx, m = ny;
  for (int k = 0; k < ml; ++k) {
    if (n % 2 || m % 2 || n / 2 < 2 || m / 2 < 2) return AJ_ERR_SHAPE;
    n /= 2;
    m /= 2;
  }
  if (ml > AJ_MAX_LEVELS) return AJ_ERR_SHAPE;
  *max_levels = ml;
  return AJ_OK;
}

int converge_depth(int nx, int ny) {
  // halve while both sizes are even and the halves keep >= 2 cells, until the
  // coarse grid has <= AJ_MAX_COARSE cells; always coarsen at least once
  int k = 0, n = nx, m = ny;
  while (n % 2 == 0 && m % 2 == 0 && n / 2 >= 2 && m / 2 >= 2 &&
         ((long)n * m > AJ_MAX_COARSE || k == 0) && k < AJ_MAX_LEVELS) {
    n /= 2;
    m /= 2;
    ++k;
  }
  return k;
}

bool eager_mode() {
  static int v = -1;
  if (v < 0) {
    const char* e = getenv("AEROJAX_EAGER");
    v = (e && e[0] && e[0] != '0') ? 1 : 0;
  }
  return v == 1;
}

bool pdl_enabled() {
  static int v = -1;
  if (v < 0) {
    const char* e = getenv("AEROJAX_PDL");
    v = (e && e[0] == '0') ? 0 : 1;
  }
  return v == 1;
}

int eager_unroll(int max_cycles) {
  const char* e = getenv("AEROJAX_UNROLL");
  int n = e ? atoi(e) : max_cycles;
  return n < 1 ? 1 : (n > max_cycles ? max_cycles : n);
}

int check_params(const AjStepParams& p) {
  if (p.nx < 4 || p.ny < 4) return AJ_ERR_SHAPE;
  if (p.dx <= 0 || p.dy <= 0) return AJ_ERR_PARAM;
  if (p.grid_type != AJ_GRID_COLLOCATED && p.grid_type != AJ_GRID_MAC) return AJ_ERR_PARAM;
  if (p.flow_type < AJ_FLOW_VON_KARMAN || p.flow_type > AJ_FLOW_TAYLOR_GREEN) return AJ_ERR_PARAM;
  if (p.les_model < AJ_LES_NONE || p.les_model > AJ_LES_DYNAMIC) return AJ_ERR_PARAM;
  if (p.mg_mode != AJ_MG_PARITY && p.mg_mode != AJ_MG_CONVERGE && p.mg_mode != AJ_MG_NONE)
    return AJ_ERR_PARAM;
  if (p.mg_mode == AJ_MG_NONE) {
    // predictor / LES workspace: no multigrid shape rules
  } else if (p.mg_mode == AJ_MG_PARITY) {
    int ml;
    int rc = parity_levels(p.nx, p.ny, p.levels > 0 ? p.levels : 4, &ml);
    if (rc != AJ_OK) return rc;
    if (p.v_cycles < 1) return AJ_ERR_PARAM;
  } else {
    int D = converge_depth(p.nx, p.ny);
    if (D < 1) return AJ_ERR_SHAPE;
    long nc = (long)(p.nx >> D) * (p.ny >> D);
    if (nc > AJ_MAX_COARSE_HARD) return AJ_ERR_SHAPE;
    if (p.mg_rtol <= 0 || p.max_cycles < 1) return AJ_ERR_PARAM;
  }
  if (p.warm_start < AJ_WARM_ZERO || p.warm_start > AJ_WARM_EXTRAPOLATE) return AJ_ERR_PARAM;
  if (p.warm_start == AJ_WARM_EXTRAPOLATE && p.mg_mode != AJ_MG_CONVERGE) return AJ_ERR_PARAM;
  if (p.cfl_dt && (p.cfl_target <= 0 || p.dt_max <= 0)) return AJ_ERR_PARAM;
  if (!p.cfl_dt && p.dt <= 0) return AJ_ERR_PARAM;
  return AJ_OK;
}

bool make_layout(const AjStepParams& p, Layout& L) {
  if (check_params(p) != AJ_OK) return false;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off += (bytes + 255) & ~(size_t)255;
    return o;
  };
  const long nx = p.nx, ny = p.ny, N = nx * ny;
  const bool mac = p.grid_type == AJ_GRID_MAC;
  const long nU = mac ? (nx + 1) * ny : N, nV = mac ? nx * (ny + 1) : N;
  L = Layout();
  L.scalars = take(sizeof(DevScalars) < 256 ? 256 : sizeof(DevScalars));
  if (!mac) L.chi = take(N * 4);
  L.sA_u = take(nU * 4);
  L.sA_v = take(nV * 4);
  L.sB_u = take(nU * 4);
  L.sB_v = take(nV * 4);
  L.sS_u = take(nU * 4);
  L.sS_v = take(nV * 4);
  L.k1_u = take(nU * 4);
  L.k1_v = take(nV * 4);
  L.nu_sgs = take(N * 4);
  L.dyn = take(16 * N * 4);
  L.b0 = take(N * 4);
  L.T0 = take(N * 4);
  if (p.mg_mode == AJ_MG_PARITY) {
    int ml;
    parity_levels(p.nx, p.ny, p.levels > 0 ? p.levels : 4, &ml);
    L.nlev = ml;
    for (int l = 0; l <= ml; ++l) {
      L.ln[l] = p.nx >> l;
      L.lm[l] = p.ny >> l;
      if (l == 0) continue;
      long n = (long)L.ln[l] * L.lm[l];
      L.X[l] = take(n * 4);
      L.T[l] = take(n * 4);
      L.B[l] = take(n * 4);
      if (mac) L.M[l] = take(n * 4);
    }
  } else if (p.mg_mode == AJ_MG_CONVERGE) {
    int D = converge_depth(p.nx, p.ny);
    L.nlev = D;
    for (int l = 0; l <= D; ++l) {
      L.ln[l] = p.nx >> l;
      L.lm[l] = p.ny >> l;
      long n = (long)L.ln[l] * L.lm[l];
      L.X[l] = take(n * 4);
      L.T[l] = take(n * 4);
      L.B[l] = take(n * 4);
    }
    L.ncoarse = L.ln[D] * L.lm[D];
    L.p64 = take(N * 8);
    L.p64b = take(N * 8);
    if (p.warm_start == AJ_WARM_EXTRAPOLATE) L.hist = take(2 * N * 8);
    L.cinv = take((size_t)L.ncoarse * L.ncoarse * 8);
    // the coarse solve: an exact separable solve at level ld when one fits,
    // else levels lc..D in one thread block with everything in shared memory
    L.ld = converge_direct_level(L);
    if (L.ld > 0) {
      L.lc = L.ld;
      L.dcy = take((size_t)L.lm[L.ld] * L.lm[L.ld] * 4);
      L.dly = take((size_t)L.lm[L.ld] * 4);
      L.dtmp = take((size_t)L.ln[L.ld] * L.lm[L.ld] * 4);
    } else {
      L.lc = converge_first_block_level(L);
    }
  }
  if (p.nn_factor > 0 && p.mg_mode == AJ_MG_CONVERGE && nn_step_shape_ok(p)) {
    L.nn_act = take(nn_step_act_bytes(p));
  }
  L.part = take(kPartials * 8);
  L.total = off;
  return true;
}

// effective parameters: step_pure hard-wires slip walls and no hyperviscosity
// (step.py:177-180) and cannot run on the MAC grid (step.py:348 broadcasts
// (nx+1, ny) against (nx, ny))
AjStepParams normalise(const AjStepParams& in) {
  AjStepParams p = in;
  if (p.levels <= 0) p.levels = 4;
  if (p.variant == AJ_VARIANT_PURE) {
    p.nu_hyper_ratio = 0.0;
    p.slip_walls = 1;
  }
  if (p.mg_tolerance <= 0) p.mg_tolerance = AJ_PARITY_TOL_DEFAULT;
  return p;
}

// ------------------------------------------------------------- graph cache
namespace {
std::mutex g_mu;
std::unordered_map<std::string, cudaGraphExec_t> g_cache;
std::deque<std::string> g_order;   // insertion order, for eviction
cudaStream_t g_capture = nullptr;
// Executable graphs kept at once.  Callers that allocate fresh output tensors
// every step produce new pointer keys; the oldest graph is destroyed beyond
// this count (an in-flight graph is freed by CUDA when it completes).
constexpr size_t kMaxGraphs = 64;

std::string make_key(int kind, const AjStepParams& p, std::initializer_list<const void*> ptrs) {
  std::string k;
  const int tv = tile_variant(p.nx, p.ny);   // the autotuned level-0 tiles are baked in
  k.append(reinterpret_cast<const char*>(&kind), sizeof(kind));
  k.append(reinterpret_cast<const char*>(&tv), sizeof(tv));
  k.append(reinterpret_cast<const char*>(&p), sizeof(p));
  for (const void* q : ptrs) k.append(reinterpret_cast<const char*>(&q), sizeof(q));
  return k;
}

// branch streams and fork/join events of the ensemble capture (created once)
cudaStream_t* ensemble_streams(int n) {
  static std::vector<cudaStream_t> v;
  while ((int)v.size() < n) {
    cudaStream_t s;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
    v.push_back(s);
  }
  return v.data();
}
cudaEvent_t* ensemble_events(int n) {
  static std::vector<cudaEvent_t> v;
  while ((int)v.size() < n) {
    cudaEvent_t e;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
    v.push_back(e);
  }
  return v.data();
}

template <typename F>
int run_captured(const std::string& key, cudaStream_t user, F&& enqueue) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(user, &cs) != cudaSuccess) return AJ_ERR_CUDA;
  if (cs == cudaStreamCaptureStatusActive) return enqueue(user);   // caller's own graph
  if (eager_mode()) return enqueue(user);                          // profiling mode
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_cache.find(key);
  if (it == g_cache.end()) {
    if (!g_capture && cudaStreamCreateWithFlags(&g_capture, cudaStreamNonBlocking) != cudaSuccess)
      return AJ_ERR_CUDA;
    if (cudaStreamBeginCapture(g_capture, cudaStreamCaptureModeRelaxed) != cudaSuccess)
      return AJ_ERR_CUDA;
    int rc = enqueue(g_capture);
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamEndCapture(g_capture, &g);
    if (rc != AJ_OK || ce != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      return rc != AJ_OK ? rc : AJ_ERR_CUDA;
    }
    cudaGraphExec_t ex;
    if (cudaGraphInstantiate(&ex, g, 0) != cudaSuccess) {
      cudaGraphDestroy(g);
      return AJ_ERR_CUDA;
    }
    cudaGraphDestroy(g);
    while (g_cache.size() >= kMaxGraphs && !g_order.empty()) {
      auto old = g_cache.find(g_order.front());
      if (old != g_cache.end()) {
        cudaGraphExecDestroy(old->second);
        g_cache.erase(old);
      }
      g_order.pop_front();
    }
    it = g_cache.emplace(key, ex).first;
    g_order.push_back(key);
  }
  return cudaGraphLaunch(it->second, user) == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}
}  // namespace

static int ws_ok(const Layout& L, void* ws, size_t bytes) {
  if (!ws || bytes < L.total) return AJ_ERR_WORKSPACE;
  if (reinterpret_cast<uintptr_t>(ws) % 256) return AJ_ERR_WORKSPACE;
  return AJ_OK;
}

struct NnRef {
  const uint16_t* packed = nullptr;
  const float* master = nullptr;
};

// Side branches of a step (two streams, four events) per lane: lane i of an
// ensemble capture uses its own, so that no two instances' branches chain.
// enqueue_step (and aj_poisson_mg) hold g_forks_mu while they record, so that
// two host threads (each capturing into its own graph, or launching eagerly)
// never interleave records of the same events or of the converging solve's
// loop-body stream.
std::mutex g_forks_mu;
struct StepForks {
  cudaStream_t les, init, io;
  cudaEvent_t start, les_done, dt_done, init_done, io_p_in, io_p_ready, io_p_done;
};
static const StepForks* step_forks(int lane) {
  static std::vector<StepForks> v;
  static std::mutex mu;
  std::lock_guard<std::mutex> lk(mu);
  while ((int)v.size() <= lane) {
    StepForks f;
    if (cudaStreamCreateWithFlags(&f.les, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&f.init, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&f.io, cudaStreamNonBlocking) != cudaSuccess)
      return nullptr;
    cudaEvent_t* e[7] = {&f.start,   &f.les_done,   &f.dt_done,  &f.init_done,
                         &f.io_p_in, &f.io_p_ready, &f.io_p_done};
    for (cudaEvent_t* q : e)
      if (cudaEventCreateWithFlags(q, cudaEventDisableTiming) != cudaSuccess) return nullptr;
    v.push_back(f);
  }
  return &v[lane];
}

// Host buffers of a step (aj_step_host): the pressure guess is uploaded on a
// side branch that only the pressure solve waits for, and the new pressure
// is downloaded on that branch while the correction runs.
struct HostIO {
  const float* h_p = nullptr;   // host pressure guess (nullable)
  float* h_po = nullptr;        // host pressure result
  size_t p_bytes = 0;
};

// One step.  Two pieces of work run beside the main chain: the LES viscosity
// (it reads only the input velocities) beside the CFL reduction, and the
// converging solve's initial state (it needs dt and the history, not the
// rhs) beside the predictor and the divergence.
static int enqueue_step(const AjStepParams& p, const Layout& L, void* ws, const float* u,
                        const float* v, const float* mask, const float* p_guess, float* uo,
                        float* vo, float* po, AjStats* stats, cudaStream_t st,
                        NnRef nn = NnRef(), int lane = 0, const HostIO* io = nullptr) {
  std::lock_guard<std::mutex> forks_lock(g_forks_mu);
  const StepForks* fk = step_forks(lane);
  if (!fk) return AJ_ERR_CUDA;
  if (io && io->h_p) {   // the guess's upload, beside everything up to the solve
    if (cudaEventRecord(fk->start, st) != cudaSuccess ||
        cudaStreamWaitEvent(fk->io, fk->start, 0) != cudaSuccess ||
        cudaMemcpyAsync(const_cast<float*>(p_guess), io->h_p, io->p_bytes,
                        cudaMemcpyHostToDevice, fk->io) != cudaSuccess ||
        cudaEventRecord(fk->io_p_in, fk->io) != cudaSuccess)
      return AJ_ERR_CUDA;
  }
  const bool mac = p.grid_type == AJ_GRID_MAC;
  // step_pure computes the LES field on the collocated path but never passes it
  // on (step.py:177-180): nothing to do.  The GUI step and MAC use it.
  const bool les = p.les_model != AJ_LES_NONE && (p.variant == AJ_VARIANT_GUI || mac);
  const bool conv = p.mg_mode == AJ_MG_CONVERGE;
  const float* nsg = nullptr;
  int dc = 0;
  int rc;
  if (les) {
    float* f = at<float>(ws, L.nu_sgs);
    if (cudaEventRecord(fk->start, st) != cudaSuccess ||
        cudaStreamWaitEvent(fk->les, fk->start, 0) != cudaSuccess)
      return AJ_ERR_CUDA;
    rc = launch_les(p, L, ws, p.les_model, u, v, mac, f, nullptr, fk->les);
    if (rc != AJ_OK) return rc;
    if (cudaEventRecord(fk->les_done, fk->les) != cudaSuccess) return AJ_ERR_CUDA;
    nsg = f;
    dc = (p.variant == AJ_VARIANT_GUI && !mac) ? 1 : 0;
  }
  rc = p.cfl_dt ? launch_cfl(p, ws, u, v, nullptr, st) : launch_set_dt(p, ws, st);
  if (rc != AJ_OK) return rc;
  if (conv) {
    if (cudaEventRecord(fk->dt_done, st) != cudaSuccess ||
        cudaStreamWaitEvent(fk->init, fk->dt_done, 0) != cudaSuccess)
      return AJ_ERR_CUDA;
    // the initial state may read the guess: after its upload
    if (io && io->h_p && cudaStreamWaitEvent(fk->init, fk->io_p_in, 0) != cudaSuccess)
      return AJ_ERR_CUDA;
    rc = converge_init(p, L, ws, p_guess, fk->init);
    if (rc != AJ_OK) return rc;
    if (cudaEventRecord(fk->init_done, fk->init) != cudaSuccess) return AJ_ERR_CUDA;
  }
  if (les && cudaStreamWaitEvent(st, fk->les_done, 0) != cudaSuccess) return AJ_ERR_CUDA;
  float* us = at<float>(ws, L.sS_u);
  float* vs = at<float>(ws, L.sS_v);
  if (tile_predictor_ok(p, u, mask, nsg)) {
    // the three stages, boundary rows and the pressure rhs in one tile kernel
    const float* sb[4] = {at<float>(ws, L.sA_u), at<float>(ws, L.sA_v), at<float>(ws, L.sB_u),
                          at<float>(ws, L.sB_v)};
    rc = launch_predictor_tile(p, ws, u, v, mask, nsg, us, vs, at<float>(ws, L.b0), sb, st);
    if (rc != AJ_OK) return rc;
  } else {
    rc = launch_predictor(p, L, ws, u, v, mask, nsg, dc, us, vs, st);
    if (rc != AJ_OK) return rc;
    // with the learned warm start on the MAC grid, the network's features
    // kernel forms the right-hand side (one launch fewer before the network)
    if (!nn_forms_rhs(p, nn.packed != nullptr)) {
      rc = launch_rhs(p, L, ws, us, vs, mask, at<float>(ws, L.b0), st);
      if (rc != AJ_OK) return rc;
    }
  }
  if (conv && cudaStreamWaitEvent(st, fk->init_done, 0) != cudaSuccess) return AJ_ERR_CUDA;
  if (io && io->h_p && cudaStreamWaitEvent(st, fk->io_p_in, 0) != cudaSuccess)
    return AJ_ERR_CUDA;
  NnWarm nw;
  nw.packed = nn.packed;
  nw.master = nn.master;
  nw.mask = mask;
  if (nn_forms_rhs(p, nn.packed != nullptr) && !tile_predictor_ok(p, u, mask, nsg)) {
    nw.us = us;
    nw.vs = vs;
  }
  rc = launch_pressure(p, L, ws, mask, p_guess, po, stats, st, nn.packed ? &nw : nullptr, conv);
  if (rc != AJ_OK) return rc;
  if (io) {   // the pressure's download, beside the correction
    if (cudaEventRecord(fk->io_p_ready, st) != cudaSuccess ||
        cudaStreamWaitEvent(fk->io, fk->io_p_ready, 0) != cudaSuccess ||
        cudaMemcpyAsync(io->h_po, po, io->p_bytes, cudaMemcpyDeviceToHost, fk->io) !=
            cudaSuccess ||
        cudaEventRecord(fk->io_p_done, fk->io) != cudaSuccess)
      return AJ_ERR_CUDA;
  }
  rc = launch_correct(p, L, ws, us, vs, po, mask, uo, vo, st);
  if (rc != AJ_OK) return rc;
  if (io && cudaStreamWaitEvent(st, fk->io_p_done, 0) != cudaSuccess) return AJ_ERR_CUDA;
  return AJ_OK;
}

}  // namespace aj

using namespace aj;

extern "C" {

int32_t aj_version(void) { return 100; }

int32_t aj_check_params(const AjStepParams* prm) {
  if (!prm) return AJ_ERR_PARAM;
  AjStepParams p = normalise(*prm);
  int rc = check_params(p);
  if (rc != AJ_OK) return rc;
  if (p.mg_mode == AJ_MG_NONE) return AJ_OK;     // predictor / LES only: any flow type
  if (p.variant == AJ_VARIANT_PURE && p.grid_type == AJ_GRID_MAC) return AJ_ERR_PARAM;
  // the lid-driven cavity and Taylor-Green flows run with the reference's own
  // V-cycle; the converging solver's operator pins the von Karman outlet
  if (p.flow_type != AJ_FLOW_VON_KARMAN && p.mg_mode != AJ_MG_PARITY) return AJ_ERR_PARAM;
  return AJ_OK;
}

// the parameters of a call that runs a pressure solve
static int32_t solve_check(const AjStepParams* prm) {
  int32_t rc = aj_check_params(prm);
  if (rc != AJ_OK) return rc;
  return prm->mg_mode == AJ_MG_NONE ? AJ_ERR_PARAM : AJ_OK;
}

size_t aj_workspace_size(const AjStepParams* prm) {
  if (!prm) return 0;
  Layout L;
  if (!make_layout(normalise(*prm), L)) return 0;
  return L.total;
}

int32_t aj_prepare(const AjStepParams* prm, const float* mask, const float* sdf, void* ws,
                   size_t bytes, void* stream) {
  if (!prm || !mask) return AJ_ERR_PARAM;
  AjStepParams p = normalise(*prm);
  int rc = check_params(p);
  if (rc != AJ_OK) return rc;
  Layout L;
  make_layout(p, L);
  if ((rc = ws_ok(L, ws, bytes)) != AJ_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  if (cudaMemsetAsync(ws, 0, L.total, st) != cudaSuccess) return AJ_ERR_CUDA;
  if (p.has_sdf && !sdf) return AJ_ERR_PARAM;
  if ((rc = launch_chi(p, L, ws, mask, sdf, st)) != AJ_OK) return rc;
  if ((rc = prepare_pressure(p, L, ws, mask, st)) != AJ_OK) return rc;
  return cudaStreamSynchronize(st) == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

int32_t aj_step(const AjStepParams* prm, const float* u, const float* v, const float* mask,
                const float* p_guess, float* u_out, float* v_out, float* p_out, void* ws,
                size_t bytes, AjStats* stats, void* stream) {
  if (!prm || !u || !v || !mask || !u_out || !v_out || !p_out) return AJ_ERR_PARAM;
  int rc = solve_check(prm);
  if (rc != AJ_OK) return rc;
  AjStepParams p = normalise(*prm);
  if (p.warm_start == AJ_WARM_GUESS && !p_guess) return AJ_ERR_PARAM;
  Layout L;
  make_layout(p, L);
  if ((rc = ws_ok(L, ws, bytes)) != AJ_OK) return rc;
  const float* pg = p.warm_start ? p_guess : nullptr;
  std::string key = make_key(1, p, {ws, u, v, mask, pg, u_out, v_out, p_out, stats});
  return run_captured(key, (cudaStream_t)stream, [&](cudaStream_t s) {
    return enqueue_step(p, L, ws, u, v, mask, pg, u_out, v_out, p_out, stats, s);
  });
}

int32_t aj_step_nn(const AjStepParams* prm, const float* u, const float* v, const float* mask,
                   const float* p_prev, const uint16_t* nn_packed, const float* nn_master,
                   float* u_out, float* v_out, float* p_out, void* ws, size_t bytes,
                   AjStats* stats, void* stream) {
  if (!prm || !u || !v || !mask || !p_prev || !nn_packed || !nn_master || !u_out || !v_out ||
      !p_out)
    return AJ_ERR_PARAM;
  int rc = solve_check(prm);
  if (rc != AJ_OK) return rc;
  AjStepParams p = normalise(*prm);
  if (p.mg_mode != AJ_MG_CONVERGE || p.nn_factor <= 0) return AJ_ERR_PARAM;
  if (!nn_step_shape_ok(p)) return AJ_ERR_SHAPE;
  if (p.warm_start != AJ_WARM_EXTRAPOLATE) p.warm_start = AJ_WARM_GUESS;
  Layout L;
  make_layout(p, L);
  if ((rc = ws_ok(L, ws, bytes)) != AJ_OK) return rc;
  std::string key = make_key(3, p, {ws, u, v, mask, p_prev, nn_packed, nn_master, u_out, v_out,
                                    p_out, stats});
  NnRef nn;
  nn.packed = nn_packed;
  nn.master = nn_master;
  return run_captured(key, (cudaStream_t)stream, [&](cudaStream_t s) {
    return enqueue_step(p, L, ws, u, v, mask, p_prev, u_out, v_out, p_out, stats, s, nn);
  });
}

int32_t aj_step_host(const AjStepParams* prm, const float* h_u, const float* h_v,
                     const float* mask, const float* h_p, float* h_u_out, float* h_v_out,
                     float* h_p_out, float* d_in, float* d_out, const uint16_t* nn_packed,
                     const float* nn_master, void* ws, size_t bytes, AjStats* stats,
                     void* stream) {
  if (!prm || !h_u || !h_v || !mask || !h_u_out || !h_v_out || !h_p_out || !d_in || !d_out)
    return AJ_ERR_PARAM;
  if ((nn_packed == nullptr) != (nn_master == nullptr)) return AJ_ERR_PARAM;
  int rc = solve_check(prm);
  if (rc != AJ_OK) return rc;
  AjStepParams p = normalise(*prm);
  if (nn_packed) {
    if (p.mg_mode != AJ_MG_CONVERGE || p.nn_factor <= 0 || !h_p) return AJ_ERR_PARAM;
    if (!nn_step_shape_ok(p)) return AJ_ERR_SHAPE;
    if (p.warm_start != AJ_WARM_EXTRAPOLATE) p.warm_start = AJ_WARM_GUESS;
  }
  if (p.warm_start == AJ_WARM_GUESS && !h_p) return AJ_ERR_PARAM;
  Layout L;
  make_layout(p, L);
  if ((rc = ws_ok(L, ws, bytes)) != AJ_OK) return rc;
  const bool mac = p.grid_type == AJ_GRID_MAC;
  const size_t nu = mac ? (size_t)(p.nx + 1) * p.ny : (size_t)p.nx * p.ny;
  const size_t nv = mac ? (size_t)p.nx * (p.ny + 1) : (size_t)p.nx * p.ny;
  const size_t np = (size_t)p.nx * p.ny;
  float *du = d_in, *dv = d_in + nu, *dp = d_in + nu + nv;
  float *duo = d_out, *dvo = d_out + nu, *dpo = d_out + nu + nv;
  const float* hp = p.warm_start ? h_p : nullptr;
  HostIO io;
  io.h_p = hp;
  io.h_po = h_p_out;
  io.p_bytes = np * 4;
  NnRef nn;
  nn.packed = nn_packed;
  nn.master = nn_master;
  std::string key = make_key(5, p, {ws, h_u, h_v, mask, hp, h_u_out, h_v_out, h_p_out, d_in,
                                    d_out, nn_packed, nn_master, stats});
  return run_captured(key, (cudaStream_t)stream, [&](cudaStream_t s) {
    // u and v as one copy each way on the step's stream: splitting them over
    // four concurrent branches measured no faster (the host link, not the
    // number of copy engines, sets the rate)
    if (cudaMemcpyAsync(du, h_u, nu * 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(dv, h_v, nv * 4, cudaMemcpyHostToDevice, s) != cudaSuccess)
      return (int)AJ_ERR_CUDA;
    // the pressure guess goes up, and the new pressure comes down, on the
    // step's io stream (enqueue_step), beside the predictor and the correction
    int r = enqueue_step(p, L, ws, du, dv, mask, hp ? dp : nullptr, duo, dvo, dpo, stats, s, nn,
                         0, &io);
    if (r != AJ_OK) return r;
    if (cudaMemcpyAsync(h_u_out, duo, nu * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(h_v_out, dvo, nv * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess)
      return (int)AJ_ERR_CUDA;
    return (int)AJ_OK;
  });
}

// the configurations the reverse pass covers: the collocated step_pure and
// GUI step (without LES) with the von Karman boundaries, upwind RK3/RK2, a
// fixed dt and the parity V-cycle
static int vjp_params_ok(const AjStepParams& p) {
  if (p.grid_type != AJ_GRID_COLLOCATED || p.flow_type != AJ_FLOW_VON_KARMAN ||
      p.mg_mode != AJ_MG_PARITY || p.advection != AJ_ADV_UPWIND || p.cfl_dt || p.warm_start ||
      p.nn_factor > 0)
    return AJ_ERR_PARAM;
  if (p.variant == AJ_VARIANT_GUI && p.les_model != AJ_LES_NONE) return AJ_ERR_PARAM;
  if (p.nx < 3 || p.ny < 3) return AJ_ERR_SHAPE;
  return AJ_OK;
}

size_t aj_step_vjp_workspace_size(const AjStepParams* prm) {
  if (!prm) return 0;
  AjStepParams p = normalise(*prm);
  Layout L;
  if (vjp_params_ok(p) != AJ_OK || !make_layout(p, L)) return 0;
  return step_vjp_workspace(p, L);
}

int32_t aj_step_vjp(const AjStepParams* prm, const float* u, const float* v, const float* mask,
                    const float* gu_out, const float* gv_out, const float* gp_out, float* gu,
                    float* gv, float* gsdf, double* gscal, void* ws, size_t bytes, void* aws,
                    size_t adj_bytes, void* stream) {
  if (!prm || !u || !v || !mask || !gu_out || !gv_out || !gu || !gv || !aws) return AJ_ERR_PARAM;
  int rc = solve_check(prm);
  if (rc != AJ_OK) return rc;
  AjStepParams p = normalise(*prm);
  if ((rc = vjp_params_ok(p)) != AJ_OK) return rc;
  Layout L;
  make_layout(p, L);
  if ((rc = ws_ok(L, ws, bytes)) != AJ_OK) return rc;
  if (adj_bytes < step_vjp_workspace(p, L)) return AJ_ERR_WORKSPACE;
  std::string key = make_key(6, p, {ws, aws, u, v, mask, gu_out, gv_out, gp_out, gu, gv, gsdf,
                                    gscal});
  return run_captured(key, (cudaStream_t)stream, [&](cudaStream_t s) {
    return launch_step_vjp(p, L, ws, aws, u, v, mask, gu_out, gv_out, gp_out, gu, gv, gsdf,
                           gscal, s);
  });
}

int32_t aj_step_vjp_kernel_count(const AjStepParams* prm) {
  if (!prm) return -1;
  AjStepParams p = normalise(*prm);
  Layout L;
  if (vjp_params_ok(p) != AJ_OK || !make_layout(p, L)) return -1;
  return step_vjp_kernel_count(p, L);
}

const float* aj_workspace_rhs(const AjStepParams* prm, void* ws) {
  if (!prm || !ws) return nullptr;
  Layout L;
  if (!make_layout(normalise(*prm), L)) return nullptr;
  return at<float>(ws, L.b0);
}

int32_t aj_poisson_mg(const AjStepParams* prm, const float* rhs, const float* mask,
                      const float* p0, float* p_out, void* ws, size_t bytes, AjStats* stats,
                      void* stream) {
  if (!prm || !rhs || !mask || !p_out) return AJ_ERR_PARAM;
  AjStepParams p = normalise(*prm);
  int rc = check_params(p);
  if (rc != AJ_OK) return rc;
  if (p.mg_mode == AJ_MG_NONE) return AJ_ERR_PARAM;
  if (p.flow_type != AJ_FLOW_VON_KARMAN && p.mg_mode != AJ_MG_PARITY) return AJ_ERR_PARAM;
  Layout L;
  make_layout(p, L);
  if ((rc = ws_ok(L, ws, bytes)) != AJ_OK) return rc;
  if (p.mg_mode == AJ_MG_CONVERGE && p.warm_start != AJ_WARM_EXTRAPOLATE)
    p.warm_start = p0 ? AJ_WARM_GUESS : AJ_WARM_ZERO;
  std::string key = make_key(2, p, {ws, rhs, mask, p0, p_out, stats});
  return run_captured(key, (cudaStream_t)stream, [&](cudaStream_t s) {
    // the converging solve records its loop body through a shared side
    // stream: the same lock as a step's enqueue
    std::lock_guard<std::mutex> forks_lock(g_forks_mu);
    int r = launch_mg_rhs(p, L, ws, rhs, mask, s);
    if (r != AJ_OK) return r;
    return launch_pressure(p, L, ws, mask, p0, p_out, stats, s);
  });
}

int32_t aj_les(const AjStepParams* prm, int32_t model, const float* u, const float* v,
               float* nu_sgs, float* cd_out, void* ws, size_t bytes, void* stream) {
  if (!prm || !u || !v || !nu_sgs) return AJ_ERR_PARAM;
  AjStepParams p = normalise(*prm);
  if (p.nx < 3 || p.ny < 3) return AJ_ERR_SHAPE;
  Layout L;
  AjStepParams q = p;
  q.grid_type = AJ_GRID_COLLOCATED;
  q.mg_mode = AJ_MG_NONE;       // layout only needs the field buffers
  q.warm_start = AJ_WARM_ZERO;
  q.cfl_dt = 0;
  q.dt = 1.0;
  if (model == AJ_LES_DYNAMIC) {
    if (!make_layout(q, L)) return AJ_ERR_SHAPE;
    int rc = ws_ok(L, ws, bytes);
    if (rc != AJ_OK) return rc;
  }
  return launch_les(p, L, ws, model, u, v, 0, nu_sgs, cd_out, (cudaStream_t)stream);
}

int32_t aj_predictor(const AjStepParams* prm, const float* u, const float* v, const float* mask,
                     const float* nu_sgs, int32_t double_count, float* u_star, float* v_star,
                     void* ws, size_t bytes, void* stream) {
  if (!prm || !u || !v || !mask || !u_star || !v_star) return AJ_ERR_PARAM;
  AjStepParams p = normalise(*prm);
  int rc = check_params(p);
  if (rc != AJ_OK) return rc;
  Layout L;
  make_layout(p, L);
  if ((rc = ws_ok(L, ws, bytes)) != AJ_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  rc = p.cfl_dt ? launch_cfl(p, ws, u, v, nullptr, st) : launch_set_dt(p, ws, st);
  if (rc != AJ_OK) return rc;
  return launch_predictor(p, L, ws, u, v, mask, nu_sgs, double_count, u_star, v_star, st);
}

int32_t aj_cfl_dt(const AjStepParams* prm, const float* u, const float* v, float* dt_out,
                  void* ws, size_t bytes, void* stream) {
  if (!prm || !u || !v || !dt_out || !ws || bytes < 256) return AJ_ERR_PARAM;
  AjStepParams p = normalise(*prm);
  if (p.cfl_target <= 0 || p.dt_max <= 0) return AJ_ERR_PARAM;
  return launch_cfl(p, ws, u, v, dt_out, (cudaStream_t)stream);
}

int32_t aj_profile_kernel(const AjStepParams* prm, int32_t which, const float* u,
                          const float* v, const float* mask, void* ws, size_t bytes,
                          void* stream) {
  if (!prm) return AJ_ERR_PARAM;
  AjStepParams p = normalise(*prm);
  int rc = check_params(p);
  if (rc != AJ_OK) return rc;
  Layout L;
  make_layout(p, L);
  if ((rc = ws_ok(L, ws, bytes)) != AJ_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  if (which >= 0 && which <= 2) return profile_pressure_kernel(p, L, ws, which, st);
  if (which == 3) {   // the predictor (all stages) from (u, v) into the workspace
    if (!u || !v || !mask) return AJ_ERR_PARAM;
    return launch_predictor(p, L, ws, u, v, mask, nullptr, 0, at<float>(ws, L.sS_u),
                            at<float>(ws, L.sS_v), st);
  }
  return AJ_ERR_PARAM;
}

int32_t aj_kernel_count(const AjStepParams* prm, int32_t cycles) {
  if (!prm) return -1;
  AjStepParams p = normalise(*prm);
  Layout L;
  if (!make_layout(p, L)) return -1;
  const bool mac = p.grid_type == AJ_GRID_MAC;
  int n = 1;                                                    // cfl or set-dt
  if (p.les_model != AJ_LES_NONE && (p.variant == AJ_VARIANT_GUI || mac))
    n += p.les_model == AJ_LES_DYNAMIC ? (mac ? 1 : 0) + 4 : 1;
  if (tile_predictor_params_ok(p)) n += tile_predictor_kernels();   // stages + rhs in tile kernels
  else n += (p.fast_mode ? 2 : 3) + (nn_forms_rhs(p, p.nn_factor > 0) ? 0 : 1);   // stages, rhs
  if (p.mg_mode == AJ_MG_PARITY) {
    const int coarse = parity_coarsest_fused(L) ? 1 : 10;
    int per_cycle = 2 * L.nlev + coarse;                        // levels, coarsest
    if (p.flow_type == AJ_FLOW_TAYLOR_GREEN) per_cycle = 6 * L.nlev + coarse + 1;   // unfused
    n += 1 + p.v_cycles * per_cycle;                            // begin + cycles
    if (p.flow_type == AJ_FLOW_LID_DRIVEN_CAVITY) n += 4;       // mean and centre pin
  } else {
    int body = 2 * L.lc + 1 + (L.ld > 0 ? 2 : 0);               // downs, coarse solve, ups
    n += 2 + (cycles > 1 ? cycles : 1) * body + 1;              // init, resid, loop, out+stats
  }
  if (p.mg_mode == AJ_MG_PARITY) n += 1;                        // stats
  n += 1;                                                       // correction
  // features, scales, the convolutions (12, or 10 with the two
  // full-resolution layer pairs fused), correction
  if (p.nn_factor > 0) n += 2 + nn_inference_conv_launches() + 1;
  return n;
}

int32_t aj_autotune(const AjStepParams* prm, void* ws, size_t bytes, int32_t reps,
                    float* times_ms, int32_t* chosen, void* stream) {
  if (!prm) return AJ_ERR_PARAM;
  AjStepParams p = normalise(*prm);
  int rc = check_params(p);
  if (rc != AJ_OK) return rc;
  if (p.mg_mode != AJ_MG_CONVERGE) return AJ_ERR_PARAM;
  Layout L;
  make_layout(p, L);
  if ((rc = ws_ok(L, ws, bytes)) != AJ_OK) return rc;
  int ch = 0;
  rc = converge_autotune(p, L, ws, reps > 0 ? reps : 10, times_ms, &ch, (cudaStream_t)stream);
  if (chosen) *chosen = ch;
  return rc;
}

int32_t aj_ensemble_step(int32_t n, const AjStepParams* prms, const float* const* u,
                         const float* const* v, const float* const* mask,
                         const float* const* p_guess, float* const* u_out, float* const* v_out,
                         float* const* p_out, void* const* ws, const size_t* ws_bytes,
                         AjStats* stats, void* stream) {
  if (n < 1 || n > AJ_ENSEMBLE_MAX || !prms || !u || !v || !mask || !u_out || !v_out || !p_out ||
      !ws || !ws_bytes)
    return AJ_ERR_PARAM;
  std::vector<AjStepParams> P(n);
  std::vector<Layout> Ls(n);
  std::string key;
  for (int i = 0; i < n; ++i) {
    int rc = solve_check(&prms[i]);
    if (rc != AJ_OK) return rc;
    P[i] = normalise(prms[i]);
    if (P[i].warm_start == AJ_WARM_GUESS && !(p_guess && p_guess[i])) return AJ_ERR_PARAM;
    if (!u[i] || !v[i] || !mask[i] || !u_out[i] || !v_out[i] || !p_out[i]) return AJ_ERR_PARAM;
    make_layout(P[i], Ls[i]);
    if ((rc = ws_ok(Ls[i], ws[i], ws_bytes[i])) != AJ_OK) return rc;
    const float* pg = (P[i].warm_start && p_guess) ? p_guess[i] : nullptr;
    key += make_key(4, P[i], {ws[i], u[i], v[i], mask[i], pg, u_out[i], v_out[i], p_out[i],
                              stats ? (const void*)(stats + i) : nullptr});
  }
  // one graph: the instances are independent branches forked from the
  // capturing stream and joined back, so they run concurrently
  return run_captured(key, (cudaStream_t)stream, [&](cudaStream_t s) {
    cudaStream_t* br = ensemble_streams(n);
    cudaEvent_t* ev = ensemble_events(n + 1);
    if (!br || !ev) return (int)AJ_ERR_CUDA;
    if (cudaEventRecord(ev[n], s) != cudaSuccess) return (int)AJ_ERR_CUDA;
    for (int i = 0; i < n; ++i) {
      if (cudaStreamWaitEvent(br[i], ev[n], 0) != cudaSuccess) return (int)AJ_ERR_CUDA;
      const float* pg = (P[i].warm_start && p_guess) ? p_guess[i] : nullptr;
      int rc = enqueue_step(P[i], Ls[i], ws[i], u[i], v[i], mask[i], pg, u_out[i], v_out[i],
                            p_out[i], stats ? stats + i : nullptr, br[i], NnRef(), i);
      if (rc != AJ_OK) return rc;
      if (cudaEventRecord(ev[i], br[i]) != cudaSuccess) return (int)AJ_ERR_CUDA;
    }
    for (int i = 0; i < n; ++i)
      if (cudaStreamWaitEvent(s, ev[i], 0) != cudaSuccess) return (int)AJ_ERR_CUDA;
    return (int)AJ_OK;
  });
}

int32_t aj_release_graphs(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto& kv : g_cache) cudaGraphExecDestroy(kv.second);
  g_cache.clear();
  g_order.clear();
  return AJ_OK;
}

}  // extern "C"
