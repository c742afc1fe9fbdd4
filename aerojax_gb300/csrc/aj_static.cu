// Allocation-free entry point: the reference-parity multigrid (collocated
// grid) running on a scratch area that the library itself owns as a
// file-scope device array, for callers that cannot allocate device memory.
//
// Who needs it: hosts that hand out no device memory of their own for a call
// (a plugin whose host owns every byte through its own allocator, such as a
// framework's caching allocator or an XLA custom call without a scratch
// buffer), and latency-critical loops where cudaMalloc's implicit device
// synchronisation is not acceptable.  Such a caller passes only the
// right-hand side, the mask and the output pressure.
//
// The scratch array below is part of the library image: it is reserved on
// every device where the library's module is loaded - at first use under the
// default lazy module loading, at context creation with
// CUDA_MODULE_LOADING=EAGER - and held until the process exits.  Grids above
// AJ_STATIC_MAX_CELLS cells are rejected.  All calls share the one array, which keeps the last call's
// contents; each call clears the part that must start at zero.  Calls whose
// work overlaps on the GPU (other streams, other host threads) race on the
// array: order them on one stream or serialise them.
#include "aj_internal.cuh"
#include <mutex>

namespace aj {

constexpr size_t kStaticScratchBytes = (size_t)14 << 20;   // 14 MiB

// Worst case of static_layout at AJ_STATIC_MAX_CELLS: the level-0 rhs and
// scratch (8 B per cell), three arrays per coarse level (12 B per cell times
// sum 4^-l < 1/3, i.e. < 4 B per cell), and at most 255 B of alignment per
// array for the scalars and up to 16 levels.
static_assert((size_t)AJ_STATIC_MAX_CELLS * 12 + 256 * (3 + 3 * 16) <= kStaticScratchBytes,
              "the static scratch array cannot hold the largest allowed grid");

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

namespace {
std::mutex g_static_mu;
void* g_static_ptr[64] = {nullptr};   // device address of the array, per device ordinal

// Set-up, once per device, with that device current: the address of the
// array as the device sees it.  (On the host, g_static_scratch names a host
// shadow, not device memory, so it is never passed to a kernel.)
int static_scratch_address(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return AJ_ERR_CUDA;
  std::lock_guard<std::mutex> lk(g_static_mu);
  if (!g_static_ptr[dev]) {
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_static_scratch) != cudaSuccess || !ptr) {
      cudaGetLastError();
      return AJ_ERR_CUDA;
    }
    g_static_ptr[dev] = ptr;
  }
  *out = g_static_ptr[dev];
  return AJ_OK;
}

// Compact layout: device scalars, the level-0 right-hand side and scratch,
// and three arrays per coarse level - only what the parity solve touches.
bool static_layout(const AjStepParams& p, Layout& L) {
  int ml;
  if (parity_levels(p.nx, p.ny, p.levels, &ml) != AJ_OK) return false;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off += (bytes + 255) & ~(size_t)255;
    return o;
  };
  L = Layout();
  L.scalars = take(256);
  const long N = (long)p.nx * p.ny;
  L.b0 = take(N * 4);
  L.T0 = take(N * 4);
  L.nlev = ml;
  for (int l = 0; l <= ml; ++l) {
    L.ln[l] = p.nx >> l;
    L.lm[l] = p.ny >> l;
    if (l == 0) continue;
    long n = (long)L.ln[l] * L.lm[l];
    L.X[l] = take(n * 4);
    L.T[l] = take(n * 4);
    L.B[l] = take(n * 4);
  }
  L.total = off;
  return true;
}
}  // namespace

}  // namespace aj

using namespace aj;

extern "C" int32_t aj_poisson_mg_static(const AjStepParams* prm, const float* rhs,
                                        const float* mask, float* p_out, AjStats* stats,
                                        void* stream) {
  if (!prm || !rhs || !mask || !p_out) return AJ_ERR_PARAM;
  // the same parameter rules as aj_poisson_mg, in the one mode this entry
  // point runs (the parity solve from a zero guess on the collocated grid)
  AjStepParams p = normalise(*prm);
  p.mg_mode = AJ_MG_PARITY;
  p.warm_start = AJ_WARM_ZERO;
  int rc = check_params(p);
  if (rc != AJ_OK) return rc;                                           // multigrid_solver.py:104-106
  if (p.grid_type != AJ_GRID_COLLOCATED || p.flow_type != AJ_FLOW_VON_KARMAN) return AJ_ERR_PARAM;
  if ((long)p.nx * p.ny > AJ_STATIC_MAX_CELLS) return AJ_ERR_WORKSPACE;   // above the stated limit
  Layout L;
  if (!static_layout(p, L)) return AJ_ERR_SHAPE;
  if (L.total > kStaticScratchBytes) return AJ_ERR_WORKSPACE;
  // the array used is the current device's: the stream and the buffers must
  // belong to that device
  int dev = -1, sdev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return AJ_ERR_CUDA;
  cudaStream_t st = (cudaStream_t)stream;
  if (st && cudaStreamGetDevice(st, &sdev) == cudaSuccess && sdev != dev) return AJ_ERR_PARAM;
  cudaGetLastError();
  for (const void* ptr : {(const void*)rhs, (const void*)mask, (const void*)p_out}) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, ptr) != cudaSuccess) {
      cudaGetLastError();
      return AJ_ERR_PARAM;
    }
    if (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged) return AJ_ERR_PARAM;
    if (at.device != dev) return AJ_ERR_PARAM;
  }
  void* ws = nullptr;
  rc = static_scratch_address(&ws);
  if (rc != AJ_OK) return rc;
  // the device scalars must start at zero on every call (the array keeps the
  // previous call's contents); every other region is written before it is read
  if (cudaMemsetAsync(ws, 0, 256, st) != cudaSuccess) return AJ_ERR_CUDA;
  rc = launch_mg_rhs(p, L, ws, rhs, mask, st);
  if (rc != AJ_OK) return rc;
  return launch_pressure(p, L, ws, mask, nullptr, p_out, stats, st);
}
