// Triangle counting that allocates nothing: xgm_tc_solver_static.
//
// Some callers cannot allocate device memory at the moment they count: code inside a
// host framework that owns all device memory through its own allocator (a second
// allocator would fight it for the same HBM), or a hot loop whose latency budget has
// no room for a cudaMalloc and the device-wide synchronisation it can bring.  This
// entry point serves them.  It runs the same persistent counting kernel as
// xgm_tc_solver, but its task lists, list sizes, queue heads and result live in one
// file-scope device array of fixed size instead of memory the engine allocates per
// call.  The graph itself (built earlier through xgm_graph_*) and the host result are
// the caller's input and output.
//
// The array is kStaticBytes (48 MiB) and holds the task lists of graphs of up to
// kStaticMaxVertices (2^21) vertices; larger graphs are rejected with
// XGM_ERR_UNSUPPORTED.  Every GPU that loads the library keeps the array until the
// process exits.  All calls share it and it keeps the last call's contents, so each
// call clears its scalars first, and calls whose GPU work overlaps (two streams, two
// threads) race and must be serialised by the caller.  The first call on a device
// does the set-up: it looks up the array's device address (cudaGetSymbolAddress)
// with that device current; make that first call before any stream capture.  The
// call waits for its stream to finish and returns the count; the caller's current
// device is left as it was.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "api_internal.h"

namespace xgm {

namespace {

constexpr int64_t kStaticMaxVertices = int64_t(1) << 21;
constexpr size_t kStaticBytes = size_t(48) << 20;

// Layout inside the array (bytes, 256-aligned pieces):
//   [0, 256)              scalars: count, err, queue heads, counters, list sizes
//   cta   int32[maxV]     CTA vertex tasks
//   warp  int32[maxV]     warp vertex tasks
//   hubs  int32[maxV]     hub vertices
//   off   int64[maxV+1]   hub sub-task offsets
struct StaticScalars {
  unsigned long long count;
  uint32_t err;
  uint32_t pad;
  QueueHeads q;
  unsigned long long n_cta, n_warp;
  unsigned long long hub_packed;  // (hubs << 40) | sub-tasks, one atomic for both
  int64_t n[8];                   // TaskLists sizes (no wide-warp, search or bucket list here)
};
static_assert(sizeof(StaticScalars) <= 256, "scalars fit the first 256 bytes");
constexpr size_t kOffCtaL = 256;
constexpr size_t kOffWarpL = kOffCtaL + 4 * kStaticMaxVertices;
constexpr size_t kOffHubL = kOffWarpL + 4 * kStaticMaxVertices;
constexpr size_t kOffHubOff = kOffHubL + 4 * kStaticMaxVertices;
constexpr size_t kStaticUsed = kOffHubOff + 8 * (kStaticMaxVertices + 1);
static_assert(kStaticUsed <= kStaticBytes, "layout fits the array");

static __device__ __align__(256) unsigned char g_tc_scratch[kStaticBytes];

// Unordered compaction by atomics (counts do not depend on task order).  Hubs take
// their list slot and sub-task offset from one 64-bit atomic, so offsets increase with
// the slot as the kernel's binary search over them requires.
__global__ void k_static_classify(const longlong2* dptr, int64_t nv, StaticScalars* sc,
                                  int32_t* cta, int32_t* warp, int32_t* hubs, int64_t* off) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nv;
       r += (int64_t)gridDim.x * blockDim.x) {
    const longlong2 d = dptr[r];
    const long long s = d.y - d.x;
    if (s < 2) continue;
    if (s <= kWarpCap) {
      warp[atomicAdd(&sc->n_warp, 1ull)] = (int32_t)r;
    } else if (s <= kCtaCap) {
      cta[atomicAdd(&sc->n_cta, 1ull)] = (int32_t)r;
    } else {
      const unsigned long long p = atomicAdd(&sc->hub_packed, (1ull << 40) | (unsigned long long)s);
      const long long slot = (long long)(p >> 40);
      hubs[slot] = (int32_t)r;
      off[slot] = (long long)(p & ((1ull << 40) - 1));
    }
  }
}

__global__ void k_static_sizes(StaticScalars* sc, int64_t* off) {
  const long long hubs = (long long)(sc->hub_packed >> 40);
  const long long sub = (long long)(sc->hub_packed & ((1ull << 40) - 1));
  sc->n[0] = sub;
  sc->n[1] = (int64_t)sc->n_cta;
  sc->n[2] = (int64_t)sc->n_warp;
  sc->n[3] = hubs;
  sc->n[4] = 0;
  sc->n[5] = 0;
  sc->n[6] = 0;
  sc->n[7] = 0;
  off[hubs] = sub;
}

struct StaticState {
  std::mutex mu;
  void* addr[64] = {};
};
StaticState g_state;

// Device address of the array on the current device; looked up once per device.
xgm_status static_scratch(int device, unsigned char** out) {
  if (device < 0 || device >= 64) return XGM_ERR_INVALID;
  std::lock_guard<std::mutex> lock(g_state.mu);
  if (!g_state.addr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_tc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_tc_scratch)", __FILE__, __LINE__);
    g_state.addr[device] = p;
  }
  *out = static_cast<unsigned char*>(g_state.addr[device]);
  return XGM_OK;
}

}  // namespace

}  // namespace xgm

using namespace xgm;

namespace {

xgm_status tc_static(xgm_ctx* ctx, const xgm_graph* g, uint64_t* total);

// Makes ctx's device current for the call and puts the caller's device back after it.
struct DeviceScope {
  int prev = -1;
  cudaError_t enter(int device) {
    cudaError_t e = cudaGetDevice(&prev);
    if (e != cudaSuccess) { prev = -1; return e; }
    return prev == device ? cudaSuccess : cudaSetDevice(device);
  }
  ~DeviceScope() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

}  // namespace

extern "C" xgm_status xgm_tc_solver_static(xgm_ctx* ctx, const xgm_graph* g, uint64_t* total) {
  if (!ctx || !g || !total) return XGM_ERR_INVALID;
  if (g->ctx != ctx) {
    set_thread_error("xgm_tc_solver_static: the graph belongs to another context");
    return finish_status(ctx, XGM_ERR_INVALID);
  }
  if (g->g.nv > kStaticMaxVertices) {
    set_thread_error("xgm_tc_solver_static holds graphs of up to 2^21 vertices (48 MiB "
                     "static scratch); use xgm_tc_solver for larger graphs");
    return finish_status(ctx, XGM_ERR_UNSUPPORTED);
  }
  DeviceScope scope;
  const cudaError_t e = scope.enter(ctx->device);
  if (e != cudaSuccess) return finish_status(ctx, cuda_fail(e, "cudaSetDevice", __FILE__, __LINE__));
  return tc_static(ctx, g, total);
}

namespace {

xgm_status tc_static(xgm_ctx* ctx, const xgm_graph* g, uint64_t* total) {
  const DevGraph& G = g->g;
  unsigned char* base = nullptr;
  xgm_status st = static_scratch(ctx->device, &base);
  if (st != XGM_OK) return finish_status(ctx, st);
  cudaStream_t s = ctx->stream;
  StaticScalars* sc = reinterpret_cast<StaticScalars*>(base);
  int32_t* cta = reinterpret_cast<int32_t*>(base + kOffCtaL);
  int32_t* warp = reinterpret_cast<int32_t*>(base + kOffWarpL);
  int32_t* hubs = reinterpret_cast<int32_t*>(base + kOffHubL);
  int64_t* off = reinterpret_cast<int64_t*>(base + kOffHubOff);
  XGM_CUDA_TRY(cudaMemsetAsync(sc, 0, sizeof(StaticScalars), s));
  if (G.nv > 0) {
    int64_t blocks = (G.nv + 255) / 256;
    if (blocks > 65536) blocks = 65536;
    k_static_classify<<<(unsigned)blocks, 256, 0, s>>>(G.dptr, G.nv, sc, cta, warp, hubs, off);
    XGM_CUDA_TRY(cudaGetLastError());
  }
  k_static_sizes<<<1, 1, 0, s>>>(sc, off);
  XGM_CUDA_TRY(cudaGetLastError());
  TaskLists t;
  t.cta = cta;
  t.warp = warp;
  t.split_v = hubs;
  t.split_off = off;
  t.n = sc->n;
  XGM_CUDA_TRY(launch_clique(3, G.view(), t, &sc->q, &sc->count, &sc->err,
                             ensure_clique_grid(ctx), s));
  StaticScalars h;
  XGM_CUDA_TRY(cudaMemcpyAsync(&h, sc, sizeof(h), cudaMemcpyDeviceToHost, s));
  XGM_CUDA_TRY(cudaStreamSynchronize(s));
  st = check_device_flag(ctx, h.err);
  if (st != XGM_OK) return st;
  *total = h.count;
  return XGM_OK;
}

}  // namespace
