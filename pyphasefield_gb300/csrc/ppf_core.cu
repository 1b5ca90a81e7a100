// Library plumbing: error strings, argument validation shared by all
// kernels, device queries and the CUDA-graph capture helpers.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <cudaTypedefs.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>

#include "ppf_common.cuh"
#include "ppf_tma.cuh"

namespace ppf {

static thread_local std::string g_last_error;

int32_t fail(int32_t code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

void clear_error() { g_last_error.clear(); }

int32_t make_geo(const PpfGrid* g, int want_ndim_min, int want_ndim_max,
                 Geo* out) {
  if (!g) return fail(PPF_ERR_INVALID, "grid is NULL");
  if (g->reserved != 0) return fail(PPF_ERR_INVALID, "grid.reserved must be 0");
  if (g->ndim < want_ndim_min || g->ndim > want_ndim_max)
    return fail(PPF_ERR_INVALID, "grid.ndim=%d not in [%d, %d]", g->ndim,
                want_ndim_min, want_ndim_max);
  Geo r{};
  r.ndim = g->ndim;
  for (int a = 0; a < g->ndim; ++a) {
    if (g->shape[a] < 1 || g->shape[a] > (int64_t)(1 << 30))
      return fail(PPF_ERR_INVALID, "grid.shape[%d]=%lld out of range", a,
                  (long long)g->shape[a]);
    r.n[a] = (int)g->shape[a];
  }
  for (int a = g->ndim; a < 3; ++a) r.n[a] = 1;
  const int64_t nx = g->shape[g->ndim - 1];
  if (g->pitch < nx || (g->pitch % 4) != 0)
    return fail(PPF_ERR_INVALID,
                "grid.pitch=%lld must be >= %lld and a multiple of 4",
                (long long)g->pitch, (long long)nx);
  r.pitch = g->pitch;
  r.plane = g->ndim == 3 ? g->pitch * g->shape[1] : 0;
  *out = r;
  return PPF_OK;
}

template <typename T>
int32_t make_bc(const PpfBoundary* b, const Geo& geo, double dx, int nfields,
                int max_depth, Bc<T>* out) {
  if (!b) return fail(PPF_ERR_INVALID, "boundary is NULL");
  Bc<T> r{};
  for (int a = 0; a < 3; ++a) {
    const int t = a < geo.ndim ? b->type[a] : PPF_BC_PERIODIC;
    if (t != PPF_BC_PERIODIC && t != PPF_BC_NEUMANN && t != PPF_BC_DIRCHLET)
      return fail(PPF_ERR_INVALID, "boundary.type[%d]=%d unknown", a, t);
    r.type[a] = t;
    for (int f = 0; f < 2; ++f)
      for (int s = 0; s < 2; ++s) {
        const double v = b->value[f][a][s];
        if (!std::isfinite(v))
          return fail(PPF_ERR_INVALID, "boundary value not finite");
        double sh = 0.0;
        if (t == PPF_BC_NEUMANN) {
          sh = (s == 0 ? -dx : dx) * v;
          if (v != 0.0 && f < nfields && max_depth > 1)
            return fail(PPF_ERR_UNSUPPORTED,
                        "non-zero NEUMANN gradient needs halo depth 1 "
                        "(requested %d)",
                        max_depth);
        } else if (t == PPF_BC_DIRCHLET) {
          sh = v;
        }
        r.shift[f][a][s] = (T)sh;
      }
  }
  *out = r;
  return PPF_OK;
}

template int32_t make_bc<float>(const PpfBoundary*, const Geo&, double, int,
                                int, Bc<float>*);
template int32_t make_bc<double>(const PpfBoundary*, const Geo&, double, int,
                                 int, Bc<double>*);

__global__ void counter_add_kernel(uint64_t* c, uint64_t inc) {
  pdl_wait();
  *c += inc;
}

// ------------------------------------------------------------ status word
__device__ int g_status;

unsigned long long current_context_id() {
  using GetCurrent = CUresult (*)(CUcontext*);
  using GetId = CUresult (*)(CUcontext, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = (GetCurrent)p;
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = (GetId)p;
  });
  if (!get_current || !get_id) return 0;
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
  unsigned long long id = 0;
  return get_id(ctx, &id) == CUDA_SUCCESS ? id : 0;
}

int* status_ptr() {
  static SymbolCache cache;
  void* p = nullptr;
  if (symbol_address(g_status, cache, &p) != PPF_OK) return nullptr;
  return (int*)p;
}

// Moves the library's status bits into the caller's word: *dst |= bits,
// library word cleared (stream-ordered, so it can sit in a captured graph).
__global__ void status_collect_kernel(int* lib, int* dst) {
  pdl_wait();
  const int v = atomicExch(lib, 0);
  if (v) atomicOr(dst, v);
}

// Waits on an mbarrier that nothing completes, with a small poll limit, to
// exercise the timeout path: the wait gives up and reports
// PPF_STATUS_TIMEOUT; nothing is left in flight.
__global__ void wait_timeout_kernel(uint32_t limit, int* status) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_init_fence();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (!mbar_wait(&bar, 0, limit)) atomicOr(status, PPF_STATUS_TIMEOUT);
    // complete the phase so the barrier is left quiescent
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(&bar)) : "memory");
  }
}

// ------------------------------------------------------------ tensor maps
namespace {

struct MapKey {
  const void* base;
  int elem, rank, kind;  // kind 0: float / double tiles, 1: bf16 with 128-byte swizzle
  uint64_t dims[3], strides[2];
  uint32_t box[3];
  int device;
  bool operator==(const MapKey& o) const { return std::memcmp(this, &o, sizeof(*this)) == 0; }
};
struct MapKeyHash {
  size_t operator()(const MapKey& k) const {
    const unsigned char* p = reinterpret_cast<const unsigned char*>(&k);
    size_t h = 1469598103934665603ull;
    for (size_t i = 0; i < sizeof(k); ++i) h = (h ^ p[i]) * 1099511628211ull;
    return h;
  }
};

std::mutex g_map_mutex;
std::unordered_map<MapKey, CUtensorMap, MapKeyHash>& map_cache() {
  static std::unordered_map<MapKey, CUtensorMap, MapKeyHash> m;
  return m;
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  }
  return fn;
}

}  // namespace

static int32_t tensor_map_kind(CUtensorMap* out, const void* base, int elem_bytes, int rank,
                               const uint64_t* dims, const uint64_t* strides_bytes,
                               const uint32_t* box, int kind) {
  MapKey key;
  std::memset(&key, 0, sizeof(key));
  key.base = base;
  key.elem = elem_bytes;
  key.rank = rank;
  key.kind = kind;
  for (int i = 0; i < rank; ++i) {
    key.dims[i] = dims[i];
    key.box[i] = box[i];
  }
  for (int i = 0; i + 1 < rank; ++i) key.strides[i] = strides_bytes[i];
  cudaGetDevice(&key.device);
  std::lock_guard<std::mutex> lock(g_map_mutex);
  auto& cache = map_cache();
  auto it = cache.find(key);
  if (it != cache.end()) {
    *out = it->second;
    return PPF_OK;
  }
  auto fn = encode_fn();
  if (!fn) return fail(PPF_ERR_CUDA, "cuTensorMapEncodeTiled unavailable from the driver");
  if (((uintptr_t)base) % 16) return fail(PPF_ERR_INVALID, "field base not 16-byte aligned");
  cuuint32_t estr[3] = {1, 1, 1};
  CUtensorMap m;
  const CUtensorMapDataType dt = kind == 1 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16
                                 : (elem_bytes == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                                    : CU_TENSOR_MAP_DATA_TYPE_FLOAT64);
  CUresult r = fn(&m, dt, (cuuint32_t)rank, const_cast<void*>(base), (const cuuint64_t*)dims,
                  (const cuuint64_t*)strides_bytes, (const cuuint32_t*)box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE,
                  kind == 1 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(PPF_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  if (cache.size() > 4096) cache.clear();
  cache.emplace(key, m);
  *out = m;
  return PPF_OK;
}

int32_t tensor_map(CUtensorMap* out, const void* base, int elem_bytes, int rank,
                   const uint64_t* dims, const uint64_t* strides_bytes, const uint32_t* box) {
  return tensor_map_kind(out, base, elem_bytes, rank, dims, strides_bytes, box, 0);
}

int32_t tensor_map_bf16_sw128(CUtensorMap* out, const void* base, uint64_t cols, uint64_t rows,
                              uint64_t row_bytes, uint32_t box_cols, uint32_t box_rows) {
  if (box_cols * 2 > 128) return fail(PPF_ERR_INVALID, "swizzled box wider than 128 bytes");
  if (row_bytes % 16) return fail(PPF_ERR_INVALID, "row stride not a multiple of 16 bytes");
  const uint64_t dims[2] = {cols, rows};
  const uint64_t strides[1] = {row_bytes};
  const uint32_t box[2] = {box_cols, box_rows};
  return tensor_map_kind(out, base, 2, 2, dims, strides, box, 1);
}

}  // namespace ppf

using namespace ppf;

extern "C" {

int32_t ppf_version(int32_t* abi_version, char* buf, size_t len) {
  clear_error();
  if (abi_version) *abi_version = PPF_ABI_VERSION;
  if (buf && len) {
    snprintf(buf, len, "ppf_gb300 abi=%d cuda=%d sm_103a", PPF_ABI_VERSION,
             CUDART_VERSION);
  }
  return PPF_OK;
}

int32_t ppf_last_error(char* buf, size_t len) {
  if (buf && len) {
    strncpy(buf, g_last_error.c_str(), len - 1);
    buf[len - 1] = 0;
  }
  return PPF_OK;
}

int32_t ppf_device_info(int32_t device, int32_t* sm_count, int32_t* smem_optin,
                        int32_t* cc_major, int32_t* cc_minor) {
  clear_error();
  int v = 0;
  PPF_TRY_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device));
  if (sm_count) *sm_count = v;
  PPF_TRY_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
  if (smem_optin) *smem_optin = v;
  PPF_TRY_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrComputeCapabilityMajor, device));
  if (cc_major) *cc_major = v;
  PPF_TRY_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrComputeCapabilityMinor, device));
  if (cc_minor) *cc_minor = v;
  return PPF_OK;
}

int32_t ppf_counter_add_u64(uint64_t* counter, uint64_t inc, void* stream) {
  clear_error();
  if (!counter) return fail(PPF_ERR_INVALID, "counter is NULL");
  counter_add_kernel<<<1, 1, 0, (cudaStream_t)stream>>>(counter, inc);
  PPF_TRY_CUDA(cudaGetLastError());
  return PPF_OK;
}

int32_t ppf_status_take(int32_t* status) {
  clear_error();
  if (!status) return fail(PPF_ERR_INVALID, "status is NULL");
  int* p = status_ptr();
  if (!p) return fail(PPF_ERR_CUDA, "status word unavailable");
  int v = 0;
  PPF_TRY_CUDA(cudaMemcpy(&v, p, sizeof(int), cudaMemcpyDeviceToHost));
  PPF_TRY_CUDA(cudaMemset(p, 0, sizeof(int)));
  *status = v;
  return PPF_OK;
}

int32_t ppf_status_collect(int32_t* dst, void* stream) {
  clear_error();
  if (!dst) return fail(PPF_ERR_INVALID, "dst is NULL");
  int* p = status_ptr();
  if (!p) return fail(PPF_ERR_CUDA, "status word unavailable");
  status_collect_kernel<<<1, 1, 0, (cudaStream_t)stream>>>(p, (int*)dst);
  PPF_TRY_CUDA(cudaGetLastError());
  return PPF_OK;
}

int32_t ppf_selftest_wait_timeout(int32_t poll_limit, void* stream) {
  clear_error();
  if (poll_limit < 1 || poll_limit > (1 << 20))
    return fail(PPF_ERR_INVALID, "poll_limit must be in [1, 2^20]");
  int* p = status_ptr();
  if (!p) return fail(PPF_ERR_CUDA, "status word unavailable");
  wait_timeout_kernel<<<1, 32, 0, (cudaStream_t)stream>>>((uint32_t)poll_limit, p);
  PPF_TRY_CUDA(cudaGetLastError());
  return PPF_OK;
}

int32_t ppf_graph_begin(void* stream) {
  clear_error();
  if (!stream)
    return fail(PPF_ERR_INVALID, "graph capture needs a non-default stream");
  PPF_TRY_CUDA(cudaStreamBeginCapture((cudaStream_t)stream,
                                      cudaStreamCaptureModeThreadLocal));
  return PPF_OK;
}

int32_t ppf_graph_end(void* stream, void** graph_exec) {
  clear_error();
  if (!graph_exec) return fail(PPF_ERR_INVALID, "graph_exec is NULL");
  cudaGraph_t graph = nullptr;
  PPF_TRY_CUDA(cudaStreamEndCapture((cudaStream_t)stream, &graph));
  cudaGraphExec_t exec = nullptr;
  cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess)
    return fail(PPF_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
  *graph_exec = (void*)exec;
  return PPF_OK;
}

int32_t ppf_graph_launch(void* graph_exec, void* stream) {
  clear_error();
  if (!graph_exec) return fail(PPF_ERR_INVALID, "graph_exec is NULL");
  PPF_TRY_CUDA(cudaGraphLaunch((cudaGraphExec_t)graph_exec, (cudaStream_t)stream));
  return PPF_OK;
}

int32_t ppf_graph_destroy(void* graph_exec) {
  clear_error();
  if (graph_exec) PPF_TRY_CUDA(cudaGraphExecDestroy((cudaGraphExec_t)graph_exec));
  return PPF_OK;
}

}  // extern "C"
