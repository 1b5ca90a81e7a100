// Shared device/host helpers of libppf_gb300: error reporting, the fused
// ghost-cell rule, launch helpers (programmatic dependent launch) and the
// Philox4x32-10 counter-based generator used for the Warren1995 noise.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "ppf_gb300.h"

namespace ppf {

// ---------------------------------------------------------------- errors
// Records a printf-style message for ppf_last_error() and returns `code`.
int32_t fail(int32_t code, const char* fmt, ...);
// Clears the message at the start of every public entry point.
void clear_error();

#define PPF_TRY_CUDA(expr)                                                  \
  do {                                                                      \
    cudaError_t e_ = (expr);                                                \
    if (e_ != cudaSuccess)                                                  \
      return ::ppf::fail(PPF_ERR_CUDA, "%s: %s (%s:%d)", #expr,             \
                         cudaGetErrorString(e_), __FILE__, __LINE__);       \
  } while (0)

// ---------------------------------------------------------------- geometry
// Device-side view of a PpfGrid: n[] are the axis extents in C order, with
// the 2-D case stored as n[0] = rows, n[1] = columns (n[2] unused).
struct Geo {
  int n[3];
  int64_t pitch;  // elements between rows
  int64_t plane;  // elements between planes (3-D)
  int ndim;
};

// Device-side ghost rule: `shift` holds, per field/axis/side, the additive
// Neumann term (-dx*b on the low side, +dx*b on the high side,
// simulation.py:583-584) or the Dirichlet ghost value (simulation.py:591).
template <typename T>
struct Bc {
  int type[3];
  T shift[2][3][2];
};

// Device address of the library's status word (PPF_STATUS_* bits) on the
// current device; kernels that wait on barriers or check values OR
// their findings into it.
int* status_ptr();

// Identifier of the CUDA context current on this thread (cuCtxGetId: unique
// for the life of the process, so a primary context that was reset and
// re-created gets a new one); 0 when the driver cannot tell.
unsigned long long current_context_id();

// Per-device cache of the device address of one __device__ array. On the
// host a __device__ array's name stands for a host-side stand-in, not for
// device memory, so host code looks the address up (cudaGetSymbolAddress)
// with the device current and hands it to kernels. Entries are keyed by
// device and by context id, so a context reset leads to a fresh lookup;
// the mutex makes concurrent host threads safe.
struct SymbolCache {
  static constexpr int kMaxDevices = 64;
  std::mutex m;
  void* addr[kMaxDevices] = {};
  unsigned long long ctx[kMaxDevices] = {};
};

// Looks up `sym` through `cache` for the current device; the lookup is
// compiled into the translation unit that names the symbol.
template <typename S>
inline int32_t symbol_address(const S& sym, SymbolCache& cache, void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(PPF_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= SymbolCache::kMaxDevices)
    return fail(PPF_ERR_UNSUPPORTED, "device %d out of range", dev);
  const unsigned long long ctx = current_context_id();
  std::lock_guard<std::mutex> lock(cache.m);
  if (!cache.addr[dev] || cache.ctx[dev] != ctx) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, sym);
    if (e != cudaSuccess)
      return fail(PPF_ERR_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    cache.addr[dev] = p;
    cache.ctx[dev] = ctx;
  }
  *out = cache.addr[dev];
  return PPF_OK;
}

// Validates a PpfGrid and fills a Geo. Returns PPF_OK or an error code.
int32_t make_geo(const PpfGrid* g, int want_ndim_min, int want_ndim_max,
                 Geo* out);
// Validates a PpfBoundary and converts it for the device. `max_depth` is the
// halo depth the kernel will read; non-zero Neumann gradients are only exact
// at depth 1 and are rejected beyond it.
template <typename T>
int32_t make_bc(const PpfBoundary* b, const Geo& geo, double dx, int nfields,
                int max_depth, Bc<T>* out);

__host__ __device__ __forceinline__ int wrap_index(int i, int n) {
  int m = i % n;
  return m < 0 ? m + n : m;
}
// Reflection about the cell faces: -1 -> 0, -2 -> 1, n -> n-1, ... (period
// 2n so that halos deeper than the grid still land inside it).
__host__ __device__ __forceinline__ int mirror_index(int i, int n) {
  int m = wrap_index(i, 2 * n);
  return m < n ? m : 2 * n - 1 - m;
}

// Value of field `f` at a possibly out-of-range cell, with the reference's
// ghost fill (Simulation.apply_boundary_conditions, simulation.py:560-618,
// slices corrected so every axis is filled) composed in its fill order
// (axis 0 first; a later axis overwrites the corners an earlier one set):
//   PERIODIC  ghost = cell wrapped to the other side
//   NEUMANN   ghost = mirrored edge cell -/+ dx*b
//   DIRCHLET  ghost = value
// Field load: through the read-only (non-coherent) path by default, which
// is valid when the field was written by an earlier kernel; COHERENT = true
// for kernels that read what other CTAs of the same launch wrote before a
// barrier or an arrival flag (ordered by its acquire): cached in L2 only
// (ld.global.cg), so no line this SM's L1 holds from before can be read.
template <bool COHERENT, typename T>
__device__ __forceinline__ T ldf(const T* p) {
  if constexpr (COHERENT)
    return __ldcg(p);
  else
    return __ldg(p);
}

template <typename T, int ND, bool COHERENT = false>
__device__ __forceinline__ T fetch(const T* __restrict__ f, const Geo& g,
                                   const Bc<T>& bc, int fld, int i0, int i1,
                                   int i2 = 0) {
  int idx[3] = {i0, i1, i2};
  bool fixed = false;
  T base = T(0), extra = T(0);
#pragma unroll
  for (int a = 0; a < ND; ++a) {
    const int i = idx[a], n = g.n[a];
    if ((unsigned)i < (unsigned)n) continue;
    const int side = i < 0 ? 0 : 1;
    const int t = bc.type[a];
    if (t == PPF_BC_PERIODIC) {
      idx[a] = wrap_index(i, n);
    } else if (t == PPF_BC_NEUMANN) {
      idx[a] = mirror_index(i, n);
      extra += bc.shift[fld][a][side];
    } else {
      idx[a] = i < 0 ? 0 : n - 1;
      fixed = true;
      base = bc.shift[fld][a][side];
      extra = T(0);
    }
  }
  if (fixed) return base + extra;
  int64_t off;
  if (ND == 2)
    off = (int64_t)idx[0] * g.pitch + idx[1];
  else
    off = (int64_t)idx[0] * g.plane + (int64_t)idx[1] * g.pitch + idx[2];
  return ldf<COHERENT>(f + off) + extra;
}

// fetch's rule for a 2-D cell whose row lies inside the grid, split into a
// per-lane part taken once per column (source column xi; for a ghost
// column the DIRCHLET value or the shift added to the loaded value, each
// formed with the same additions as fetch) and a per-row part (value(f,
// loaded)). A strip that crosses the x edge then loads every row straight
// from one column and fixes its ghost lanes afterwards, instead of a
// divergent fetch per row. Field f of shift: 0 phi, 1 c (as fetch's fld).
template <typename T, int NF>
struct ColumnRule {
  int xi;
  bool ghost, fixed;
  T add[NF];
  __device__ __forceinline__ ColumnRule(const Geo& g, const Bc<T>& bc, int x) {
    const int n = g.n[1];
    xi = x;
    ghost = (unsigned)x >= (unsigned)n;
    fixed = false;
#pragma unroll
    for (int f = 0; f < NF; ++f) add[f] = T(0);
    if (!ghost) return;
    const int side = x < 0 ? 0 : 1;
    const int t = bc.type[1];
    if (t == PPF_BC_PERIODIC) {
      xi = wrap_index(x, n);
    } else if (t == PPF_BC_NEUMANN) {
      xi = mirror_index(x, n);
#pragma unroll
      for (int f = 0; f < NF; ++f) add[f] = T(0) + bc.shift[f][1][side];
    } else {
      xi = x < 0 ? 0 : n - 1;
      fixed = true;
#pragma unroll
      for (int f = 0; f < NF; ++f) add[f] = bc.shift[f][1][side] + T(0);
    }
  }
  __device__ __forceinline__ T value(int f, T loaded) const {
    return !ghost ? loaded : (fixed ? add[f] : loaded + add[f]);
  }
};

// True when the cell lies outside the grid along a DIRCHLET axis: such a
// ghost keeps its fixed value in every sub-step of a temporally blocked tile.
template <typename T, int ND>
__device__ __forceinline__ bool dirichlet_ghost(const Geo& g, const Bc<T>& bc,
                                                int i0, int i1, int i2 = 0) {
  const int idx[3] = {i0, i1, i2};
  bool r = false;
#pragma unroll
  for (int a = 0; a < ND; ++a)
    r |= ((unsigned)idx[a] >= (unsigned)g.n[a]) &&
         (bc.type[a] == PPF_BC_DIRCHLET);
  return r;
}

// ---------------------------------------------------------------- PDL
// Programmatic dependent launch: a kernel waits for its predecessor on the
// stream before touching global memory (reads AND writes: ping-pong buffers
// are written by the next step), and lets its successor launch early.
__device__ __forceinline__ void pdl_wait() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
}
__device__ __forceinline__ void pdl_launch_next() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename... KArgs, typename... Args>
cudaError_t launch(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem,
                   cudaStream_t s, bool pdl, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kern, args...);
}

// Sets the dynamic shared memory limit of `kern` once per process.
template <typename... KArgs>
cudaError_t allow_smem(void (*kern)(KArgs...), size_t bytes) {
  return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)bytes);
}

// ---------------------------------------------------------------- Philox
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11): 10 rounds of two 32x32->64 multiplies with the
// published multipliers and Weyl key increments.
struct U4 {
  uint32_t x, y, z, w;
};
__host__ __device__ __forceinline__ U4 philox4x32_10(U4 ctr, uint32_t k0,
                                                     uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)M0 * ctr.x;
    const uint64_t p1 = (uint64_t)M1 * ctr.z;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    ctr = U4{hi1 ^ ctr.y ^ k0, lo1, hi0 ^ ctr.w ^ k1, lo0};
    k0 += W0;
    k1 += W1;
  }
  return ctr;
}

// Noise words for the group of 4 cells (row gy, columns 4*gq .. 4*gq+3) at
// time step `step`: Philox4x32-10 with counter (gq, gy, step_lo, step_hi) and
// key (seed_lo, seed_hi). Cell (gy, gx) takes word gx & 3; its uniform number
// in [0, 1) is (word >> 8) * 2^-24, exact in float and double, so both
// precisions and the host oracle see the same number.
__host__ __device__ __forceinline__ U4 noise_group(uint64_t seed, uint64_t step,
                                                  uint32_t gy, uint32_t gq) {
  return philox4x32_10(U4{gq, gy, (uint32_t)step, (uint32_t)(step >> 32)},
                       (uint32_t)seed, (uint32_t)(seed >> 32));
}

}  // namespace ppf
