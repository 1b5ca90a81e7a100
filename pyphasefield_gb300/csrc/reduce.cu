// FP64 diagnostics over FP32/FP64 fields: total mass, free energy and a
// finite check. Two passes with a fixed reduction order (deterministic):
// pass 1 gives each CTA a contiguous range of rows and reduces it with warp
// shuffles into one double in caller-provided scratch; pass 2 sums the
// partials in one CTA. The reference has no diagnostics; these are the
// conservation and energy sums the precision split keeps in double.
#include <type_traits>

#include "ppf_common.cuh"

namespace ppf {

constexpr int kRedThreads = 256;
constexpr int kMaxPartials = 1024;

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double red[kRedThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double r = 0.0;
  if (warp == 0) {
    r = lane < kRedThreads / 32 ? red[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
  }
  return r;  // valid in thread 0
}

// Number of pass-1 CTAs for a grid with `rows` rows (rows = all axes but
// the last, multiplied).
int reduce_blocks(int64_t rows) {
  return (int)(rows < kMaxPartials ? rows : kMaxPartials);
}

struct SumOp {};
struct EnergyOp {};

template <typename T>
struct EnergyCoef {
  double w, half_kappa_over_dx2;
};

// Per-cell term. SumOp: x. EnergyOp: w f(x) + kappa/2 |forward diff / dx|^2.
template <typename T>
__device__ __forceinline__ double cell_term(SumOp, const T* __restrict__ x,
                                            const Geo&, const Bc<T>&,
                                            const EnergyCoef<T>&, int, int,
                                            int, T v) {
  return (double)v;
}
template <typename T>
__device__ __forceinline__ double cell_term(EnergyOp, const T* __restrict__ x,
                                            const Geo& g, const Bc<T>& bc,
                                            const EnergyCoef<T>& k, int i0,
                                            int i1, int i2, T v) {
  const double d = (double)v;
  const double f = d * d * (1.0 - d) * (1.0 - d);
  double grad2 = 0.0;
  if (g.ndim == 2) {
    const double a = (double)fetch<T, 2>(x, g, bc, 0, i0 + 1, i1) - d;
    const double b = (double)fetch<T, 2>(x, g, bc, 0, i0, i1 + 1) - d;
    grad2 = a * a + b * b;
  } else {
    const double a = (double)fetch<T, 3>(x, g, bc, 0, i0 + 1, i1, i2) - d;
    const double b = (double)fetch<T, 3>(x, g, bc, 0, i0, i1 + 1, i2) - d;
    const double c = (double)fetch<T, 3>(x, g, bc, 0, i0, i1, i2 + 1) - d;
    grad2 = a * a + b * b + c * c;
  }
  return k.w * f + k.half_kappa_over_dx2 * grad2;
}

// Float sums: each thread carries its running sum as an unevaluated pair of
// floats (s, c), updated with Knuth's TwoSum (six FP32 additions, exact:
// s + x = t + e with t = fl(s + x)), and turns it into a double once at the
// end. The pair holds the thread's partial sum to about 2^-48 relative, as
// a double accumulator would, without an FP64 operation per element (the
// GB300's FP64 rate bounded the double accumulation at 0.14 of the copy
// peak).
struct Pair {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float t = s + x;
    const float z = t - s;
    const float e = (s - (t - z)) + (x - z);
    s = t;
    c += e;
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

template <typename T, typename Op>
__global__ void __launch_bounds__(kRedThreads)
    reduce_pass1(Op op, const T* __restrict__ x, Geo g, Bc<T> bc,
                 EnergyCoef<T> k, double* __restrict__ partial) {
  pdl_wait();
  constexpr bool kPair = std::is_same<T, float>::value && std::is_same<Op, SumOp>::value;
  const int nx = g.n[g.ndim - 1];
  const int64_t rows = g.ndim == 2 ? (int64_t)g.n[0] : (int64_t)g.n[0] * g.n[1];
  const int64_t r0 = rows * blockIdx.x / gridDim.x;
  const int64_t r1 = rows * (blockIdx.x + 1) / gridDim.x;
  double acc = 0.0;
  Pair pacc;
  for (int64_t r = r0; r < r1; ++r) {
    int i0, i1;
    int64_t off;
    if (g.ndim == 2) {
      i0 = (int)r;
      i1 = 0;
      off = r * g.pitch;
    } else {
      i0 = (int)(r / g.n[1]);
      i1 = (int)(r - (int64_t)i0 * g.n[1]);
      off = (int64_t)i0 * g.plane + (int64_t)i1 * g.pitch;
    }
    for (int c = threadIdx.x; c < nx; c += kRedThreads) {
      const T v = x[off + c];
      if constexpr (kPair)
        pacc.add(v);
      else
        acc += g.ndim == 2 ? cell_term<T>(op, x, g, bc, k, i0, c, 0, v)
                           : cell_term<T>(op, x, g, bc, k, i0, i1, c, v);
    }
  }
  if constexpr (kPair) acc = pacc.value();
  const double s = block_sum(acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kRedThreads)
    reduce_pass2(const double* __restrict__ partial, int n, double scale,
                 double* __restrict__ out) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += kRedThreads) acc += partial[i];
  const double s = block_sum(acc);
  if (threadIdx.x == 0) out[0] = s * scale;
}

template <typename T>
__global__ void __launch_bounds__(kRedThreads)
    finite_kernel(const T* __restrict__ x, Geo g, int* __restrict__ status) {
  pdl_wait();
  const int nx = g.n[g.ndim - 1];
  const int64_t rows = g.ndim == 2 ? (int64_t)g.n[0] : (int64_t)g.n[0] * g.n[1];
  int bad = 0;
  for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
    int64_t off;
    if (g.ndim == 2) {
      off = r * g.pitch;
    } else {
      const int64_t i0 = r / g.n[1];
      off = i0 * g.plane + (r - i0 * g.n[1]) * g.pitch;
    }
    for (int c = threadIdx.x; c < nx; c += kRedThreads) bad |= !isfinite(x[off + c]);
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(status, PPF_STATUS_NONFINITE);
}

template <typename T, typename Op>
int32_t reduce_impl(Op op, const T* x, const PpfGrid* grid, const PpfBoundary* b,
                    double dx, double w, double kappa, double scale_pow_dx,
                    double* out, void* scratch, size_t scratch_bytes,
                    void* stream) {
  Geo g;
  int32_t rc = make_geo(grid, 2, 3, &g);
  if (rc) return rc;
  if (!x || !out) return fail(PPF_ERR_INVALID, "NULL pointer");
  const int64_t rows = g.ndim == 2 ? (int64_t)g.n[0] : (int64_t)g.n[0] * g.n[1];
  const int nb = reduce_blocks(rows);
  if (!scratch || scratch_bytes < (size_t)nb * sizeof(double))
    return fail(PPF_ERR_INVALID, "scratch needs %zu bytes, got %zu",
                (size_t)nb * sizeof(double), scratch_bytes);
  if (((uintptr_t)scratch) % 8 != 0)
    return fail(PPF_ERR_INVALID, "scratch must be 8-byte aligned");
  Bc<T> bc{};
  if (b) {
    if ((rc = make_bc<T>(b, g, dx, 1, 1, &bc))) return rc;
  }
  EnergyCoef<T> k{w, 0.5 * kappa / (dx * dx)};
  double scale = 1.0;
  for (int a = 0; a < g.ndim; ++a) scale *= scale_pow_dx;
  cudaStream_t s = (cudaStream_t)stream;
  reduce_pass1<T, Op><<<nb, kRedThreads, 0, s>>>(op, x, g, bc, k, (double*)scratch);
  PPF_TRY_CUDA(cudaGetLastError());
  reduce_pass2<<<1, kRedThreads, 0, s>>>((const double*)scratch, nb, scale, out);
  PPF_TRY_CUDA(cudaGetLastError());
  return PPF_OK;
}

// ------------------------------------------------------------ allocation-free sum
// Scratch of ppf_reduce_sum_f32_noalloc: the per-CTA partial sums of pass 1
// live in this fixed device array instead of caller-provided memory. Every
// GPU that loads the library holds it (8 KiB) until the process exits.
constexpr int kNoAllocPartials = 1024;
static __device__ __align__(256) double g_noalloc_partials[kNoAllocPartials];

// Device address of g_noalloc_partials on the current device. Host code must
// not pass the symbol itself to a kernel (on the host it names a stand-in,
// not device memory), so the address is looked up with the device current,
// here in the file that defines the array, and cached per device and
// context (SymbolCache: safe for concurrent host threads, looked up afresh
// after a context reset).
static int32_t noalloc_partials(double** out) {
  static SymbolCache cache;
  void* p = nullptr;
  const int32_t rc = symbol_address(g_noalloc_partials, cache, &p);
  if (rc) return rc;
  *out = static_cast<double*>(p);
  return PPF_OK;
}

template <typename T>
int32_t check_finite(const T* x, const PpfGrid* grid, int32_t* status, void* stream) {
  clear_error();
  Geo g;
  int32_t rc = make_geo(grid, 2, 3, &g);
  if (rc) return rc;
  if (!x || !status) return fail(PPF_ERR_INVALID, "NULL pointer");
  finite_kernel<T><<<152 * 4, kRedThreads, 0, (cudaStream_t)stream>>>(x, g, (int*)status);
  PPF_TRY_CUDA(cudaGetLastError());
  return PPF_OK;
}

}  // namespace ppf

using namespace ppf;

extern "C" {

int32_t ppf_reduce_sum_f32_noalloc(const float* x, const PpfGrid* grid, double* out,
                                   void* stream) {
  clear_error();
  Geo g;
  int32_t rc = make_geo(grid, 2, 3, &g);
  if (rc) return rc;
  if (!x || !out) return fail(PPF_ERR_INVALID, "NULL pointer");
  const int64_t rows = g.ndim == 2 ? (int64_t)g.n[0] : (int64_t)g.n[0] * g.n[1];
  const int nb = reduce_blocks(rows);
  if (nb > kNoAllocPartials)
    return fail(PPF_ERR_INVALID,
                "grid needs %d partial sums; the allocation-free sum holds at most %d", nb,
                kNoAllocPartials);
  double* partials = nullptr;
  if ((rc = noalloc_partials(&partials))) return rc;
  Bc<float> bc{};
  EnergyCoef<float> k{0.0, 0.0};
  cudaStream_t s = (cudaStream_t)stream;
  reduce_pass1<float, SumOp><<<nb, kRedThreads, 0, s>>>(SumOp{}, x, g, bc, k, partials);
  PPF_TRY_CUDA(cudaGetLastError());
  reduce_pass2<<<1, kRedThreads, 0, s>>>(partials, nb, 1.0, out);
  PPF_TRY_CUDA(cudaGetLastError());
  return PPF_OK;
}

int32_t ppf_reduce_scratch_bytes(const PpfGrid* grid, size_t* bytes) {
  clear_error();
  Geo g;
  int32_t rc = make_geo(grid, 2, 3, &g);
  if (rc) return rc;
  if (!bytes) return fail(PPF_ERR_INVALID, "bytes is NULL");
  const int64_t rows = g.ndim == 2 ? (int64_t)g.n[0] : (int64_t)g.n[0] * g.n[1];
  *bytes = (size_t)reduce_blocks(rows) * sizeof(double);
  return PPF_OK;
}

int32_t ppf_reduce_sum_f32(const float* x, const PpfGrid* g, double* out,
                           void* scratch, size_t scratch_bytes, void* stream) {
  clear_error();
  return reduce_impl<float>(SumOp{}, x, g, nullptr, 1.0, 0.0, 0.0, 1.0, out,
                            scratch, scratch_bytes, stream);
}
int32_t ppf_reduce_sum_f64(const double* x, const PpfGrid* g, double* out,
                           void* scratch, size_t scratch_bytes, void* stream) {
  clear_error();
  return reduce_impl<double>(SumOp{}, x, g, nullptr, 1.0, 0.0, 0.0, 1.0, out,
                             scratch, scratch_bytes, stream);
}

int32_t ppf_free_energy_f32(const float* x, const PpfGrid* g,
                            const PpfBoundary* bc, double dx, double w,
                            double kappa, double* out, void* scratch,
                            size_t scratch_bytes, void* stream) {
  clear_error();
  if (!bc) return fail(PPF_ERR_INVALID, "boundary is NULL");
  if (!(dx > 0)) return fail(PPF_ERR_INVALID, "dx must be > 0");
  return reduce_impl<float>(EnergyOp{}, x, g, bc, dx, w, kappa, dx, out, scratch,
                            scratch_bytes, stream);
}
int32_t ppf_free_energy_f64(const double* x, const PpfGrid* g,
                            const PpfBoundary* bc, double dx, double w,
                            double kappa, double* out, void* scratch,
                            size_t scratch_bytes, void* stream) {
  clear_error();
  if (!bc) return fail(PPF_ERR_INVALID, "boundary is NULL");
  if (!(dx > 0)) return fail(PPF_ERR_INVALID, "dx must be > 0");
  return reduce_impl<double>(EnergyOp{}, x, g, bc, dx, w, kappa, dx, out, scratch,
                             scratch_bytes, stream);
}

int32_t ppf_check_finite_f32(const float* x, const PpfGrid* grid, int32_t* status,
                             void* stream) {
  return check_finite<float>(x, grid, status, stream);
}
int32_t ppf_check_finite_f64(const double* x, const PpfGrid* grid, int32_t* status,
                             void* stream) {
  return check_finite<double>(x, grid, status, stream);
}

}  // extern "C"
