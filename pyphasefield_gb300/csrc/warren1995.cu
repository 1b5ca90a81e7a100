// Warren-Boettinger (1995) binary-alloy solidification step on one grid.
//
// Grid of warps: warp (strip s, band b) updates columns 30s .. 30s+29 of rows
// ROWS*b .. ROWS*b+ROWS-1 with the band update of w95_core.cuh (phi and c
// read once from global memory, L2-resident at the benchmark size, ghost
// rule applied at load time; pointwise D_C and temp once per cell; full
// anisotropic phi update with noise, non-flux-form solute update). One read
// and one write of each field per step.
//
// Reference: engine_Warren1995 (Engines/Warren1995.py:50-92).
#include <cmath>
#include <type_traits>

#include "ppf_common.cuh"
#include "w95_core.cuh"

namespace ppf {
namespace {

constexpr int kWarpsPerCta = 4;
constexpr int kCtaThreads = 32 * kWarpsPerCta;

// The generic band kernel (float64, and float with 4 / 8 / 16 rows) takes
// the registers it needs; the float two-row kernel below asks for ten
// 128-thread CTAs per SM (48 registers a thread).
template <typename T, int ROWS>
__global__ void __launch_bounds__(kCtaThreads)
    warren1995_kernel(w95::Coef<T> k, Geo g, Bc<T> bc, const T* __restrict__ phi_in,
                      const T* __restrict__ c_in, T* __restrict__ phi_out,
                      T* __restrict__ c_out, uint64_t seed, uint64_t step,
                      const uint64_t* __restrict__ step_base) {
  const int y0 = (blockIdx.y * kWarpsPerCta + threadIdx.y) * ROWS;
  if (y0 >= g.n[0]) return;  // whole warp: no shuffles are left pending
  pdl_wait();
  pdl_launch_next();
  if (step_base) step += *step_base;
  w95::band<T, ROWS>(k, g, bc, phi_in, c_in, phi_out, c_out, seed, step,
                     blockIdx.x * w95::kStrip - 1, y0);
}

// The benchmark's instantiation (float, two rows per warp). The CTA's four
// warps own four consecutive bands of one strip (a group of eight rows). The
// Philox blocks of the group's rows (4 bands x 2 rows x kGroups = 64 blocks)
// are drawn by two warps, one block per lane, before the bands' loads, into a
// shared-memory table that every band reads its words from,
// instead of each warp drawing its own 16 blocks with half its lanes idle and
// fetching words by shuffles.
constexpr int kTableJobs = kWarpsPerCta * 2 * w95::kGroups;
static_assert(kTableJobs == 64, "two warps draw a group's noise blocks");

__global__ void __launch_bounds__(kCtaThreads, 10)
    warren1995_f2_kernel(w95::Coef<float> k, Geo g, Bc<float> bc,
                         const float* __restrict__ phi_in, const float* __restrict__ c_in,
                         float* __restrict__ phi_out, float* __restrict__ c_out, uint64_t seed,
                         uint64_t step, const uint64_t* __restrict__ step_base) {
  __shared__ U4 table[kTableJobs];
  const int w = threadIdx.y, lane = threadIdx.x;
  const int band0 = blockIdx.y * (kWarpsPerCta * 2);  // first row of the group
  const int y0 = band0 + 2 * w;
  const int xs = blockIdx.x * w95::kStrip - 1;
  const uint32_t gbase = (uint32_t)(xs + 1) / 4u;  // first owned column's Philox block
  // The noise blocks depend on the step and indices only, not on the fields,
  // so they are drawn before waiting on the previous step (with programmatic
  // dependent launch, during its tail). The step offset *step_base is written
  // only between graph replays (ppf_counter_add_u64), never by the previous
  // step of the same replay.
  if (step_base) step += *step_base;
  if (k.alpha != 0.f && w < 2) {
    const int job = w * 32 + lane;  // (band b, row r, block i)
    const int b = job / (2 * w95::kGroups), r = (job / w95::kGroups) & 1;
    const int i = job % w95::kGroups;
    table[job] = noise_group(seed, step, (uint32_t)(band0 + 2 * b + r), gbase + (uint32_t)i);
  }
  pdl_wait();
  pdl_launch_next();
  const bool live = y0 < g.n[0];  // warp-uniform; dead warps still meet the barrier
  float bp[4], bcv[4], v = 0.f;
  if (live) w95::band_load<float, 2>(g, bc, phi_in, c_in, xs, y0, bp, bcv);
  __syncthreads();
  if (!live) return;
  if (k.bulk && w95::band_is_bulk(bp, v)) {
    w95::band_bulk_pk<1>(k, g, phi_out, c_out, xs, y0, bp, bcv, v);
    return;
  }
  w95::TableNoise noise{reinterpret_cast<const uint32_t*>(table + w * 2 * w95::kGroups), gbase};
  w95::band_full_pk<1>(k, g, phi_out, c_out, noise, xs, y0, bp, bcv);
}

template <typename T, int ROWS>
cudaError_t launch_rows(const w95::Coef<T>& k, const Geo& g, const Bc<T>& bc, const T* phi_in,
                        const T* c_in, T* phi_out, T* c_out, uint64_t seed, uint64_t step,
                        const uint64_t* step_base, bool pdl, cudaStream_t s) {
  const long strips = (g.n[1] + w95::kStrip - 1) / w95::kStrip;
  const long bands = (g.n[0] + ROWS - 1) / ROWS;
  const long gy = (bands + kWarpsPerCta - 1) / kWarpsPerCta;
  if (strips > (1L << 30) || gy > 65535) return cudaErrorInvalidConfiguration;
  if constexpr (std::is_same<T, float>::value && ROWS == 2)
    return launch(warren1995_f2_kernel, dim3((unsigned)strips, (unsigned)gy),
                  dim3(32, kWarpsPerCta), 0, s, pdl, k, g, bc, phi_in, c_in, phi_out, c_out,
                  seed, step, step_base);
  else
    return launch(warren1995_kernel<T, ROWS>, dim3((unsigned)strips, (unsigned)gy),
                  dim3(32, kWarpsPerCta), 0, s, pdl, k, g, bc, phi_in, c_in, phi_out, c_out,
                  seed, step, step_base);
}

template <typename T>
int32_t warren1995(const PpfWarren1995Params* p, const PpfGrid* grid, const PpfBoundary* b,
                   const T* phi_in, const T* c_in, T* phi_out, T* c_out, uint64_t seed,
                   uint64_t step, const uint64_t* step_base, const PpfTiling* tiling,
                   void* stream) {
  clear_error();
  if (!p) return fail(PPF_ERR_INVALID, "params is NULL");
  if (!(p->dx > 0) || !(p->T > 0) || !(p->T_mA > 0) || !(p->T_mB > 0) || !(p->R > 0))
    return fail(PPF_ERR_INVALID, "dx, T, T_mA, T_mB and R must be > 0");
  Geo g;
  int32_t rc = make_geo(grid, 2, 2, &g);
  if (rc) return rc;
  if (!phi_in || !c_in || !phi_out || !c_out) return fail(PPF_ERR_INVALID, "NULL field pointer");
  if (phi_in == phi_out || c_in == c_out || phi_in == c_out || c_in == phi_out ||
      phi_out == c_out)
    return fail(PPF_ERR_INVALID, "input and output fields must be distinct");
  if (tiling && tiling->depth > 1)
    return fail(PPF_ERR_UNSUPPORTED, "Warren1995 advances one step per pass");
  Bc<T> bc;
  if ((rc = make_bc<T>(b, g, p->dx, 2, 1, &bc))) return rc;
  if (tiling && tiling->tile_x && tiling->tile_x != w95::kStrip)
    return fail(PPF_ERR_UNSUPPORTED, "Warren1995 warps own %d columns", w95::kStrip);
  const int rows = tiling && tiling->tile_y ? tiling->tile_y : 2;
  const w95::Coef<T> k = w95::fold<T>(*p, !(tiling && (tiling->flags & PPF_TILING_FULL_EVAL)));

  const bool pdl = tiling && tiling->pdl;
  const cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e;
  switch (rows) {
    case 2: e = launch_rows<T, 2>(k, g, bc, phi_in, c_in, phi_out, c_out, seed, step, step_base, pdl, s); break;
    case 4: e = launch_rows<T, 4>(k, g, bc, phi_in, c_in, phi_out, c_out, seed, step, step_base, pdl, s); break;
    case 8: e = launch_rows<T, 8>(k, g, bc, phi_in, c_in, phi_out, c_out, seed, step, step_base, pdl, s); break;
    case 16: e = launch_rows<T, 16>(k, g, bc, phi_in, c_in, phi_out, c_out, seed, step, step_base, pdl, s); break;
    default: return fail(PPF_ERR_INVALID, "Warren1995 rows per warp must be 2, 4, 8 or 16");
  }
  if (e != cudaSuccess) return fail(PPF_ERR_CUDA, "warren1995 launch: %s", cudaGetErrorString(e));
  return PPF_OK;
}

}  // namespace
}  // namespace ppf

using namespace ppf;

extern "C" {

int32_t ppf_warren1995_step_f32(const PpfWarren1995Params* p, const PpfGrid* g,
                                const PpfBoundary* bc, const float* phi_in, const float* c_in,
                                float* phi_out, float* c_out, uint64_t seed, uint64_t step,
                                const uint64_t* step_base, const PpfTiling* tiling,
                                void* stream) {
  return warren1995<float>(p, g, bc, phi_in, c_in, phi_out, c_out, seed, step, step_base,
                           tiling, stream);
}
int32_t ppf_warren1995_step_f64(const PpfWarren1995Params* p, const PpfGrid* g,
                                const PpfBoundary* bc, const double* phi_in, const double* c_in,
                                double* phi_out, double* c_out, uint64_t seed, uint64_t step,
                                const uint64_t* step_base, const PpfTiling* tiling,
                                void* stream) {
  return warren1995<double>(p, g, bc, phi_in, c_in, phi_out, c_out, seed, step, step_base,
                            tiling, stream);
}

}  // extern "C"
