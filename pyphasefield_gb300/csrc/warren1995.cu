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

#include "ppf_common.cuh"
#include "w95_core.cuh"

namespace ppf {
namespace {

constexpr int kWarpsPerCta = 4;
constexpr int kCtaThreads = 32 * kWarpsPerCta;

// Resident CTAs per SM asked of the register allocator: ten 128-thread CTAs
// (48 registers a thread) for the float two-row band, the benchmark's
// kernel; the others take what they need.
template <typename T, int ROWS>
struct W95MinBlocks {
  static constexpr int value = (sizeof(T) == 4 && ROWS == 2) ? 10 : 0;
};

template <typename T, int ROWS>
__global__ void __launch_bounds__(kCtaThreads, (W95MinBlocks<T, ROWS>::value))
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

template <typename T, int ROWS>
cudaError_t launch_rows(const w95::Coef<T>& k, const Geo& g, const Bc<T>& bc, const T* phi_in,
                        const T* c_in, T* phi_out, T* c_out, uint64_t seed, uint64_t step,
                        const uint64_t* step_base, bool pdl, cudaStream_t s) {
  const long strips = (g.n[1] + w95::kStrip - 1) / w95::kStrip;
  const long bands = (g.n[0] + ROWS - 1) / ROWS;
  const long gy = (bands + kWarpsPerCta - 1) / kWarpsPerCta;
  if (strips > (1L << 30) || gy > 65535) return cudaErrorInvalidConfiguration;
  return launch(warren1995_kernel<T, ROWS>, dim3((unsigned)strips, (unsigned)gy),
                dim3(32, kWarpsPerCta), 0, s, pdl, k, g, bc, phi_in, c_in, phi_out, c_out, seed,
                step, step_base);
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
