// Warren-Boettinger (1995) binary-alloy solidification step, fused.
//
// Each warp owns a 30-column x ROWS-row block and marches down it; phi and c
// come from global memory (L2-resident at the benchmark size) with the ghost
// rule applied at load time. Per cell it computes the pointwise solute
// diffusivity D_C(phi) and the solute-trapping flux coefficient temp(phi, c)
// once (neighbours get them by shuffles or from the register window), then
// evaluates the full phi and c updates (anisotropic phase-field term, noise,
// non-flux-form solute update) and writes phi' and c'. One read and one write
// of each field per step.
//
// Reference: engine_Warren1995 (Engines/Warren1995.py:50-92), helpers
// _p, _g, _gprime (:17-28) and gradx/grady/gradxx/gradyy (:30-48). Axis 0 of
// the C-order grid is the reference's "x", axis 1 its "y".
#include <cmath>

#include "ppf_common.cuh"

namespace ppf {
namespace {

// Host-folded constants (all differences below are unscaled: the 1/(2dx),
// 1/dx^2 and dt factors are folded in here).
template <typename T>
struct W95Coef {
  T e2;          // ebar^2 / dx^2
  T dtMA, dtMB;  // dt*M_A, dt*M_B
  T WA, WB;      // W_A, W_B
  T hA, hB;      // 30 L (1/T - 1/T_m) for A and B
  T a0, a1;      // dt/dx^2 * D_S, dt/dx^2 * (D_L - D_S)
  T vr;          // v_m / R
  T ye;          // anisotropy strength y_e
  T alpha;       // noise amplitude
  int bulk;      // take the exact reduced form on bulk rows
};

// Pointwise part evaluated on every cell entering the window:
//   Dt = dt/dx^2 * D_C,   D_C = D_S + p(phi) (D_L - D_S)          (:69)
//   Qt = dt/dx^2 * temp,  temp = D_C v_m c (1-c) (H_B - H_A) / R   (:70)
template <typename T>
__device__ __forceinline__ void w95_point(const W95Coef<T>& k, T phi, T c, T& Dt, T& Qt) {
  const T p = phi * phi * phi * (T(10) + phi * (T(-15) + T(6) * phi));
  const T om = T(1) - phi;
  const T g = phi * phi * om * om;
  const T gp = phi * (T(2) + phi * (T(-6) + T(4) * phi));
  Dt = k.a0 + k.a1 * p;
  const T dH = (k.WB - k.WA) * gp + (k.hB - k.hA) * g;
  Qt = Dt * k.vr * c * (T(1) - c) * dH;
}

// Work split: a warp owns a strip of kStrip = 30 output columns (lanes 1..30;
// lanes 0 and 31 carry the west/east halo columns) and a band of ROWS rows.
// It marches down the band keeping the north/centre/south values of its
// column in registers and gets west/east neighbours by warp shuffles: no
// shared memory and no block-wide barriers. The next row's phi and c are
// loaded one row ahead of use.
constexpr int kStrip = 30;
constexpr int kWarpsPerCta = 4;
constexpr int kCtaThreads = 32 * kWarpsPerCta;

__device__ __forceinline__ float inv_norm(float r2) { return rsqrtf(r2); }
__device__ __forceinline__ double inv_norm(double r2) { return rsqrt(r2); }
// Gradients below this are treated as zero (angle 0, as arctan2(0, 0)):
// float cannot represent the direction of a smaller difference of phi.
template <typename T>
__device__ __forceinline__ T tiny_r2();
template <>
__device__ __forceinline__ float tiny_r2<float>() { return 1e-30f; }
template <>
__device__ __forceinline__ double tiny_r2<double>() { return 0.0; }

template <typename T>
__device__ __forceinline__ void load_cell(const T* __restrict__ phi, const T* __restrict__ c,
                                          const Geo& g, const Bc<T>& bc, int row, int x,
                                          bool x_in, T& p, T& cc) {
  if (x_in && (unsigned)row < (unsigned)g.n[0]) {
    const int64_t o = (int64_t)row * g.pitch + x;
    p = __ldg(phi + o);
    cc = __ldg(c + o);
  } else {
    p = fetch<T, 2>(phi, g, bc, 0, row, x);
    cc = fetch<T, 2>(c, g, bc, 1, row, x);
  }
}

template <typename T>
__device__ __forceinline__ T shfl_w(T v) { return __shfl_up_sync(0xffffffffu, v, 1); }
template <typename T>
__device__ __forceinline__ T shfl_e(T v) { return __shfl_down_sync(0xffffffffu, v, 1); }

template <typename T, int ROWS>
__global__ void __launch_bounds__(kCtaThreads)
    warren1995_kernel(W95Coef<T> k, Geo g, Bc<T> bc, const T* __restrict__ phi_in,
                      const T* __restrict__ c_in, T* __restrict__ phi_out,
                      T* __restrict__ c_out, uint64_t seed, uint64_t step,
                      const uint64_t* __restrict__ step_base) {
  const int lane = threadIdx.x, warp = threadIdx.y;
  const int ny = g.n[0], nx = g.n[1];
  const int xs = blockIdx.x * kStrip - 1;  // column of lane 0
  const int x = xs + lane;
  const int y0 = (blockIdx.y * kWarpsPerCta + warp) * ROWS;
  if (y0 >= ny) return;  // whole warp: no shuffles are left pending
  const bool x_in = xs >= 0 && xs + 31 < nx;
  const bool owner = lane >= 1 && lane <= kStrip && x < nx;

  pdl_wait();
  pdl_launch_next();
  if (step_base) step += *step_base;

  // All ROWS + 2 rows of the band (with the halo rows) are requested before
  // any is used, so each warp keeps 2 (ROWS + 2) loads in flight.
  T bp[ROWS + 2], bcv[ROWS + 2];
#pragma unroll
  for (int j = 0; j < ROWS + 2; ++j) load_cell(phi_in, c_in, g, bc, y0 - 1 + j, x, x_in, bp[j], bcv[j]);

  T pN = bp[0], cN = bcv[0], p0 = bp[1], c0 = bcv[1], DN, QN, D0, Q0;
  w95_point(k, pN, cN, DN, QN);
  w95_point(k, p0, c0, D0, Q0);
  T pNW = shfl_w(pN), pNE = shfl_e(pN);
  T pW = shfl_w(p0), pE = shfl_e(p0);
  const bool noisy = k.alpha != T(0);

#pragma unroll
  for (int r = 0; r < ROWS; ++r) {
    const int row = y0 + r;
    const T pS = bp[r + 2], cS = bcv[r + 2];
    T DS, QS;
    w95_point(k, pS, cS, DS, QS);
    const T pSW = shfl_w(pS), pSE = shfl_e(pS);
    const T cW = shfl_w(c0), cE = shfl_e(c0);
    const T lc = ((cN + cS) - T(2) * c0) + ((cW + cE) - T(2) * c0);
    T p1, c1;

    // Bulk row: every owned cell's 3x3 phi neighbourhood is exactly 1 (or
    // exactly 0). There every phi difference, g(phi) and g'(phi) is exactly
    // zero, so dphi = 0, D~ is uniform and Q~ = 0: the full expressions below
    // reduce exactly to phi' = phi, c' = c + D~ lap(c).
    bool bulk = true;
    if (k.bulk && owner) {
      const T v = p0;
      bulk = (v == T(1) || v == T(0)) && pN == v && pS == v && pW == v && pE == v &&
             pNW == v && pNE == v && pSW == v && pSE == v;
    }
    if (k.bulk && __all_sync(0xffffffffu, bulk)) {
      p1 = p0;
      c1 = c0 + D0 * lc;
    } else {
      const T DW = shfl_w(D0), DE = shfl_e(D0);
      const T QW = shfl_w(Q0), QE = shfl_e(Q0);

      // phi derivatives, unscaled: N/S is axis 0 (reference x), W/E axis 1 (y)
      const T px = pN - pS;                 // 2dx * gradx(phi)
      const T py = pW - pE;                 // 2dx * grady(phi)
      const T pxx = (pN + pS) - T(2) * p0;  // dx^2 * gradxx(phi)
      const T pyy = (pW + pE) - T(2) * p0;  // dx^2 * gradyy(phi)
      const T lp = pxx + pyy;
      const T pxy = T(0.25) * ((pNW - pSW) - (pNE - pSE));  // dx^2 * grady(gradx(phi))

      // dc * dt  (Warren1995.py:69-71)
      const T dc = D0 * lc + T(0.25) * ((DN - DS) * (cN - cS) + (DW - DE) * (cW - cE)) +
                   Q0 * lp + T(0.25) * ((QN - QS) * px + (QW - QE) * py);

      // anisotropy (Warren1995.py:76-81) without trig: theta = atan2(py, px)
      const T r2 = px * px + py * py;
      T c2 = T(1), s2 = T(0);
      if (r2 > tiny_r2<T>()) {
        const T n = inv_norm(r2);
        const T ux = px * n, uy = py * n;
        c2 = ux * ux - uy * uy;
        s2 = T(2) * ux * uy;
      }
      const T c4 = c2 * c2 - s2 * s2;
      const T s4 = T(2) * s2 * c2;
      const T eta = T(1) + k.ye * c4;
      const T etap = T(-4) * k.ye * s4;
      const T etapp = T(-16) * k.ye * c4;

      // dphi * dt  (Warren1995.py:82-86)
      const T om = T(1) - p0;
      const T g0 = p0 * p0 * om * om;
      const T gp = p0 * (T(2) + p0 * (T(-6) + T(4) * p0));
      const T HA = k.WA * gp + k.hA * g0;
      const T HB = k.WB * gp + k.hB * g0;
      const T Hs = (T(1) - c0) * HA + c0 * HB;
      const T dtM = (T(1) - c0) * k.dtMA + c0 * k.dtMB;
      const T dyx = pyy - pxx;
      const T aniso = eta * eta * lp + eta * etap * (s2 * dyx + T(2) * c2 * pxy) +
                      T(0.5) * (etap * etap + eta * etapp) * (T(-2) * s2 * pxy + lp + c2 * dyx);
      T dphi = dtM * (k.e2 * aniso - Hs);
      // noise (:85-86): cells with g(phi) = 0 get none (the term is
      // proportional to g); the warp draws only if one of its cells needs it
      const bool need = noisy && owner && g0 != T(0);
      if (__any_sync(0xffffffffu, need)) {
        const U4 w4 = noise_group(seed, step, (uint32_t)row, (uint32_t)(x >> 2));
        const int j = x & 3;
        const uint32_t w = j == 0 ? w4.x : (j == 1 ? w4.y : (j == 2 ? w4.z : w4.w));
        if (need) {
          const T u = T(w >> 8) * T(5.9604644775390625e-08);
          dphi += dtM * k.alpha * (T(2) * u - T(1)) * (T(16) * g0) * Hs;
        }
      }
      p1 = p0 + dphi;
      c1 = c0 + dc;
    }
    if (owner && row < ny) {
      const int64_t o = (int64_t)row * g.pitch + x;
      phi_out[o] = p1;
      c_out[o] = c1;
    }
    pNW = pW; pN = p0; pNE = pE; cN = c0; DN = D0; QN = Q0;
    pW = pSW; p0 = pS; pE = pSE; c0 = cS; D0 = DS; Q0 = QS;
  }
}

template <typename T, int ROWS>
cudaError_t launch_rows(const W95Coef<T>& k, const Geo& g, const Bc<T>& bc, const T* phi_in,
                        const T* c_in, T* phi_out, T* c_out, uint64_t seed, uint64_t step,
                        const uint64_t* step_base, bool pdl, cudaStream_t s) {
  const long strips = (g.n[1] + kStrip - 1) / kStrip;
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
  if (tiling && tiling->tile_x && tiling->tile_x != kStrip)
    return fail(PPF_ERR_UNSUPPORTED, "Warren1995 warps own %d columns", kStrip);
  const int rows = tiling && tiling->tile_y ? tiling->tile_y : 2;

  const double dx2 = p->dx * p->dx;
  W95Coef<T> k;
  k.e2 = (T)(p->ebar * p->ebar / dx2);
  k.dtMA = (T)(p->dt * p->M_A);
  k.dtMB = (T)(p->dt * p->M_B);
  k.WA = (T)p->W_A;
  k.WB = (T)p->W_B;
  k.hA = (T)(30.0 * p->L_A * (1.0 / p->T - 1.0 / p->T_mA));
  k.hB = (T)(30.0 * p->L_B * (1.0 / p->T - 1.0 / p->T_mB));
  k.a0 = (T)(p->dt / dx2 * p->D_S);
  k.a1 = (T)(p->dt / dx2 * (p->D_L - p->D_S));
  k.vr = (T)(p->v_m / p->R);
  k.ye = (T)p->y_e;
  k.alpha = (T)p->alpha;
  k.bulk = !(tiling && (tiling->flags & PPF_TILING_FULL_EVAL));

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
