// Warren-Boettinger (1995) binary-alloy solidification step, fused.
//
// One CTA owns a 32 x 32 tile. It loads phi and c with a one-cell halo
// (ghost rule applied at load time), computes the pointwise solute
// diffusivity D_C(phi) and the solute-trapping flux coefficient temp(phi, c)
// once per staged cell into shared memory, then evaluates the full phi and c
// updates (anisotropic phase-field term, noise, non-flux-form solute update)
// and writes phi' and c'. One HBM read and one write of each field per step.
//
// Reference: engine_Warren1995 (Engines/Warren1995.py:50-92), helpers
// _p, _g, _gprime (:17-28) and gradx/grady/gradxx/gradyy (:30-48). Axis 0 of
// the C-order grid is the reference's "x", axis 1 its "y".
#include <cmath>

#include "ppf_common.cuh"

namespace ppf {
namespace {

constexpr int kThreads = 256;

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
};

// Pointwise part evaluated on every staged cell:
//   Dt = dt/dx^2 * D_C,   D_C = D_S + p(phi) (D_L - D_S)          (:69)
//   Qt = dt/dx^2 * temp,  temp = D_C v_m c (1-c) (H_B - H_A) / R   (:70)
template <typename T>
__device__ __forceinline__ void w95_point(const W95Coef<T>& k, T phi, T c,
                                          T& Dt, T& Qt) {
  const T p = phi * phi * phi * (T(10) + phi * (T(-15) + T(6) * phi));
  const T om = T(1) - phi;
  const T g = phi * phi * om * om;
  const T gp = phi * (T(2) + phi * (T(-6) + T(4) * phi));
  Dt = k.a0 + k.a1 * p;
  const T dH = (k.WB - k.WA) * gp + (k.hB - k.hA) * g;
  Qt = Dt * k.vr * c * (T(1) - c) * dH;
}

// Tile geometry: 32 x 32 cells per CTA, 256 threads (8 warps). Lane l owns
// column l; warp w owns the kR = 4 consecutive rows 4w .. 4w+3 and sweeps
// down them keeping the north/centre/south values of its column in
// registers (12 shared-memory loads per cell instead of 25).
constexpr int kTX = 32;
constexpr int kR = 4;
constexpr int kTY = (kThreads / 32) * kR;
constexpr int kW = kTX + 2;
constexpr int kH = kTY + 2;
constexpr int kN = kW * kH;

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
__global__ void __launch_bounds__(kThreads)
    warren1995_kernel(W95Coef<T> k, Geo g, Bc<T> bc,
                      const T* __restrict__ phi_in, const T* __restrict__ c_in,
                      T* __restrict__ phi_out, T* __restrict__ c_out,
                      uint64_t seed, uint64_t step,
                      const uint64_t* __restrict__ step_base) {
  __shared__ T sP[kN], sC[kN], sD[kN], sQ[kN];
  const int lane = threadIdx.x, warp = threadIdx.y;
  const int tid = lane + 32 * warp;
  const int x0 = blockIdx.x * kTX, y0 = blockIdx.y * kTY;
  const int ny = g.n[0], nx = g.n[1];
  const bool interior = x0 >= 1 && y0 >= 1 && x0 + kTX + 1 <= nx && y0 + kTY + 1 <= ny;

  pdl_wait();
  pdl_launch_next();
  if (step_base) step += *step_base;

  // ---- stage phi, c and the pointwise D~, Q~ on the (kTY+2) x (kTX+2) region
  for (int i = tid; i < kN; i += kThreads) {
    const int ly = i / kW, lx = i - ly * kW;
    const int gy = y0 - 1 + ly, gx = x0 - 1 + lx;
    T ph, cc;
    if (interior) {
      const int64_t o = (int64_t)gy * g.pitch + gx;
      ph = __ldg(phi_in + o);
      cc = __ldg(c_in + o);
    } else {
      ph = fetch<T, 2>(phi_in, g, bc, 0, gy, gx);
      cc = fetch<T, 2>(c_in, g, bc, 1, gy, gx);
    }
    T Dt, Qt;
    w95_point(k, ph, cc, Dt, Qt);
    sP[i] = ph;
    sC[i] = cc;
    sD[i] = Dt;
    sQ[i] = Qt;
  }
  __syncthreads();

  // ---- noise: the warp's 4 rows x 32 columns are 32 groups of 4 cells; lane
  // l draws Philox for group (row l/8, columns 4*(l%8) ..) and the words are
  // handed out with shuffles. Groups whose 4 cells all have g(phi) = 0 skip
  // the draw: the noise term is proportional to g(phi).
  const bool noisy = k.alpha != T(0);
  U4 nz{0u, 0u, 0u, 0u};
  const int ly0 = 1 + warp * kR;
  if (noisy) {
    const int gr = lane >> 3, gc = lane & 7;
    const T* row = sP + (ly0 + gr) * kW + 1 + 4 * gc;
    bool need = false;
#pragma unroll
    for (int j = 0; j < 4; ++j) need |= (row[j] != T(0)) && (row[j] != T(1));
    if (need)
      nz = noise_group(seed, step, (uint32_t)(y0 + warp * kR + gr),
                       (uint32_t)((x0 >> 2) + gc));
  }

  // ---- register-blocked sweep down this warp's rows
  const int lx = lane + 1;
  const int gx = x0 + lane;
  int i = (ly0 - 1) * kW + lx;
  T pNW = sP[i - 1], pN = sP[i], pNE = sP[i + 1];
  T cN = sC[i], DN = sD[i], QN = sQ[i];
  i += kW;
  T pW = sP[i - 1], p0 = sP[i], pE = sP[i + 1];
  T c0 = sC[i], D0 = sD[i], Q0 = sQ[i];
#pragma unroll
  for (int r = 0; r < kR; ++r, i += kW) {
    const T cW = sC[i - 1], cE = sC[i + 1];
    const T DW = sD[i - 1], DE = sD[i + 1];
    const T QW = sQ[i - 1], QE = sQ[i + 1];
    const T pSW = sP[i + kW - 1], pS = sP[i + kW], pSE = sP[i + kW + 1];
    const T cS = sC[i + kW], DS = sD[i + kW], QS = sQ[i + kW];

    // phi derivatives, unscaled: N/S is axis 0 (reference x), W/E axis 1 (y)
    const T px = pN - pS;                 // 2dx * gradx(phi)
    const T py = pW - pE;                 // 2dx * grady(phi)
    const T pxx = (pN + pS) - T(2) * p0;  // dx^2 * gradxx(phi)
    const T pyy = (pW + pE) - T(2) * p0;  // dx^2 * gradyy(phi)
    const T lp = pxx + pyy;
    const T pxy = T(0.25) * ((pNW - pSW) - (pNE - pSE));  // dx^2 * grady(gradx(phi))

    // dc * dt  (Warren1995.py:69-71)
    const T lc = ((cN + cS) - T(2) * c0) + ((cW + cE) - T(2) * c0);
    const T dc = D0 * lc +
                 T(0.25) * ((DN - DS) * (cN - cS) + (DW - DE) * (cW - cE)) +
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
    if (noisy) {
      const int src = r * 8 + (lane >> 2);
      const uint32_t wx = __shfl_sync(0xffffffffu, nz.x, src);
      const uint32_t wy = __shfl_sync(0xffffffffu, nz.y, src);
      const uint32_t wz = __shfl_sync(0xffffffffu, nz.z, src);
      const uint32_t ww = __shfl_sync(0xffffffffu, nz.w, src);
      const int j = lane & 3;
      const uint32_t w = j == 0 ? wx : (j == 1 ? wy : (j == 2 ? wz : ww));
      if (g0 != T(0)) {
        const T u = T(w >> 8) * T(5.9604644775390625e-08);
        dphi += dtM * k.alpha * (T(2) * u - T(1)) * (T(16) * g0) * Hs;
      }
    }
    const int gy = y0 + ly0 - 1 + r;
    if (gy < ny && gx < nx) {
      const int64_t o = (int64_t)gy * g.pitch + gx;
      phi_out[o] = p0 + dphi;
      c_out[o] = c0 + dc;
    }
    pNW = pW; pN = p0; pNE = pE; cN = c0; DN = D0; QN = Q0;
    pW = pSW; p0 = pS; pE = pSE; c0 = cS; D0 = DS; Q0 = QS;
  }
}

template <typename T>
int32_t warren1995(const PpfWarren1995Params* p, const PpfGrid* grid,
                   const PpfBoundary* b, const T* phi_in, const T* c_in,
                   T* phi_out, T* c_out, uint64_t seed, uint64_t step,
                   const uint64_t* step_base, const PpfTiling* tiling,
                   void* stream) {
  clear_error();
  if (!p) return fail(PPF_ERR_INVALID, "params is NULL");
  if (!(p->dx > 0) || !(p->T > 0) || !(p->T_mA > 0) || !(p->T_mB > 0) || !(p->R > 0))
    return fail(PPF_ERR_INVALID, "dx, T, T_mA, T_mB and R must be > 0");
  Geo g;
  int32_t rc = make_geo(grid, 2, 2, &g);
  if (rc) return rc;
  if (!phi_in || !c_in || !phi_out || !c_out)
    return fail(PPF_ERR_INVALID, "NULL field pointer");
  if (phi_in == phi_out || c_in == c_out || phi_in == c_out || c_in == phi_out ||
      phi_out == c_out)
    return fail(PPF_ERR_INVALID, "input and output fields must be distinct");
  if (tiling && tiling->depth > 1)
    return fail(PPF_ERR_UNSUPPORTED, "Warren1995 advances one step per pass");
  Bc<T> bc;
  if ((rc = make_bc<T>(b, g, p->dx, 2, 1, &bc))) return rc;
  if (tiling && ((tiling->tile_x && tiling->tile_x != kTX) ||
                 (tiling->tile_y && tiling->tile_y != kTY)))
    return fail(PPF_ERR_UNSUPPORTED, "Warren1995 tiles are %dx%d", kTX, kTY);

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

  dim3 gd((g.n[1] + kTX - 1) / kTX, (g.n[0] + kTY - 1) / kTY);
  if (gd.y > 65535) return fail(PPF_ERR_INVALID, "grid too tall");
  PPF_TRY_CUDA(launch(warren1995_kernel<T>, gd, dim3(32, kThreads / 32), 0,
                      (cudaStream_t)stream, tiling && tiling->pdl, k, g, bc, phi_in,
                      c_in, phi_out, c_out, seed, step, step_base));
  return PPF_OK;
}

}  // namespace
}  // namespace ppf

using namespace ppf;

extern "C" {

int32_t ppf_warren1995_step_f32(const PpfWarren1995Params* p, const PpfGrid* g,
                                const PpfBoundary* bc, const float* phi_in,
                                const float* c_in, float* phi_out, float* c_out,
                                uint64_t seed, uint64_t step,
                                const uint64_t* step_base,
                                const PpfTiling* tiling, void* stream) {
  return warren1995<float>(p, g, bc, phi_in, c_in, phi_out, c_out, seed, step,
                           step_base, tiling, stream);
}
int32_t ppf_warren1995_step_f64(const PpfWarren1995Params* p, const PpfGrid* g,
                                const PpfBoundary* bc, const double* phi_in,
                                const double* c_in, double* phi_out,
                                double* c_out, uint64_t seed, uint64_t step,
                                const uint64_t* step_base,
                                const PpfTiling* tiling, void* stream) {
  return warren1995<double>(p, g, bc, phi_in, c_in, phi_out, c_out, seed, step,
                            step_base, tiling, stream);
}

}  // extern "C"
