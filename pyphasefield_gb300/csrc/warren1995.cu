// Warren-Boettinger (1995) binary-alloy solidification step, fused.
//
// Persistent CTAs walk 32 x 32 tiles. For each tile, TMA stages phi and c
// with a one-cell halo (ghost rule applied to edge tiles), the CTA computes
// the pointwise solute
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
#include "ppf_tma.cuh"

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

// Tile geometry: 32 x 32 cells. Lane l owns column l; warp w owns the kR = 4
// consecutive rows 4w .. 4w+3 and sweeps down them keeping the
// north/centre/south values of its column in registers (12 shared-memory
// loads per cell instead of 25).
constexpr int kTX = 32;
constexpr int kR = 4;
constexpr int kTY = (kThreads / 32) * kR;
constexpr int kW = kTX + 2;  // pointwise region (tile + 1-cell halo)
constexpr int kH = kTY + 2;
constexpr int kN = kW * kH;
// TMA box: 16-byte aligned start 4 columns left of the tile, 1-row halo.
constexpr int kXOff = 4;
constexpr int kBX = kTX + 2 * kXOff;
constexpr int kBY = kTY + 2;
constexpr int kRaw = kXOff - 1;  // raw column of region column 0

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
constexpr int raw_elems() {
  return ((kBX * kBY * (int)sizeof(T) + 127) / 128 * 128) / (int)sizeof(T);
}
template <typename T>
size_t w95_smem_bytes() {
  return 128 + (size_t)4 * raw_elems<T>() * sizeof(T) + (size_t)2 * kN * sizeof(T);
}

template <typename T>
__device__ __forceinline__ T* align128(unsigned char* p) {
  return reinterpret_cast<T*>((reinterpret_cast<uintptr_t>(p) + 127) & ~uintptr_t(127));
}

// Persistent kernel: CTA b processes tiles b, b + G, b + 2G, ... The phi and c
// tiles of the next tile are fetched by TMA into the other half of a
// two-stage ring while the current tile computes. Cells outside the grid
// arrive zero-filled and are rewritten with the boundary rule on edge tiles.
template <typename T>
__global__ void __launch_bounds__(kThreads, 4)
    warren1995_kernel(const __grid_constant__ CUtensorMap map_phi,
                      const __grid_constant__ CUtensorMap map_c, W95Coef<T> k, Geo g, Bc<T> bc,
                      const T* __restrict__ phi_in, const T* __restrict__ c_in,
                      T* __restrict__ phi_out, T* __restrict__ c_out, uint64_t seed,
                      uint64_t step, const uint64_t* __restrict__ step_base, int tiles_x,
                      int ntiles, int* __restrict__ status) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ int abort_flag;
  constexpr int RE = raw_elems<T>();
  T* base = align128<T>(smem_raw);
  T* const sD = base + 4 * RE;
  T* const sQ = sD + kN;
  const int lane = threadIdx.x, warp = threadIdx.y;
  const int tid = lane + 32 * warp;
  const int ny = g.n[0], nx = g.n[1];
  const bool leader = tid == 0;

  if (leader) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_init_fence();
    abort_flag = 0;
  }
  __syncthreads();
  pdl_wait();
  pdl_launch_next();
  if (step_base) step += *step_base;

  auto issue = [&](int t, int st) {
    const int x0 = (t % tiles_x) * kTX, y0 = (t / tiles_x) * kTY;
    fence_proxy_async();
    mbar_expect_tx(&bars[st], (uint32_t)(2 * kBX * kBY * sizeof(T)));
    tma_load_2d(base + (2 * st) * RE, &map_phi, x0 - kXOff, y0 - 1, &bars[st]);
    tma_load_2d(base + (2 * st + 1) * RE, &map_c, x0 - kXOff, y0 - 1, &bars[st]);
  };

  int t = blockIdx.x;
  if (leader && t < ntiles) issue(t, 0);
  for (int it = 0; t < ntiles; ++it, t += gridDim.x) {
    const int st = it & 1;
    const int tn = t + gridDim.x;
    if (leader && tn < ntiles) issue(tn, st ^ 1);
    if (!mbar_wait(&bars[st], (uint32_t)((it >> 1) & 1))) abort_flag = 1;
    __syncthreads();
    if (abort_flag) {
      if (leader) {
        atomicOr(status, PPF_STATUS_TIMEOUT);
        mbar_wait(&bars[st], (uint32_t)((it >> 1) & 1));
        if (tn < ntiles) mbar_wait(&bars[st ^ 1], (uint32_t)(((it + 1) >> 1) & 1));
      }
      __syncthreads();
      return;
    }
    const T* sP = base + (2 * st) * RE;
    const T* sC = base + (2 * st + 1) * RE;
    const int x0 = (t % tiles_x) * kTX, y0 = (t / tiles_x) * kTY;

    // ---- edge tiles: ghost cells by the boundary rule
    if (x0 < 1 || y0 < 1 || x0 + kTX + 1 > nx || y0 + kTY + 1 > ny) {
      T* wP = base + (2 * st) * RE;
      T* wC = base + (2 * st + 1) * RE;
      for (int i = tid; i < kN; i += kThreads) {
        const int ly = i / kW, lx = i - ly * kW;
        const int gy = y0 - 1 + ly, gx = x0 - 1 + lx;
        if ((unsigned)gy >= (unsigned)ny || (unsigned)gx >= (unsigned)nx) {
          wP[ly * kBX + lx + kRaw] = fetch<T, 2>(phi_in, g, bc, 0, gy, gx);
          wC[ly * kBX + lx + kRaw] = fetch<T, 2>(c_in, g, bc, 1, gy, gx);
        }
      }
      __syncthreads();
    }

    // ---- pointwise D~, Q~ on the (kTY+2) x (kTX+2) region
    for (int i = tid; i < kN; i += kThreads) {
      const int ly = i / kW, lx = i - ly * kW;
      const int r = ly * kBX + lx + kRaw;
      T Dt, Qt;
      w95_point(k, sP[r], sC[r], Dt, Qt);
      sD[i] = Dt;
      sQ[i] = Qt;
    }
    __syncthreads();

    // ---- noise: the warp's 4 rows x 32 columns are 32 groups of 4 cells;
    // lane l draws Philox for group (row l/8, columns 4*(l%8) ..) and the
    // words are handed out with shuffles. Groups whose 4 cells all have
    // g(phi) = 0 skip the draw: the noise term is proportional to g(phi).
    const bool noisy = k.alpha != T(0);
    U4 nz{0u, 0u, 0u, 0u};
    const int ly0 = 1 + warp * kR;
    if (noisy) {
      const int gr = lane >> 3, gc = lane & 7;
      const T* row = sP + (ly0 + gr) * kBX + 1 + 4 * gc + kRaw;
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
    int ir = (ly0 - 1) * kBX + lx + kRaw;  // raw index (phi, c)
    int id = (ly0 - 1) * kW + lx;          // region index (D~, Q~)
    T pNW = sP[ir - 1], pN = sP[ir], pNE = sP[ir + 1];
    T cN = sC[ir], DN = sD[id], QN = sQ[id];
    ir += kBX;
    id += kW;
    T pW = sP[ir - 1], p0 = sP[ir], pE = sP[ir + 1];
    T c0 = sC[ir], D0 = sD[id], Q0 = sQ[id];
#pragma unroll
    for (int r = 0; r < kR; ++r, ir += kBX, id += kW) {
      const T cW = sC[ir - 1], cE = sC[ir + 1];
      const T DW = sD[id - 1], DE = sD[id + 1];
      const T QW = sQ[id - 1], QE = sQ[id + 1];
      const T pSW = sP[ir + kBX - 1], pS = sP[ir + kBX], pSE = sP[ir + kBX + 1];
      const T cS = sC[ir + kBX], DS = sD[id + kW], QS = sQ[id + kW];

      // phi derivatives, unscaled: N/S is axis 0 (reference x), W/E axis 1 (y)
      const T px = pN - pS;                 // 2dx * gradx(phi)
      const T py = pW - pE;                 // 2dx * grady(phi)
      const T pxx = (pN + pS) - T(2) * p0;  // dx^2 * gradxx(phi)
      const T pyy = (pW + pE) - T(2) * p0;  // dx^2 * gradyy(phi)
      const T lp = pxx + pyy;
      const T pxy = T(0.25) * ((pNW - pSW) - (pNE - pSE));  // dx^2 * grady(gradx(phi))

      // dc * dt  (Warren1995.py:69-71)
      const T lc = ((cN + cS) - T(2) * c0) + ((cW + cE) - T(2) * c0);
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
    __syncthreads();  // stage st and D~/Q~ are rewritten next
  }
}

// CTAs of `kern` resident per SM, and the SM count (cached per process).
template <typename K>
int resident_ctas(K kern, size_t smem, int* sms) {
  static int cached_sms = 0;
  if (!cached_sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&cached_sms, cudaDevAttrMultiProcessorCount, dev);
  }
  *sms = cached_sms;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, kThreads, smem) != cudaSuccess)
    n = 1;
  return n > 0 ? n : 1;
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

  const uint64_t dims[2] = {(uint64_t)g.n[1], (uint64_t)g.n[0]};
  const uint64_t strides[1] = {(uint64_t)g.pitch * sizeof(T)};
  const uint32_t box[2] = {(uint32_t)kBX, (uint32_t)kBY};
  CUtensorMap mp, mc;
  if ((rc = tensor_map(&mp, phi_in, (int)sizeof(T), 2, dims, strides, box))) return rc;
  if ((rc = tensor_map(&mc, c_in, (int)sizeof(T), 2, dims, strides, box))) return rc;
  int* st = status_ptr();
  if (!st) return fail(PPF_ERR_CUDA, "status word unavailable");

  auto kern = warren1995_kernel<T>;
  const size_t smem = w95_smem_bytes<T>();
  PPF_TRY_CUDA(allow_smem(kern, smem));
  const int tiles_x = (g.n[1] + kTX - 1) / kTX;
  const long ntiles = (long)tiles_x * ((g.n[0] + kTY - 1) / kTY);
  if (ntiles > (1L << 30)) return fail(PPF_ERR_INVALID, "grid too large");
  int sms = 0;
  const int per_sm = resident_ctas(kern, smem, &sms);
  const long slots = (long)per_sm * sms;
  const int grid_x = (int)(ntiles < slots ? ntiles : slots);
  PPF_TRY_CUDA(launch(kern, dim3(grid_x), dim3(32, kThreads / 32), smem, (cudaStream_t)stream,
                      tiling && tiling->pdl, mp, mc, k, g, bc, phi_in, c_in, phi_out, c_out, seed,
                      step, step_base, tiles_x, (int)ntiles, st));
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
