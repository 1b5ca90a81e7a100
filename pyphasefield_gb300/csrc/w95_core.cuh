// Warren-Boettinger (1995) solidification update for one warp-owned band,
// shared by the single-grid kernel (warren1995.cu) and the ensemble kernel
// (ensemble.cu).
//
// A warp owns a strip of kStrip = 30 output columns (lanes 1..30; lanes 0 and
// 31 carry the west/east halo columns) and a band of ROWS rows. It requests
// all ROWS + 2 rows of phi and c (band plus halo rows) before using any, then
// marches down the band keeping north/centre/south values of its column in
// registers and getting west/east neighbours by warp shuffles: no shared
// memory, no block-wide barriers.
//
// Reference: engine_Warren1995 (Engines/Warren1995.py:50-92), helpers
// _p, _g, _gprime (:17-28) and gradx/grady/gradxx/gradyy (:30-48). Axis 0 of
// the C-order grid is the reference's "x", axis 1 its "y".
#pragma once

#include <type_traits>

#include "ppf_common.cuh"

namespace ppf {
namespace w95 {

constexpr int kStrip = 30;

// Host-folded constants (all differences below are unscaled: the 1/(2dx),
// 1/dx^2 and dt factors are folded in here).
template <typename T>
struct Coef {
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

// Folds the engine parameters (user_data constants plus the derived ebar,
// W_A, W_B, M_A, M_B of just_before_simulating) into Coef.
template <typename T>
__host__ inline Coef<T> fold(const PpfWarren1995Params& p, bool bulk) {
  const double dx2 = p.dx * p.dx;
  Coef<T> k;
  k.e2 = (T)(p.ebar * p.ebar / dx2);
  k.dtMA = (T)(p.dt * p.M_A);
  k.dtMB = (T)(p.dt * p.M_B);
  k.WA = (T)p.W_A;
  k.WB = (T)p.W_B;
  k.hA = (T)(30.0 * p.L_A * (1.0 / p.T - 1.0 / p.T_mA));
  k.hB = (T)(30.0 * p.L_B * (1.0 / p.T - 1.0 / p.T_mB));
  k.a0 = (T)(p.dt / dx2 * p.D_S);
  k.a1 = (T)(p.dt / dx2 * (p.D_L - p.D_S));
  k.vr = (T)(p.v_m / p.R);
  k.ye = (T)p.y_e;
  k.alpha = (T)p.alpha;
  k.bulk = bulk ? 1 : 0;
  return k;
}

// Pointwise part evaluated on every cell entering the window:
//   Dt = dt/dx^2 * D_C,   D_C = D_S + p(phi) (D_L - D_S)          (:69)
//   Qt = dt/dx^2 * temp,  temp = D_C v_m c (1-c) (H_B - H_A) / R   (:70)
template <typename T>
__device__ __forceinline__ void point(const Coef<T>& k, T phi, T c, T& Dt, T& Qt) {
  const T p = phi * phi * phi * (T(10) + phi * (T(-15) + T(6) * phi));
  const T om = T(1) - phi;
  const T g = phi * phi * om * om;
  const T gp = phi * (T(2) + phi * (T(-6) + T(4) * phi));
  Dt = k.a0 + k.a1 * p;
  const T dH = (k.WB - k.WA) * gp + (k.hB - k.hA) * g;
  Qt = Dt * k.vr * c * (T(1) - c) * dH;
}

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

// One cell of phi and c; cells outside the grid through the boundary rule.
// COHERENT: see ldf (ppf_common.cuh).
template <typename T, bool COHERENT = false>
__device__ __forceinline__ void load_cell(const T* __restrict__ phi, const T* __restrict__ c,
                                          const Geo& g, const Bc<T>& bc, int row, int x,
                                          bool x_in, T& p, T& cc) {
  if (x_in && (unsigned)row < (unsigned)g.n[0]) {
    const int64_t o = (int64_t)row * g.pitch + x;
    p = ldf<COHERENT>(phi + o);
    cc = ldf<COHERENT>(c + o);
  } else {
    p = fetch<T, 2, COHERENT>(phi, g, bc, 0, row, x);
    cc = fetch<T, 2, COHERENT>(c, g, bc, 1, row, x);
  }
}

// Noise words of a band, computed once per Philox block. Cell (row, x)
// takes word x % 4 of the block with counter (x / 4, row, step). A band's
// owned columns x0 .. x0 + 29 start at a multiple of kStrip, an even column,
// so x0 % 4 is 0 or 2 and they span at most kGroups = 8 blocks per row. The
// ROWS * kGroups blocks of a band are spread over the lanes (one block per
// lane and pass: four rows in one pass) and each cell fetches its word from
// the computing lane by shuffles, instead of every lane evaluating the block
// of its own column.
static_assert(kStrip % 2 == 0 && kStrip <= 30, "owned columns must span at most 8 blocks");
constexpr int kGroups = 8;

template <int ROWS>
struct BandNoise {
  static constexpr int kJobs = ROWS * kGroups;
  static constexpr int kPasses = (kJobs + 31) / 32;
  U4 w[kPasses];

  __device__ __forceinline__ void draw(uint64_t seed, uint64_t step, int y0, uint32_t gbase) {
    const int lane = threadIdx.x;
#pragma unroll
    for (int p = 0; p < kPasses; ++p) {
      const int job = p * 32 + lane;
      const int r = job / kGroups, i = job - r * kGroups;
      w[p] = job < kJobs ? noise_group(seed, step, (uint32_t)(y0 + r), gbase + (uint32_t)i)
                         : U4{0u, 0u, 0u, 0u};
    }
  }
  // Word of column x (x / 4 - gbase in [0, kGroups)) on band row r; every
  // lane of the warp must call this together.
  __device__ __forceinline__ uint32_t word(int r, int x, uint32_t gbase) const {
    int i = (int)((uint32_t)x / 4u - gbase);
    i = i < 0 ? 0 : (i >= kGroups ? kGroups - 1 : i);  // halo lanes: any valid source
    const int job = r * kGroups + i;
    uint32_t v[4] = {0u, 0u, 0u, 0u};
#pragma unroll
    for (int p = 0; p < kPasses; ++p) {
      const int src = job - p * 32;
      const uint32_t a = __shfl_sync(0xffffffffu, w[p].x, src & 31);
      const uint32_t b = __shfl_sync(0xffffffffu, w[p].y, src & 31);
      const uint32_t c = __shfl_sync(0xffffffffu, w[p].z, src & 31);
      const uint32_t d = __shfl_sync(0xffffffffu, w[p].w, src & 31);
      if (src >= 0 && src < 32) {
        v[0] = a;
        v[1] = b;
        v[2] = c;
        v[3] = d;
      }
    }
    const int j = x & 3;
    return j == 0 ? v[0] : (j == 1 ? v[1] : (j == 2 ? v[2] : v[3]));
  }
};

template <typename T>
__device__ __forceinline__ T shfl_w(T v) { return __shfl_up_sync(0xffffffffu, v, 1); }
template <typename T>
__device__ __forceinline__ T shfl_e(T v) { return __shfl_down_sync(0xffffffffu, v, 1); }

}  // namespace w95
}  // namespace ppf
#include "w95_pack.cuh"
namespace ppf {
namespace w95 {

// Loads of one band (rows y0 - 1 .. y0 + ROWS, this lane's column). A band
// whose rows and 32 columns all lie inside the grid (warp-uniform test) reads
// straight from one base pointer; one whose rows lie inside but whose strip
// crosses the x edge reads every row from its lane's source column and fixes
// the ghost lanes after the loads (ColumnRule); the first and last row bands
// take the boundary rule per cell outside the grid.
template <typename T, int ROWS, bool COHERENT = false>
__device__ __forceinline__ void band_load(const Geo& g, const Bc<T>& bc,
                                          const T* __restrict__ phi_in,
                                          const T* __restrict__ c_in, int xs, int y0,
                                          T (&bp)[ROWS + 2], T (&bcv)[ROWS + 2]) {
  const int x = xs + (int)threadIdx.x;
  if (xs >= 0 && xs + 32 <= g.n[1] && y0 >= 1 && y0 + ROWS + 1 <= g.n[0]) {
    const int64_t o = (int64_t)(y0 - 1) * g.pitch + x;
    const T* p = phi_in + o;
    const T* c = c_in + o;
#pragma unroll
    for (int j = 0; j < ROWS + 2; ++j) {
      bp[j] = ldf<COHERENT>(p + (int64_t)j * g.pitch);
      bcv[j] = ldf<COHERENT>(c + (int64_t)j * g.pitch);
    }
    return;
  }
  if (y0 >= 1 && y0 + ROWS + 1 <= g.n[0]) {
    const ColumnRule<T, 2> cr(g, bc, x);
    const int64_t o = (int64_t)(y0 - 1) * g.pitch + cr.xi;
    const T* p = phi_in + o;
    const T* c = c_in + o;
#pragma unroll
    for (int j = 0; j < ROWS + 2; ++j) {
      bp[j] = ldf<COHERENT>(p + (int64_t)j * g.pitch);
      bcv[j] = ldf<COHERENT>(c + (int64_t)j * g.pitch);
    }
#pragma unroll
    for (int j = 0; j < ROWS + 2; ++j) {
      bp[j] = cr.value(0, bp[j]);
      bcv[j] = cr.value(1, bcv[j]);
    }
    return;
  }
  const bool x_in = (unsigned)x < (unsigned)g.n[1];
#pragma unroll
  for (int j = 0; j < ROWS + 2; ++j)
    load_cell<T, COHERENT>(phi_in, c_in, g, bc, y0 - 1 + j, x, x_in, bp[j], bcv[j]);
}

template <typename T, int ROWS>
__device__ __forceinline__ void band_compute(const Coef<T>& k, const Geo& g,
                                             T* __restrict__ phi_out, T* __restrict__ c_out,
                                             uint64_t seed, uint64_t step, int xs, int y0,
                                             const T (&bp)[ROWS + 2], const T (&bcv)[ROWS + 2]);

// One band: strip whose lane 0 sits at column xs, rows y0 .. y0+ROWS-1.
template <typename T, int ROWS, bool COHERENT = false>
__device__ __forceinline__ void band(const Coef<T>& k, const Geo& g, const Bc<T>& bc,
                                     const T* __restrict__ phi_in, const T* __restrict__ c_in,
                                     T* __restrict__ phi_out, T* __restrict__ c_out,
                                     uint64_t seed, uint64_t step, int xs, int y0) {
  T bp[ROWS + 2], bcv[ROWS + 2];
  band_load<T, ROWS, COHERENT>(g, bc, phi_in, c_in, xs, y0, bp, bcv);
  band_compute<T, ROWS>(k, g, phi_out, c_out, seed, step, xs, y0, bp, bcv);
}

template <typename T, int ROWS>
__device__ __forceinline__ void band_compute(const Coef<T>& k, const Geo& g,
                                             T* __restrict__ phi_out, T* __restrict__ c_out,
                                             uint64_t seed, uint64_t step, int xs, int y0,
                                             const T (&bp)[ROWS + 2], const T (&bcv)[ROWS + 2]) {
  if constexpr (std::is_same<T, float>::value && (ROWS == 2 || ROWS == 4 || ROWS == 8)) {
    band_compute_pk<ROWS / 2>(k, g, phi_out, c_out, seed, step, xs, y0, bp, bcv);
    return;
  }
  const int lane = threadIdx.x;
  const int ny = g.n[0], nx = g.n[1];
  const int x = xs + lane;
  const bool owner = lane >= 1 && lane <= kStrip && x < nx;

  T pN = bp[0], cN = bcv[0], p0 = bp[1], c0 = bcv[1], DN, QN, D0, Q0;
  point(k, pN, cN, DN, QN);
  point(k, p0, c0, D0, Q0);
  T pNW = shfl_w(pN), pNE = shfl_e(pN);
  T pW = shfl_w(p0), pE = shfl_e(p0);
  const bool noisy = k.alpha != T(0);
  // first owned column's Philox block (owners are lanes 1..30, x >= 0)
  const uint32_t gbase = (uint32_t)(xs + 1) / 4u;
  BandNoise<ROWS> noise;
  bool drawn = false;

#pragma unroll
  for (int r = 0; r < ROWS; ++r) {
    const int row = y0 + r;
    const T pS = bp[r + 2], cS = bcv[r + 2];
    T DS, QS;
    point(k, pS, cS, DS, QS);
    const T pSW = shfl_w(pS), pSE = shfl_e(pS);
    const T cW = shfl_w(c0), cE = shfl_e(c0);
    const T lc = ((cN + cS) - T(2) * c0) + ((cW + cE) - T(2) * c0);
    T p1, c1;

    // Bulk row: every owned cell's 3x3 phi neighbourhood is exactly 1 (or
    // exactly 0). There every phi difference, g(phi) and g'(phi) is exactly
    // zero, so dphi = 0, D~ is uniform and Q~ = 0: the full expressions below
    // reduce exactly to phi' = phi, c' = c + D~ lap(c).
    // (bitwise, branch-free test: no divergence on the common non-bulk path)
    bool bulk = false;
    if (k.bulk) {
      const T v = p0;
      const bool b = ((v == T(1)) | (v == T(0))) & (pN == v) & (pS == v) & (pW == v) &
                     (pE == v) & (pNW == v) & (pNE == v) & (pSW == v) & (pSE == v);
      bulk = __all_sync(0xffffffffu, b | !owner);
    }
    if (bulk) {
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
        if (!drawn) {  // the band's blocks, at the first row that needs any
          noise.draw(seed, step, y0, gbase);
          drawn = true;
        }
        const uint32_t w = noise.word(r, x, gbase);
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
    (void)lane;
  }
}

}  // namespace w95
}  // namespace ppf
