// NCGPU: the multi-component solidification engine with quaternion
// orientation fields (pyphasefield Engines/NCGPU.py, and its variant
// Engines/NCGPU_new.py), 2 to 6 components.
//
//   ncgpu_table_kernel: the pure-element energies and interaction
//       parameters at every cell's temperature, once per run (the
//       temperature is fixed while the engine steps).
//   ncgpu_thermo_kernel  (NComponent_helper_kernel, NCGPU.py:248-303,
//       NCGPU_new.py:256-314): per cell the molar Gibbs energies of the
//       solid (first phase, sorted) and liquid, from the pure-element
//       energies of the TDB (piecewise in T, basis 1, T, T ln T, T^2, T^3,
//       T^7, 1/T, T^-9) plus R T sum x ln x and the binary Redlich-Kister
//       terms, in double; dG/dc by the reference's forward difference (step
//       1e-7; one for every component in NCGPU, one per component in
//       NCGPU_new); stores G_S - G_L, the mobility M_c and dF/dc (with the
//       Langevin noise) for the update.
//   ncgpu_kernel (NComponent_kernel, NCGPU.py:37-242, NCGPU_new.py:38-252):
//       phi (anisotropic through the quaternion-rotated gradient psi; plus
//       the phase noise in NCGPU_new), q1 and q4 (orientation diffusion,
//       plus the orientation noise in NCGPU_new, normalised to unit
//       length), c (div M_c grad dF/dc minus the c-weighted term), phi
//       clamped to [1e-6, 1 - 1e-6] ([1e-4, 0.9999] in NCGPU_new).
// Ghost cells follow the boundary rule while the tiles are read (periodic
// or zero-gradient), for the fields, the temperature and the per-cell
// thermodynamic terms alike.
#include <math.h>
#include <type_traits>
#include <string.h>

#include "ppf_common.cuh"

namespace ppf {
namespace {

constexpr int kMaxComp = PPF_NCGPU_MAX_COMP;

template <typename T>
struct NcCoef {
  T idx, dt, v_m, D_L, D_S, M_qmax, H, y_e, beta, ebar2, eqbar2, noise;
  T noise_phi, noise_q;  // NCGPU_new only
  T phi_lo, phi_hi;      // the phi clamp
  int variant;           // PPF_NCGPU_VARIANT_*
  T W[kMaxComp], M[kMaxComp];
};

// Noise streams: 0 .. ncomp - 2 the concentration noise of each component
// (NCGPU draws stream 0 only), then the phase and the orientation noise of
// NCGPU_new.
constexpr int kStreamPhi = 8, kStreamQ1 = 9, kStreamQ4 = 10;

constexpr int kMaxExcess = PPF_NCGPU_MAX_EXCESS;

struct NcGibbs {
  double piece[2][kMaxComp][4][10];  // [phase][component][piece] {lo, hi, 8 coefficients}
  int npieces[2][kMaxComp];
  int nex;                            // binary Redlich-Kister terms
  int ex_meta[kMaxExcess][5];         // phase, a, b, order, npieces
  double ex_piece[kMaxExcess][4][10];
};

// The concentration fields and the per-component thermodynamic terms.
template <typename T>
struct NcPtrs {
  const T* c[kMaxComp - 1];
  T* c_out[kMaxComp - 1];
  T* Mc[kMaxComp - 1];
  T* dF[kMaxComp - 1];
};

// A function piecewise in T over the basis 1, T, T ln T, T^2, T^3, T^7,
// 1/T, T^-9: pieces[k] = {T_lo, T_hi, 8 coefficients}.
__device__ __forceinline__ double piecewise(const double (*pieces)[10], int np, double T,
                                           double lnT) {
  for (int k = 0; k < np; ++k) {
    const double* c = pieces[k];
    if (T >= c[0] && T < c[1]) {
      const double T2 = T * T, T3 = T2 * T, T7 = T3 * T3 * T, iT = 1.0 / T;
      const double iT3 = iT * iT * iT, iT9 = iT3 * iT3 * iT3;
      return c[2] + c[3] * T + c[4] * T * lnT + c[5] * T2 + c[6] * T3 + c[7] * T7 +
             c[8] * iT + c[9] * iT9;
    }
  }
  return 0.0;  // outside every range, as a piecewise TDB function gives
}

__device__ __forceinline__ double g_pure(const NcGibbs& g, int ph, int comp, double T,
                                         double lnT) {
  return piecewise(g.piece[ph][comp], g.npieces[ph][comp], T, lnT);
}

__device__ __forceinline__ double l_excess(const NcGibbs& g, int e, double T, double lnT) {
  return piecewise(g.ex_piece[e], g.ex_meta[e][4], T, lnT);
}

// N(0,1) of cell (row, col) at a step: Box-Muller on two uniforms from a
// Philox4x32-10 block (counter (col / 2, row, step), key seed ^ (0x5eed0000 +
// stream)), pair col % 2.
template <typename T>
__device__ __forceinline__ T noise_normal(uint64_t seed, uint64_t step, int row, int col,
                                          int stream) {
  const U4 w = philox4x32_10(U4{(uint32_t)(col >> 1), (uint32_t)row, (uint32_t)step,
                                (uint32_t)(step >> 32)},
                             (uint32_t)seed ^ (0x5EED0000u + (uint32_t)stream),
                             (uint32_t)(seed >> 32));
  const uint32_t a = (col & 1) ? w.z : w.x, b = (col & 1) ? w.w : w.y;
  // the uniforms are exact in either precision
  const T u1 = ((T)(a >> 8) + T(0.5)) * (T(1) / T(16777216));
  const T u2 = (T)(b >> 8) * (T(1) / T(16777216));
  return sqrt(T(-2) * log(u1)) * cospi(T(2) * u2);
}

// The pure-element Gibbs energies of both phases at a cell's temperature:
// tab[l] = G_solid,l, tab[N + l] = G_liquid,l.
template <int N>
__device__ __forceinline__ void pure_energies(const NcGibbs& gb, double t, double lnT,
                                              double* tab) {
#pragma unroll
  for (int l = 0; l < N; ++l) {
    tab[l] = g_pure(gb, 0, l, t, lnT);
    tab[N + l] = g_pure(gb, 1, l, t, lnT);
  }
}

// The per-cell table of pure-element energies and interaction parameters
// (2 ncomp + nex planes of doubles in the grid's layout) for a temperature
// field that stays fixed over many steps: the thermodynamics kernel then
// reads them instead of evaluating the piecewise polynomials and a
// logarithm. For float fields the same memory holds 3 ncomp - 2 + nex float
// planes: G_solid,l - G_liquid,l (l < ncomp), then G_solid,l - G_solid,last
// and G_liquid,l - G_liquid,last (l < ncomp - 1), then the L of each excess
// term.
template <typename T, int N>
__global__ void __launch_bounds__(256)
    ncgpu_table_kernel(Geo g, const __grid_constant__ NcGibbs gb, const T* __restrict__ temp,
                       double* __restrict__ tab) {
  pdl_wait();
  pdl_launch_next();
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  if (x >= g.n[1]) return;
  const int64_t i = (int64_t)y * g.pitch + x;
  const int64_t plane = (int64_t)g.n[0] * g.pitch;
  const double t = (double)temp[i], lnT = log(t);
  double v[2 * N];
  pure_energies<N>(gb, t, lnT, v);
  if constexpr (std::is_same<T, float>::value) {
    // the float path's layout (float planes in the same memory): the
    // differences it uses, formed here in double once per run
    float* ft = reinterpret_cast<float*>(tab);
#pragma unroll
    for (int l = 0; l < N; ++l) ft[l * plane + i] = (float)(v[l] - v[N + l]);
#pragma unroll
    for (int l = 0; l < N - 1; ++l) {
      ft[(N + l) * plane + i] = (float)(v[l] - v[N - 1]);
      ft[(2 * N - 1 + l) * plane + i] = (float)(v[N + l] - v[2 * N - 1]);
    }
    for (int e = 0; e < gb.nex; ++e)
      ft[(3 * N - 2 + e) * plane + i] = (float)l_excess(gb, e, t, lnT);
  } else {
#pragma unroll
    for (int l = 0; l < 2 * N; ++l) tab[l * plane + i] = v[l];
    for (int e = 0; e < gb.nex; ++e) tab[(2 * N + e) * plane + i] = l_excess(gb, e, t, lnT);
  }
}

// 1e7 (f(x + d) - f(x)) for f(x) = x ln x (0 at x <= 0) and d = s 1e-7,
// s = +1 or -1: the reference's forward difference of the ideal mixing term
// at step 1e-7, in a form without cancellation: d ln x + (x + d) log1p(d / x)
// in float while |d / x| <= 0.01, in double below that (a nearly absent
// component).
__device__ __forceinline__ float dxlogx(float x, float s) {
  if (x >= 1e-5f) {
    const float r = s * 1e-7f / x;
    return s * logf(x) + (x * 1e7f + s) * log1pf(r);
  }
  const double xd = (double)x, xp = xd + (double)s * 0.0000001;
  const double a = xp > 0 ? xp * log(xp) : 0.0, b = xd > 0 ? xd * log(xd) : 0.0;
  return (float)(10000000.0 * (a - b));
}

// The float path of the thermodynamics kernel: the pure-element energies
// (and their differences) in double, everything else in float, and the
// forward differences of the reference taken as sums of per-term
// differences, so that no difference of two Gibbs energies of ~1e4 J/mol is
// formed in float. Up (component `up` by +1e-7) and down (the last
// component by -1e-7) steps, as in the reference.
template <int N>
struct NcF32Thermo {
  float x[N];
  float gdiff[N];        // G_solid,l - G_liquid,l
  float dls[N - 1], dll[N - 1];  // G_phase,l - G_phase,N-1 (solid, liquid), l < N - 1
  float L[kMaxExcess];
  float rt;

  // 1e7 (E(x + 1e-7 e_up - 1e-7 e_last) - E(x)) of the solid (es) and the
  // liquid (el) molar Gibbs energy
  __device__ __forceinline__ void fd(const NcGibbs& gb, int up, float& es, float& el) const {
    const float dmix = dxlogx(x[up], 1.f) + dxlogx(x[N - 1], -1.f);
    float xs = dls[up], xl = dll[up];
    for (int e = 0; e < gb.nex; ++e) {
      const int a = gb.ex_meta[e][1], b = gb.ex_meta[e][2], ord = gb.ex_meta[e][3];
      const float sa = a == up ? 1.f : (a == N - 1 ? -1.f : 0.f);
      const float sb = b == up ? 1.f : (b == N - 1 ? -1.f : 0.f);
      if (sa == 0.f && sb == 0.f) continue;
      float xa = 0.f, xb = 0.f;
#pragma unroll
      for (int l = 0; l < N; ++l) {
        xa = l == a ? x[l] : xa;
        xb = l == b ? x[l] : xb;
      }
      // term = L xa xb u^k, u = xa - xb: 1e7 dterm = L (dP' (u + du)^k + P dU')
      // with P = xa xb, dP' = 1e7 dP, dU' = 1e7 ((u + du)^k - u^k)
      const float u = xa - xb, su = sa - sb, du = su * 1e-7f;
      const float P = xa * xb;
      const float dP = sa * xb + xa * sb + 1e-7f * sa * sb;
      float upow = 1.f, dU = 0.f;  // (u + du)^k and its difference, term by term
      float binom = 1.f;
      // (u + du)^k - u^k = sum_{j >= 1} C(k, j) u^(k-j) du^j
      // scaled: su sum_j C(k, j) u^(k-j) du^(j-1)
      float upk[8];
      upk[0] = 1.f;
      for (int j = 1; j <= ord && j < 8; ++j) upk[j] = upk[j - 1] * u;
      for (int j = 0; j < ord; ++j) upow *= u + du;
      float dup = 1.f;  // du^(j-1)
      for (int j = 1; j <= ord && j < 8; ++j) {
        binom = binom * (float)(ord - j + 1) / (float)j;
        dU += binom * upk[ord - j] * dup;
        dup *= du;
      }
      const float dterm = L[e] * (dP * upow + P * su * dU);
      if (gb.ex_meta[e][0] == 0)
        xs += dterm;
      else
        xl += dterm;
    }
    es = xs + rt * dmix;
    el = xl + rt * dmix;
  }
};

template <int NC>
__device__ __forceinline__ void ncgpu_thermo_f32(const Geo& g, const NcCoef<float>& k,
                                                 const NcGibbs& gb, const float* __restrict__ phi,
                                                 NcPtrs<float> cp, const float* __restrict__ temp,
                                                 const double* __restrict__ tab,
                                                 float* __restrict__ dG, uint64_t seed,
                                                 uint64_t st, int x, int y, int64_t i) {
  constexpr int N = NC + 1;
  const int64_t plane = (int64_t)g.n[0] * g.pitch;
  const float tf = temp[i];
  const double t = (double)tf;
  NcF32Thermo<N> th;
  double last = 1.0;
#pragma unroll
  for (int l = 0; l < NC; ++l) {
    th.x[l] = cp.c[l][i];
    last -= (double)th.x[l];
  }
  th.x[NC] = (float)last;
  if (tab) {
    // float planes written by ncgpu_table_kernel<float>
    const float* ft = reinterpret_cast<const float*>(tab);
#pragma unroll
    for (int l = 0; l < N; ++l) th.gdiff[l] = __ldg(ft + l * plane + i);
#pragma unroll
    for (int l = 0; l < N - 1; ++l) {
      th.dls[l] = __ldg(ft + (N + l) * plane + i);
      th.dll[l] = __ldg(ft + (2 * N - 1 + l) * plane + i);
    }
    for (int e = 0; e < gb.nex; ++e) th.L[e] = __ldg(ft + (3 * N - 2 + e) * plane + i);
  } else {
    double G[2 * N];
    const double lnT = log(t);
    pure_energies<N>(gb, t, lnT, G);
#pragma unroll
    for (int l = 0; l < N; ++l) th.gdiff[l] = (float)(G[l] - G[N + l]);
#pragma unroll
    for (int l = 0; l < N - 1; ++l) {
      th.dls[l] = (float)(G[l] - G[N - 1]);
      th.dll[l] = (float)(G[N + l] - G[2 * N - 1]);
    }
    for (int e = 0; e < gb.nex; ++e) th.L[e] = (float)l_excess(gb, e, t, lnT);
  }
  th.rt = 8.3145f * tf;
  // G_S - G_L: the mixing term is the same in both phases and cancels
  float dg = 0.f;
#pragma unroll
  for (int l = 0; l < N; ++l) dg += th.x[l] * th.gdiff[l];
  for (int e = 0; e < gb.nex; ++e) {
    const int a = gb.ex_meta[e][1], b = gb.ex_meta[e][2], ord = gb.ex_meta[e][3];
    float xa = 0.f, xb = 0.f;
#pragma unroll
    for (int l = 0; l < N; ++l) {
      xa = l == a ? th.x[l] : xa;
      xb = l == b ? th.x[l] : xb;
    }
    float term = xa * xb * th.L[e];
    for (int j = 0; j < ord; ++j) term *= xa - xb;
    dg += gb.ex_meta[e][0] == 0 ? term : -term;
  }
  const float p = phi[i];
  const float gg = p * p * (1.f - p) * (1.f - p);
  const float h = p * p * p * (6.f * p * p - 15.f * p + 10.f);
  const float namp = k.noise * sqrtf(2.f * 8.314f * tf / k.v_m);
  dG[i] = dg;
  const float mob = k.v_m * (k.D_L + h * (k.D_S - k.D_L)) / (8.314f * tf);
  if (k.variant == 0) {
    float es, el;
    th.fd(gb, 0, es, el);
    const float nz = k.noise > 0.f ? namp * noise_normal<float>(seed, st, y, x, 0) : 0.f;
    const float dfc = (el + h * (es - el)) / k.v_m;
#pragma unroll
    for (int l = 0; l < NC; ++l) {
      cp.Mc[l][i] = th.x[l] * mob;
      cp.dF[l][i] = dfc + (k.W[l] - k.W[NC]) * gg * tf + nz;
    }
  } else {
#pragma unroll
    for (int l = 0; l < NC; ++l) {
      float es, el;
      th.fd(gb, l, es, el);
      const float nz = k.noise > 0.f ? namp * noise_normal<float>(seed, st, y, x, l) : 0.f;
      cp.Mc[l][i] = th.x[l] * mob;
      cp.dF[l][i] = (el + h * (es - el)) / k.v_m + (k.W[l] - k.W[NC]) * gg * tf + nz;
    }
  }
}

template <typename T, int NC>
__global__ void __launch_bounds__(256)
    ncgpu_thermo_kernel(Geo g, NcCoef<T> k, const __grid_constant__ NcGibbs gb,
                        const T* __restrict__ phi,
                        NcPtrs<T> cp, const T* __restrict__ temp, const double* __restrict__ tab,
                        T* __restrict__ dG, uint64_t seed, uint64_t step,
                        const uint64_t* step_base) {
  pdl_wait();
  pdl_launch_next();
  constexpr int N = NC + 1;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  if (x >= g.n[1]) return;
  const int64_t i = (int64_t)y * g.pitch + x;
  const uint64_t st = step + (step_base ? *step_base : 0);
  if constexpr (std::is_same<T, float>::value) {
    ncgpu_thermo_f32<NC>(g, k, gb, phi, cp, temp, tab, dG, seed, st, x, y, i);
    return;
  }
  const double t = (double)temp[i];
  double xs[N], xp[N], G[2 * N];
  double last = 1.0;
#pragma unroll
  for (int l = 0; l < NC; ++l) {
    xs[l] = (double)cp.c[l][i];
    last -= xs[l];
  }
  xs[NC] = last;
  const int64_t plane = (int64_t)g.n[0] * g.pitch;
  const double lnT = tab ? 0.0 : log(t);
  if (tab) {
#pragma unroll
    for (int l = 0; l < 2 * N; ++l) G[l] = __ldg(tab + l * plane + i);
  } else {
    pure_energies<N>(gb, t, lnT, G);
  }
  const double* Gs = G;
  const double* Gl = G + N;
  // the ideal part (sum x G and sum x ln x) and the binary Redlich-Kister
  // terms x_a x_b L (x_a - x_b)^k of both phases at a composition xv
  auto energies = [&](const double* xv, double& mixv, double& ls, double& ll, double& es,
                      double& el) {
    mixv = ls = ll = es = el = 0.0;
#pragma unroll
    for (int l = 0; l < N; ++l) {
      if (xv[l] > 0) mixv += xv[l] * log(xv[l]);
      ls += xv[l] * Gs[l];
      ll += xv[l] * Gl[l];
    }
    for (int e = 0; e < gb.nex; ++e) {
      const int a = gb.ex_meta[e][1], b = gb.ex_meta[e][2], ord = gb.ex_meta[e][3];
      const double L = tab ? __ldg(tab + (2 * N + e) * plane + i) : l_excess(gb, e, t, lnT);
      double xa = 0.0, xb = 0.0;
#pragma unroll
      for (int l = 0; l < N; ++l) {
        xa = l == a ? xv[l] : xa;
        xb = l == b ? xv[l] : xb;
      }
      double term = xa * xb * L;
      for (int j = 0; j < ord; ++j) term *= xa - xb;
      if (gb.ex_meta[e][0] == 0)
        es += term;
      else
        el += term;
    }
  };
  const double rt = 8.3145 * t;
  double mix, lin_s, lin_l, ex_s, ex_l;
  energies(xs, mix, lin_s, lin_l, ex_s, ex_l);
  const double gs = lin_s + rt * mix + ex_s;
  const double gl = lin_l + rt * mix + ex_l;
  const T p = phi[i];
  const T gg = p * p * (T(1) - p) * (T(1) - p);
  const T h = p * p * p * (T(6) * p * p - T(15) * p + T(10));
  const T tt = (T)t;
  const T namp = k.noise * sqrt(T(2) * T(8.314) * tt / k.v_m);
  dG[i] = (T)(gs - gl);
  if (k.variant == 0) {
    // the reference's forward difference (NCGPU.py:282-286): the last
    // component down, the first up, one derivative for every component, as
    // the difference of the two molar Gibbs energies; one noise draw
    // shared by every component
#pragma unroll
    for (int l = 0; l < N; ++l) xp[l] = xs[l];
    xp[NC] -= 0.0000001;
    xp[0] += 0.0000001;
    double mixp, linp_s, linp_l, exp_s, exp_l;
    energies(xp, mixp, linp_s, linp_l, exp_s, exp_l);
    const double dgl = 10000000.0 * ((linp_l + rt * mixp + exp_l) - gl);
    const double dgs = 10000000.0 * ((linp_s + rt * mixp + exp_s) - gs);
    const T nz = k.noise > T(0) ? namp * noise_normal<T>(seed, st, y, x, 0) : T(0);
    const T dfc = (T)((dgl + (double)h * (dgs - dgl)) / (double)k.v_m);
#pragma unroll
    for (int l = 0; l < NC; ++l) {
      cp.Mc[l][i] = k.v_m * (T)xs[l] * (k.D_L + h * (k.D_S - k.D_L)) / (T(8.314) * tt);
      cp.dF[l][i] = dfc + (k.W[l] - k.W[NC]) * gg * tt + nz;
    }
  } else {
    // NCGPU_new (NCGPU_new.py:298-313): the last component down once, then
    // each component up and back in place, one derivative and one noise
    // draw (stream l) per component
#pragma unroll
    for (int l = 0; l < N; ++l) xp[l] = xs[l];
    xp[NC] -= 0.0000001;
#pragma unroll
    for (int l = 0; l < NC; ++l) {
      xp[l] += 0.0000001;
      double mixp, linp_s, linp_l, exp_s, exp_l;
      energies(xp, mixp, linp_s, linp_l, exp_s, exp_l);
      const double dgl = 10000000.0 * ((linp_l + rt * mixp + exp_l) - gl);
      const double dgs = 10000000.0 * ((linp_s + rt * mixp + exp_s) - gs);
      const T nz = k.noise > T(0) ? namp * noise_normal<T>(seed, st, y, x, l) : T(0);
      cp.Mc[l][i] = k.v_m * (T)xs[l] * (k.D_L + h * (k.D_S - k.D_L)) / (T(8.314) * tt);
      cp.dF[l][i] = (T)((dgl + (double)h * (dgs - dgl)) / (double)k.v_m) +
                    (k.W[l] - k.W[NC]) * gg * tt + nz;
      xp[l] -= 0.0000001;
    }
  }
}

template <typename T>
__device__ __forceinline__ T divagradb(T a, T axp, T axm, T ayp, T aym, T b, T bxp, T bxm,
                                       T byp, T bym, T idx) {
  return T(0.5) * idx * idx *
         ((axp + a) * (bxp - b) - (a + axm) * (b - bxm) + (ayp + a) * (byp - b) -
          (a + aym) * (b - bym));
}

// The update of cell (y, x). A cell whose 3 x 3 neighbourhood lies inside
// the grid reads its neighbours directly, the others through the boundary
// rule; INNER: every cell of the warp is of the first kind, so the body has
// no boundary-rule code at all (a compact instruction stream for the
// interior warps, which are nearly all of them).
template <typename T, int NC, bool INNER>
__device__ __forceinline__ void ncgpu_cell(const Geo& g, const Bc<T>& bc, const NcCoef<T>& k,
                                           const T* __restrict__ phi, const T* __restrict__ q1,
                                           const T* __restrict__ q4, const NcPtrs<T>& cp,
                                           const T* __restrict__ temp, const T* __restrict__ dG,
                                           T* __restrict__ phi_o, T* __restrict__ q1_o,
                                           T* __restrict__ q4_o, uint64_t seed, uint64_t step,
                                           const uint64_t* step_base, int x, int y) {
  const int64_t i = (int64_t)y * g.pitch + x;
  const bool inner = INNER || (x >= 1 && x + 1 < g.n[1] && y >= 1 && y + 1 < g.n[0]);
  auto F = [&](const T* f, int dy, int dx) {
    if constexpr (INNER)
      return __ldg(f + i + (int64_t)dy * g.pitch + dx);
    else
      return inner ? __ldg(f + i + (int64_t)dy * g.pitch + dx)
                   : fetch<T, 2>(f, g, bc, 0, y + dy, x + dx);
  };
  const T idx = k.idx;
  const T ph = phi[i];
  const T gg = ph * ph * (T(1) - ph) * (T(1) - ph);
  const T h = ph * ph * ph * (T(6) * ph * ph - T(15) * ph + T(10));
  const T hprime = T(30) * gg;
  const T gprime = T(4) * ph * ph * ph - T(6) * ph * ph + T(2) * ph;
  const T pxp = F(phi, 0, 1), pxm = F(phi, 0, -1), pyp = F(phi, 1, 0), pym = F(phi, -1, 0);
  const T dpx = T(0.5) * (pxp - pxm) * idx, dpy = T(0.5) * (pyp - pym) * idx;
  const T dpx2 = dpx * dpx, dpy2 = dpy * dpy;
  const T t = temp[i];
  const T txp = F(temp, 0, 1), txm = F(temp, 0, -1), typ = F(temp, 1, 0), tym = F(temp, -1, 0);
  const T dTx = T(0.5) * idx * (txp - txm), dTy = T(0.5) * idx * (typ - tym);
  const T pxx = (pxp + pxm - T(2) * ph) * idx * idx;
  const T pyy = (pyp + pym - T(2) * ph) * idx * idx;
  const T lphi = pxx + pyy;
  const T pxy = T(0.25) * (F(phi, 1, 1) - F(phi, 1, -1) - F(phi, -1, 1) + F(phi, -1, -1)) *
                idx * idx;
  T mg2 = dpx2 + dpy2;
  if (mg2 < T(1e-6)) mg2 = T(1e-6);
  const T a1 = q1[i], a4 = q4[i];
  const T q1xp = F(q1, 0, 1), q1xm = F(q1, 0, -1), q1yp = F(q1, 1, 0), q1ym = F(q1, -1, 0);
  const T q4xp = F(q4, 0, 1), q4xm = F(q4, 0, -1), q4yp = F(q4, 1, 0), q4ym = F(q4, -1, 0);
  const T dq1x = T(0.5) * idx * (q1xp - q1xm), dq1y = T(0.5) * idx * (q1yp - q1ym);
  const T dq4x = T(0.5) * idx * (q4xp - q4xm), dq4y = T(0.5) * idx * (q4yp - q4ym);
  // |grad q| across each face, g = idx sqrt(s), and the reciprocal of its
  // value clamped below at beta, from one reciprocal square root per face
  // (s = 0, a uniform orientation, takes 1 / beta)
  T gxp, gxm, gyp, gym, igxp, igxm, igyp, igym;
  {
    const T dx_ = T(1) / idx, ibeta = T(1) / k.beta;
    auto face = [&](T dq1, T dq4, T& gf, T& igf) {
      const T sq = dq1 * dq1 + dq4 * dq4;
      const T r = sq > T(0) ? rsqrt(sq) : T(0);
      gf = idx * (sq * r);
      igf = gf < k.beta ? ibeta : dx_ * r;
    };
    face(q1xp - a1, q4xp - a4, gxp, igxp);
    face(q1xm - a1, q4xm - a4, gxm, igxm);
    face(q1yp - a1, q4yp - a4, gyp, igyp);
    face(q1ym - a1, q4ym - a4, gym, igym);
  }
  const T mgq = T(0.5) * (gxp + gxm + gyp + gym);
  // psi: the phi gradient rotated by the orientation. The anisotropy terms
  // divide powers of psi by powers of |grad phi|^2 (up to the 8th); they are
  // evaluated here on the unit vectors u = grad phi / m, s = psi / m
  // (m = |grad phi|, clamped as the reference clamps |grad phi|^2 to 1e-6):
  // the same expressions, without the float overflow of |grad phi|^8 at
  // centimetre cell sizes
  const T q2q2 = a1 * a1 - a4 * a4, qq2 = T(2) * a1 * a4;
  const T im = rsqrt(mg2), m = mg2 * im;
  const T ux = dpx * im, uy = dpy * im;
  const T sx = (q2q2 * dpx - qq2 * dpy) * im, sy = (qq2 * dpx + q2q2 * dpy) * im;
  const T sx2 = sx * sx, sy2 = sy * sy;
  const T sx3 = sx2 * sx, sy3 = sy2 * sy;
  const T s4 = sx2 * sx2 + sy2 * sy2;
  const T dq2q2dx = T(2) * a1 * dq1x - T(2) * a4 * dq4x;
  const T dqq2dx = T(2) * a4 * dq1x + T(2) * a1 * dq4x;
  const T dq2q2dy = T(2) * a1 * dq1y - T(2) * a4 * dq4y;
  const T dqq2dy = T(2) * a4 * dq1y + T(2) * a1 * dq4y;
  const T dpsxdx = dq2q2dx * dpx + q2q2 * pxx - dqq2dx * dpy - qq2 * pxy;
  const T dpsxdy = dq2q2dy * dpx + q2q2 * pxy - dqq2dy * dpy - qq2 * pyy;
  const T dpsydx = dq2q2dx * dpy + q2q2 * pxy + dqq2dx * dpx + qq2 * pxx;
  const T dpsydy = dq2q2dy * dpy + q2q2 * pyy + dqq2dy * dpx + qq2 * pxy;
  const T ux2 = ux * ux, uy2 = uy * uy;
  T tx = dTx * m * (T(2) * sx3 * q2q2 + T(2) * sy3 * qq2 - ux * s4);
  tx += t * (T(6) * sx2 * dpsxdx * q2q2 + T(2) * sx3 * m * dq2q2dx + T(6) * sy2 * dpsydx * qq2 +
             T(2) * sy3 * m * dqq2dx);
  tx -= t * (T(2) * sx3 * q2q2 + T(2) * sy3 * qq2) * (T(2) * ux * pxx + T(2) * uy * pxy);
  tx -= t * (pxx * s4 + ux * (T(4) * sx3 * dpsxdx + T(4) * sy3 * dpsydx));
  tx += t * (ux * s4 * (T(4) * ux2 * ux * pxx + T(4) * ux * pxx * uy2 + T(4) * uy * pxy * ux2 +
                        T(4) * uy2 * uy * pxy));
  tx *= T(4) * k.y_e * k.ebar2;
  T ty = dTy * m * (-T(2) * sx3 * qq2 + T(2) * sy3 * q2q2 - uy * s4);
  ty += t * (-T(6) * sx2 * dpsxdy * qq2 - T(2) * sx3 * m * dqq2dy + T(6) * sy2 * dpsydy * q2q2 +
             T(2) * sy3 * m * dq2q2dy);
  ty -= t * (-T(2) * sx3 * qq2 + T(2) * sy3 * q2q2) * (T(2) * ux * pxy + T(2) * uy * pyy);
  ty -= t * (pyy * s4 + uy * (T(4) * sx3 * dpsxdy + T(4) * sy3 * dpsydy));
  ty += t * (uy * s4 * (T(4) * ux2 * ux * pxy + T(4) * ux * pxy * uy2 + T(4) * uy * pyy * ux2 +
                        T(4) * uy2 * uy * pyy));
  ty *= T(4) * k.y_e * k.ebar2;
  T cW = T(0), M_phi = T(0), c_N = T(1);
#pragma unroll
  for (int l = 0; l < NC; ++l) {
    const T cl = cp.c[l][i];
    cW += cl * k.W[l];
    M_phi += cl * k.M[l];
    c_N -= cl;
  }
  cW += c_N * k.W[NC];
  M_phi += c_N * k.M[NC];
  const T M_q = k.M_qmax + (T(1e-6) - k.M_qmax) * h;
  T dphidt = k.ebar2 * (T(1) - T(3) * k.y_e) * (t * lphi + dTx * dpx + dTy * dpy);
  dphidt += tx + ty;
  dphidt -= hprime * dG[i] / k.v_m;
  dphidt -= gprime * t * cW;
  dphidt -= T(4) * k.H * t * ph * mgq;
  dphidt *= M_phi;
  if (k.variant != 0) {
    // NCGPU_new's phase noise, after the mobility (NCGPU_new.py:186-189)
    const uint64_t st = step + (step_base ? *step_base : 0);
    dphidt += sqrt(T(2) * T(8.314) * t * M_phi / k.v_m) *
              noise_normal<T>(seed, st, y, x, kStreamPhi) * k.noise_phi;
  }
  // c_l: div(M_l grad dF_l) - sum_m div(M_l c_m grad dF_m)
  T dc[NC];
#pragma unroll
  for (int l = 0; l < NC; ++l) {
    const T* Mc = cp.Mc[l];
    const T m0 = Mc[i], mxp = F(Mc, 0, 1), mxm = F(Mc, 0, -1), myp = F(Mc, 1, 0),
            mym = F(Mc, -1, 0);
    const T* dF = cp.dF[l];
    T d = divagradb(m0, mxp, mxm, myp, mym, dF[i], F(dF, 0, 1), F(dF, 0, -1), F(dF, 1, 0),
                    F(dF, -1, 0), idx);
#pragma unroll
    for (int mm = 0; mm < NC; ++mm) {
      const T* c = cp.c[mm];
      const T* dFm = cp.dF[mm];
      d -= divagradb(m0 * c[i], mxp * F(c, 0, 1), mxm * F(c, 0, -1), myp * F(c, 1, 0),
                     mym * F(c, -1, 0), dFm[i], F(dFm, 0, 1), F(dFm, 0, -1), F(dFm, 1, 0),
                     F(dFm, -1, 0), idx);
    }
    dc[l] = d;
  }
  // orientation
  const T Dq = T(2) * k.H * t * ph * ph;
  const T Dxp = T(2) * k.H * txp * pxp * pxp, Dxm = T(2) * k.H * txm * pxm * pxm;
  const T Dyp = T(2) * k.H * typ * pyp * pyp, Dym = T(2) * k.H * tym * pym * pym;
  const T rxp = (Dq + Dxp) * igxp, rxm = (Dq + Dxm) * igxm;
  const T ryp = (Dq + Dyp) * igyp, rym = (Dq + Dym) * igym;
  auto fori = [&](T q, T qxp, T qxm, T qyp, T qym) {
    return T(0.5) * idx * idx *
           (rxp * (qxp - q) - rxm * (q - qxm) + ryp * (qyp - q) - rym * (q - qym));
  };
  const T f1 = fori(a1, q1xp, q1xm, q1yp, q1ym);
  const T f4 = fori(a4, q4xp, q4xm, q4yp, q4ym);
  const T lq1 = (q1xp + q1xm + q1yp + q1ym - T(4) * a1) * idx * idx;
  const T lq4 = (q4xp + q4xm + q4yp + q4ym - T(4) * a4) * idx * idx;
  // NCGPU_new's orientation noise enters the brackets (NCGPU_new.py:225-231);
  // NCGPU adds nothing (x + 0 = x)
  T nq1 = T(0), nq4 = T(0);
  if (k.variant != 0) {
    const uint64_t st = step + (step_base ? *step_base : 0);
    const T qa = k.noise_q * sqrt(T(0.0000000001) * T(8.314) * t / k.v_m);
    nq1 = qa * noise_normal<T>(seed, st, y, x, kStreamQ1);
    nq4 = qa * noise_normal<T>(seed, st, y, x, kStreamQ4);
  }
  const T b1 = f1 + lq1 * k.eqbar2 + nq1, b4 = f4 + lq4 * k.eqbar2 + nq4;
  const T dq1 = M_q * ((T(1) - a1 * a1) * b1 - a1 * a4 * b4);
  const T dq4 = M_q * ((T(1) - a4 * a4) * b4 - a1 * a4 * b1);
  T pn = ph + k.dt * dphidt;
  pn = pn < k.phi_lo ? k.phi_lo : pn;
  pn = pn > k.phi_hi ? k.phi_hi : pn;
  const T n1 = a1 + k.dt * dq1, n4 = a4 + k.dt * dq4;
  const T irn = rsqrt(n1 * n1 + n4 * n4);
  phi_o[i] = pn;
  q1_o[i] = n1 * irn;
  q4_o[i] = n4 * irn;
#pragma unroll
  for (int l = 0; l < NC; ++l) cp.c_out[l][i] = cp.c[l][i] + k.dt * dc[l];
}

template <typename T, int NC>
__global__ void __launch_bounds__(256)
    ncgpu_kernel(Geo g, Bc<T> bc, NcCoef<T> k, const T* __restrict__ phi,
                 const T* __restrict__ q1, const T* __restrict__ q4, NcPtrs<T> cp,
                 const T* __restrict__ temp, const T* __restrict__ dG, T* __restrict__ phi_o,
                 T* __restrict__ q1_o, T* __restrict__ q4_o, uint64_t seed, uint64_t step,
                 const uint64_t* step_base) {
  pdl_wait();
  pdl_launch_next();
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  if (x >= g.n[1]) return;
  // Interior warps (warp-uniform: the warp's 32 columns x0 .. x0 + 31 and
  // their neighbours lie inside the grid, and so do rows y - 1 and y + 1)
  // take the body without boundary-rule code. Not for float64 with three or
  // more components: the second body costs those kernels registers (spills,
  // or one CTA per SM at six components: measured 8 % slower).
  if constexpr (std::is_same<T, float>::value || NC <= 2) {
    const int x0 = x - (int)(threadIdx.x & 31);
    if (y >= 1 && y + 1 < g.n[0] && x0 >= 1 && x0 + 33 <= g.n[1]) {
      ncgpu_cell<T, NC, true>(g, bc, k, phi, q1, q4, cp, temp, dG, phi_o, q1_o, q4_o, seed, step,
                              step_base, x, y);
      return;
    }
  }
  ncgpu_cell<T, NC, false>(g, bc, k, phi, q1, q4, cp, temp, dG, phi_o, q1_o, q4_o, seed, step,
                           step_base, x, y);
}

template <typename T, int NC>
cudaError_t launch_ncgpu(dim3 grid2, cudaStream_t st, const Geo& g, const Bc<T>& bc,
                         const NcCoef<T>& k, const NcGibbs& gb, const T* const* in,
                         T* const* out, const NcPtrs<T>& cp, const T* temp, const double* tab,
                         T* dG, uint64_t seed, uint64_t step, const uint64_t* step_base) {
  cudaError_t e = launch(ncgpu_thermo_kernel<T, NC>, grid2, dim3(256), 0, st, true, g, k, gb,
                         in[0], cp, temp, tab, dG, seed, step, step_base);
  if (e != cudaSuccess) return e;
  return launch(ncgpu_kernel<T, NC>, grid2, dim3(256), 0, st, true, g, bc, k, in[0], in[1], in[2],
                cp, temp, (const T*)dG, out[0], out[1], out[2], seed, step, step_base);
}

int32_t make_gibbs(const PpfNcgpuParams* p, NcGibbs* gb) {
  for (int ph = 0; ph < 2; ++ph)
    for (int c = 0; c < p->ncomp; ++c)
      if (p->npieces[ph][c] < 0 || p->npieces[ph][c] > 4)
        return fail(PPF_ERR_INVALID, "npieces must be 0..4");
  static_assert(sizeof(gb->piece) == sizeof(p->gibbs), "Gibbs table layout");
  memcpy(gb->piece, p->gibbs, sizeof(gb->piece));
  memcpy(gb->npieces, p->npieces, sizeof(gb->npieces));
  if (p->nexcess < 0 || p->nexcess > kMaxExcess)
    return fail(PPF_ERR_INVALID, "nexcess must be 0..%d", kMaxExcess);
  gb->nex = p->nexcess;
  memset(gb->ex_meta, 0, sizeof(gb->ex_meta));
  memset(gb->ex_piece, 0, sizeof(gb->ex_piece));
  for (int e = 0; e < p->nexcess; ++e) {
    const PpfNcgpuExcess& x = p->excess[e];
    if (x.phase < 0 || x.phase > 1 || x.a < 0 || x.a >= p->ncomp || x.b < 0 ||
        x.b >= p->ncomp || x.a == x.b || x.order < 0 || x.order > 16 || x.npieces < 0 ||
        x.npieces > 4)
      return fail(PPF_ERR_INVALID, "excess term %d: phase 0..1, components a != b below ncomp, "
                  "order 0..16, npieces 0..4", e);
    gb->ex_meta[e][0] = x.phase;
    gb->ex_meta[e][1] = x.a;
    gb->ex_meta[e][2] = x.b;
    gb->ex_meta[e][3] = x.order;
    gb->ex_meta[e][4] = x.npieces;
    static_assert(sizeof(gb->ex_piece[0]) == sizeof(x.piece), "excess table layout");
    memcpy(gb->ex_piece[e], x.piece, sizeof(x.piece));
  }
  return PPF_OK;
}

template <typename T>
int32_t ncgpu_tables(const PpfNcgpuParams* p, const PpfGrid* grid, const T* temp, double* tables,
                     void* stream) {
  clear_error();
  if (!p || !temp || !tables) return fail(PPF_ERR_INVALID, "NULL argument");
  Geo g;
  int32_t rc = make_geo(grid, 2, 2, &g);
  if (rc) return rc;
  if (p->ncomp < 2 || p->ncomp > kMaxComp)
    return fail(PPF_ERR_UNSUPPORTED, "NCGPU: 2 to %d components (got %d)", kMaxComp, p->ncomp);
  if (g.n[0] > 65535) return fail(PPF_ERR_INVALID, "more than 65535 rows");
  NcGibbs gb;
  if ((rc = make_gibbs(p, &gb))) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const dim3 grid2((g.n[1] + 255) / 256, g.n[0]);
  cudaError_t e;
#define PPF_NC_CASE(n)                                                                        \
  case n:                                                                                     \
    e = launch(ncgpu_table_kernel<T, n>, grid2, dim3(256), 0, st, true, g, gb, temp, tables); \
    break;
  switch (p->ncomp) {
    PPF_NC_CASE(2)
    PPF_NC_CASE(3)
    PPF_NC_CASE(4)
    PPF_NC_CASE(5)
    default:
    PPF_NC_CASE(6)
  }
#undef PPF_NC_CASE
  PPF_TRY_CUDA(e);
  return PPF_OK;
}

template <typename T>
int32_t ncgpu_step(const PpfNcgpuParams* p, const PpfGrid* grid, const PpfBoundary* bcin,
                   const T* const* in, T* const* out, const T* temp, const double* tables,
                   T* transfer, uint64_t seed, uint64_t step, const uint64_t* step_base,
                   void* stream) {
  clear_error();
  if (!p || !in || !out) return fail(PPF_ERR_INVALID, "NULL argument");
  Geo g;
  int32_t rc = make_geo(grid, 2, 2, &g);
  if (rc) return rc;
  const int ncomp = p->ncomp;
  if (ncomp < 2 || ncomp > kMaxComp)
    return fail(PPF_ERR_UNSUPPORTED, "NCGPU: 2 to %d components (got %d)", kMaxComp, ncomp);
  const int nc = ncomp - 1;
  for (int f = 0; f < 3 + nc; ++f)
    if (!in[f] || !out[f]) return fail(PPF_ERR_INVALID, "NULL field pointer");
  if (!temp || !transfer) return fail(PPF_ERR_INVALID, "NULL temperature or transfer buffer");
  if (g.n[0] > 65535) return fail(PPF_ERR_INVALID, "more than 65535 rows");
  Bc<T> bc;
  if ((rc = make_bc<T>(bcin, g, p->dx, 1, 1, &bc))) return rc;
  for (int a = 0; a < 2; ++a) {
    if (bcin && bcin->type[a] == PPF_BC_DIRCHLET)
      return fail(PPF_ERR_UNSUPPORTED,
                  "NCGPU: periodic or zero-gradient boundaries only (the per-cell "
                  "thermodynamic terms of ghost cells follow their fields)");
    for (int s = 0; s < 2; ++s)
      if (bcin && bcin->type[a] == PPF_BC_NEUMANN && bcin->value[0][a][s] != 0.0)
        return fail(PPF_ERR_UNSUPPORTED, "NCGPU: Neumann boundaries with zero gradient only");
  }
  NcCoef<T> k;
  k.idx = (T)(1.0 / p->dx);
  k.dt = (T)p->dt;
  k.v_m = (T)p->v_m;
  k.D_L = (T)p->D_L;
  k.D_S = (T)p->D_S;
  k.M_qmax = (T)p->M_qmax;
  k.H = (T)p->H;
  k.y_e = (T)p->y_e;
  k.beta = (T)p->beta;
  k.ebar2 = (T)p->ebar2;
  if (p->variant != PPF_NCGPU_VARIANT_NCGPU && p->variant != PPF_NCGPU_VARIANT_NEW)
    return fail(PPF_ERR_INVALID, "variant must be PPF_NCGPU_VARIANT_NCGPU or _NEW");
  k.variant = p->variant;
  const bool nv = p->variant == PPF_NCGPU_VARIANT_NEW;
  k.eqbar2 = (T)(nv ? p->eqbar2 : 0.25 * p->ebar2);
  k.noise = (T)p->noise_scale;
  k.noise_phi = (T)(nv ? p->noise_phi : 0.0);
  k.noise_q = (T)(nv ? p->noise_q : 0.0);
  k.phi_lo = (T)(nv ? 0.0001 : 0.000001);
  k.phi_hi = (T)(nv ? 0.9999 : 0.999999);
  for (int c = 0; c < kMaxComp; ++c) {
    k.W[c] = (T)p->W[c];
    k.M[c] = (T)p->M[c];
  }
  NcGibbs gb;
  if ((rc = make_gibbs(p, &gb))) return rc;
  const int64_t fsz = (int64_t)g.n[0] * g.pitch;
  NcPtrs<T> cp{};
  for (int l = 0; l < nc; ++l) {
    cp.c[l] = in[3 + l];
    cp.c_out[l] = out[3 + l];
    cp.Mc[l] = transfer + (1 + l) * fsz;
    cp.dF[l] = transfer + (1 + nc + l) * fsz;
  }
  T* dG = transfer;
  cudaStream_t st = (cudaStream_t)stream;
  const dim3 grid2((g.n[1] + 255) / 256, g.n[0]);
  static_assert(kMaxComp == 6, "one instantiation per concentration-field count");
  cudaError_t e;
#define PPF_NC_CASE(n)                                                                      \
  case n:                                                                                   \
    e = launch_ncgpu<T, n>(grid2, st, g, bc, k, gb, in, out, cp, temp, tables, dG, seed, step,  \
                           step_base);                                                      \
    break;
  switch (nc) {
    PPF_NC_CASE(1)
    PPF_NC_CASE(2)
    PPF_NC_CASE(3)
    PPF_NC_CASE(4)
    default:
    PPF_NC_CASE(5)
  }
#undef PPF_NC_CASE
  PPF_TRY_CUDA(e);
  return PPF_OK;
}

// Temperature of a LINEAR_GRADIENT profile that changes in time: every cell
// rises by dT = dTdt * dt after each step (update_thermal_gradient_2D_kernel,
// ppf_gpu_utils.py:326-334; Simulation.simulate calls it after each engine
// step, simulation.py:262-266).
template <typename T>
__global__ void __launch_bounds__(256) temperature_advance_kernel(Geo g, T* __restrict__ t, T dT) {
  pdl_wait();
  pdl_launch_next();
  const int nx = g.n[1];
  for (int r = blockIdx.y; r < g.n[0]; r += gridDim.y)
    for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < nx; x += gridDim.x * blockDim.x)
      t[(int64_t)r * g.pitch + x] += dT;
}

template <typename T>
int32_t temperature_advance(const PpfGrid* grid, T* t, double dT, void* stream) {
  clear_error();
  Geo g;
  int32_t rc = make_geo(grid, 2, 2, &g);
  if (rc) return rc;
  if (!t) return fail(PPF_ERR_INVALID, "temperature is NULL");
  if (!isfinite(dT)) return fail(PPF_ERR_INVALID, "dT must be finite");
  const dim3 grid2((g.n[1] + 255) / 256, (unsigned)(g.n[0] < 65535 ? g.n[0] : 65535));
  PPF_TRY_CUDA(launch(temperature_advance_kernel<T>, grid2, dim3(256), 0, (cudaStream_t)stream,
                      true, g, t, (T)dT));
  return PPF_OK;
}

}  // namespace
}  // namespace ppf

using namespace ppf;

extern "C" {

int32_t ppf_ncgpu_step_f32(const PpfNcgpuParams* p, const PpfGrid* g, const PpfBoundary* bc,
                           const float* const* fields_in, float* const* fields_out,
                           const float* temperature, const double* tables, float* transfer,
                           uint64_t seed, uint64_t step, const uint64_t* step_base,
                           void* stream) {
  return ncgpu_step<float>(p, g, bc, fields_in, fields_out, temperature, tables, transfer, seed,
                           step, step_base, stream);
}

int32_t ppf_ncgpu_step_f64(const PpfNcgpuParams* p, const PpfGrid* g, const PpfBoundary* bc,
                           const double* const* fields_in, double* const* fields_out,
                           const double* temperature, const double* tables, double* transfer,
                           uint64_t seed, uint64_t step, const uint64_t* step_base,
                           void* stream) {
  return ncgpu_step<double>(p, g, bc, fields_in, fields_out, temperature, tables, transfer, seed,
                            step, step_base, stream);
}

int32_t ppf_ncgpu_temperature_advance_f32(const PpfGrid* g, float* temperature, double dT,
                                          void* stream) {
  return temperature_advance<float>(g, temperature, dT, stream);
}
int32_t ppf_ncgpu_temperature_advance_f64(const PpfGrid* g, double* temperature, double dT,
                                          void* stream) {
  return temperature_advance<double>(g, temperature, dT, stream);
}

int32_t ppf_ncgpu_tables_f32(const PpfNcgpuParams* p, const PpfGrid* g, const float* temperature,
                             double* tables, void* stream) {
  return ncgpu_tables<float>(p, g, temperature, tables, stream);
}

int32_t ppf_ncgpu_tables_f64(const PpfNcgpuParams* p, const PpfGrid* g, const double* temperature,
                             double* tables, void* stream) {
  return ncgpu_tables<double>(p, g, temperature, tables, stream);
}

}  // extern "C"
