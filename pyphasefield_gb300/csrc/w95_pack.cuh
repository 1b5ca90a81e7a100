// Warren-Boettinger (1995) band update for float and two rows per warp with
// packed FP32x2 arithmetic (add/sub/mul/fma.rn.f32x2): the band's two output
// rows travel as the two halves of one 64-bit register pair, so every
// arithmetic instruction of the update advances both rows. Same equations
// and cell layout as the scalar band in w95_core.cuh (Engines/Warren1995.py
// :50-92); the exact bulk form and the noise stream are unchanged.
#pragma once

#include <cstdint>

namespace ppf {
namespace w95 {

struct F2 {
  uint64_t v;
};

__device__ __forceinline__ F2 pk(float a, float b) {
  F2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ F2 sp(float a) { return pk(a, a); }
__device__ __forceinline__ float lo(F2 x) {
  float a, b;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(x.v));
  return a;
}
__device__ __forceinline__ float hi(F2 x) {
  float a, b;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(x.v));
  return b;
}
__device__ __forceinline__ F2 operator+(F2 a, F2 b) {
  F2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ F2 operator-(F2 a, F2 b) {
  F2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ F2 operator*(F2 a, F2 b) {
  F2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
// a * b + c, one rounding per half
__device__ __forceinline__ F2 fma2(F2 a, F2 b, F2 c) {
  F2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
  return r;
}

// D~ and Q~ (see point() in w95_core.cuh) for two cells at once.
__device__ __forceinline__ void point2(const Coef<float>& k, F2 phi, F2 c, F2& Dt, F2& Qt) {
  const F2 one = sp(1.f);
  const F2 p = phi * phi * phi * fma2(phi, fma2(sp(6.f), phi, sp(-15.f)), sp(10.f));
  const F2 om = one - phi;
  const F2 g = phi * phi * (om * om);
  const F2 gp = phi * fma2(phi, fma2(sp(4.f), phi, sp(-6.f)), sp(2.f));
  Dt = fma2(sp(k.a1), p, sp(k.a0));
  const F2 dH = fma2(sp(k.WB - k.WA), gp, sp(k.hB - k.hA) * g);
  Qt = Dt * sp(k.vr) * c * (one - c) * dH;
}

template <typename T>
__device__ __forceinline__ T shfl_w(T v);
template <typename T>
__device__ __forceinline__ T shfl_e(T v);

// Two-row band (ROWS = 2) of the float kernel: rows y0, y0 + 1 are the low
// and high halves. bp / bcv hold phi / c of rows y0 - 1 .. y0 + 2.
__device__ __forceinline__ void band_compute_f2(const Coef<float>& k, const Geo& g,
                                                float* __restrict__ phi_out,
                                                float* __restrict__ c_out, uint64_t seed,
                                                uint64_t step, int xs, int y0,
                                                const float (&bp)[4], const float (&bcv)[4]) {
  const int lane = threadIdx.x;
  const int ny = g.n[0], nx = g.n[1];
  const int x = xs + lane;
  const bool owner = lane >= 1 && lane <= kStrip && x < nx;

  // west / east neighbours of the four rows
  float w[4], e[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    w[j] = shfl_w(bp[j]);
    e[j] = shfl_e(bp[j]);
  }
  const F2 pN = pk(bp[0], bp[1]), p0 = pk(bp[1], bp[2]), pS = pk(bp[2], bp[3]);
  const F2 cN = pk(bcv[0], bcv[1]), c0 = pk(bcv[1], bcv[2]), cS = pk(bcv[2], bcv[3]);
  const F2 pNW = pk(w[0], w[1]), pNE = pk(e[0], e[1]);
  const F2 pW = pk(w[1], w[2]), pE = pk(e[1], e[2]);
  const F2 pSW = pk(w[2], w[3]), pSE = pk(e[2], e[3]);
  const F2 cW = pk(shfl_w(bcv[1]), shfl_w(bcv[2])), cE = pk(shfl_e(bcv[1]), shfl_e(bcv[2]));
  F2 D01, Q01, D23, Q23;
  point2(k, pN, cN, D01, Q01);
  point2(k, pS, cS, D23, Q23);
  const F2 DN = D01, DS = D23, QN = Q01, QS = Q23;
  const float D1 = hi(D01), D2 = lo(D23), Q1 = hi(Q01), Q2 = lo(Q23);
  const F2 D0 = pk(D1, D2), Q0 = pk(Q1, Q2);
  const F2 two = sp(2.f);
  const F2 lc = fma2(sp(-2.f), c0, cN + cS) + fma2(sp(-2.f), c0, cW + cE);

  // exact bulk form (see band_compute): both rows of every owned cell
  bool bulk = false;
  if (k.bulk) {
    bool b = true;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const float v = bp[r + 1];
      b = b & ((v == 1.f) | (v == 0.f)) & (bp[r] == v) & (bp[r + 2] == v) & (w[r + 1] == v) &
          (e[r + 1] == v) & (w[r] == v) & (e[r] == v) & (w[r + 2] == v) & (e[r + 2] == v);
    }
    bulk = __all_sync(0xffffffffu, b | !owner);
  }
  F2 p1, c1;
  if (bulk) {
    p1 = p0;
    c1 = c0 + D0 * lc;
  } else {
    const F2 DW = pk(shfl_w(D1), shfl_w(D2)), DE = pk(shfl_e(D1), shfl_e(D2));
    const F2 QW = pk(shfl_w(Q1), shfl_w(Q2)), QE = pk(shfl_e(Q1), shfl_e(Q2));
    const F2 quarter = sp(0.25f);

    const F2 px = pN - pS;
    const F2 py = pW - pE;
    const F2 pxx = fma2(sp(-2.f), p0, pN + pS);
    const F2 pyy = fma2(sp(-2.f), p0, pW + pE);
    const F2 lp = pxx + pyy;
    const F2 pxy = quarter * ((pNW - pSW) - (pNE - pSE));

    // dc * dt (Warren1995.py:69-71); in bulk every added term is exactly 0
    const F2 fl = fma2(DW - DE, cW - cE, (DN - DS) * (cN - cS));
    F2 dc = fma2(quarter, fl, D0 * lc);
    dc = fma2(Q0, lp, dc);
    const F2 fq = fma2(QW - QE, py, (QN - QS) * px);
    dc = fma2(quarter, fq, dc);

    // anisotropy without trig: theta = atan2(py, px)
    const F2 r2 = fma2(px, px, py * py);
    const float r2a = lo(r2), r2b = hi(r2);
    const F2 n = pk(rsqrtf(fmaxf(r2a, 1e-30f)), rsqrtf(fmaxf(r2b, 1e-30f)));
    const F2 ux = px * n, uy = py * n;
    const F2 c2u = ux * ux - uy * uy;
    const F2 s2u = two * ux * uy;
    const bool ga = r2a > tiny_r2<float>(), gb = r2b > tiny_r2<float>();
    const F2 c2 = pk(ga ? lo(c2u) : 1.f, gb ? hi(c2u) : 1.f);
    const F2 s2 = pk(ga ? lo(s2u) : 0.f, gb ? hi(s2u) : 0.f);
    const F2 c4 = c2 * c2 - s2 * s2;
    const F2 s4 = two * s2 * c2;
    const F2 eta = fma2(sp(k.ye), c4, sp(1.f));
    const F2 etap = sp(-4.f * k.ye) * s4;
    const F2 etapp = sp(-16.f * k.ye) * c4;

    // dphi * dt (Warren1995.py:82-86)
    const F2 om = sp(1.f) - p0;
    const F2 g0 = p0 * p0 * (om * om);
    const F2 gp = p0 * fma2(p0, fma2(sp(4.f), p0, sp(-6.f)), two);
    const F2 HA = fma2(sp(k.WA), gp, sp(k.hA) * g0);
    const F2 HB = fma2(sp(k.WB), gp, sp(k.hB) * g0);
    const F2 oc = sp(1.f) - c0;
    const F2 Hs = fma2(oc, HA, c0 * HB);
    const F2 dtM = fma2(oc, sp(k.dtMA), c0 * sp(k.dtMB));
    const F2 dyx = pyy - pxx;
    const F2 t1 = eta * eta * lp;
    const F2 t2 = eta * etap * fma2(s2, dyx, two * c2 * pxy);
    const F2 t3 = sp(0.5f) * fma2(etap, etap, eta * etapp) *
                  fma2(c2, dyx, fma2(sp(-2.f), s2 * pxy, lp));
    const F2 aniso = t1 + t2 + t3;
    F2 dphi = dtM * (sp(k.e2) * aniso - Hs);

    // noise (:85-86) on cells with g(phi) != 0, drawn as in band_compute
    const float g0a = lo(g0), g0b = hi(g0);
    const bool noisy = k.alpha != 0.f;
    const bool need0 = noisy && owner && g0a != 0.f;
    const bool need1 = noisy && owner && g0b != 0.f;
    if (__any_sync(0xffffffffu, need0 || need1)) {
      const uint32_t gbase = (uint32_t)(xs + 1) / 4u;
      BandNoise<2> noise;
      noise.draw(seed, step, y0, gbase);
      const uint32_t wa = noise.word(0, x, gbase), wb = noise.word(1, x, gbase);
      const F2 u = pk(float(wa >> 8) * 5.9604644775390625e-08f,
                      float(wb >> 8) * 5.9604644775390625e-08f);
      const F2 nz = dtM * sp(k.alpha) * fma2(two, u, sp(-1.f)) * (sp(16.f) * g0) * Hs;
      dphi = dphi + pk(need0 ? lo(nz) : 0.f, need1 ? hi(nz) : 0.f);
    }
    p1 = p0 + dphi;
    c1 = c0 + dc;
  }
  if (owner) {
    const int64_t o = (int64_t)y0 * g.pitch + x;
    if (y0 < ny) {
      phi_out[o] = lo(p1);
      c_out[o] = lo(c1);
    }
    if (y0 + 1 < ny) {
      phi_out[o + g.pitch] = hi(p1);
      c_out[o + g.pitch] = hi(c1);
    }
  }
}

}  // namespace w95
}  // namespace ppf
